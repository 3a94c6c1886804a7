"""Shared helpers for the CUDA-vs-oracle parity tests."""
from __future__ import annotations

import numpy as np

from deorbit_gb300 import ic
from oracle import oracle as O

STATE = ["x", "y", "z", "vx", "vy", "vz", "u", "rho", "hh", "P", "cs", "csig",
         "Sxx", "Syy", "Szz", "Sxy", "Sxz", "Syz", "D"]
DERIV = ["ax", "ay", "az", "dudt", "dSxx", "dSyy", "dSzz", "dSxy", "dSxz", "dSyz", "eps_work"]


def rel_l2(a, b):
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    nb = np.linalg.norm(b)
    if nb == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)


def max_rel(a, b):
    """max |a - b| normalised by the dataset max |b| (the reference GPU gates' norm)."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    s = np.abs(b).max()
    return float(np.abs(a - b).max() / s) if s > 0 else float(np.abs(a - b).max())


def vec_rel_l2(gpu, orc, names):
    """rel-L2 over a group of components (positions / velocities as vectors)."""
    a = np.concatenate([gpu[k] for k in names])
    b = np.concatenate([orc[k] for k in names])
    return rel_l2(a, b)


def pair(sc, precision):
    """Same scenario in the CUDA solver (one impact) and the oracle."""
    from deorbit_gb300 import sph

    ctx = sph.Context(precision)
    b = ic.to_context(ctx, sc)
    orc = O.from_scenario(sc)
    return ctx, b, orc


def read_all(ctx, b, names):
    return {k: ctx.read(b, k) for k in names}


def field_errors(gpu, orc, names):
    return {k: rel_l2(gpu[k], orc[k]) for k in names}
