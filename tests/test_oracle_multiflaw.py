"""The oracle's multi-flaw damage extension against the published law it
restates (Benz & Asphaug 1995, Icarus 107 / Comput. Phys. Commun. 87): the
reference SPH has single-flaw damage only (sph.hpp:117-128,336-348), so these
checks pin the extension to the law instead of to reference outputs.

Seeding: a brittle material with Weibull constants k, m over N particles of
volume V = dx^3 each holds N_f = ceil(N ln N) flaws whose thresholds follow the
cumulative law n(eps) = k N V eps^m, i.e. the j-th weakest flaw has
eps_j = (j / (k N V))^(1/m); flaws land on particles uniformly at random, every
particle ends with at least one, and eps_act is each particle's weakest.
Growth: with n_act = #(flaws with eps_j < sigma_max / E) of a particle's n_f,
D^(1/3) grows by n_act^(1/3) c_g / R_s dt (c_g = 0.4 sqrt(E / rho),
R_s = 0.5 h0 / eta) and D is capped at n_act / n_f; no growth when sigma_max <= 0
or below the weakest flaw; D never decreases."""
import math

import numpy as np
import pytest

from deorbit_gb300 import ic
from oracle import oracle as O


def _system(n, mats, mat_ids, dx=31.25):
    S = O.OracleSystem()
    for d in mats:
        S.add_material(O.material_from_dict(d))
    S.set_params(eta=1.3, h_init=1.3 * dx, damage_on=1, flaw_model=1)
    rng = np.random.default_rng(3)
    pos = rng.uniform(0, 100 * dx, size=(n, 3))
    S.add_many(pos, np.zeros((n, 3)), np.full(n, 1.0), np.zeros(n), np.asarray(mat_ids, np.int32),
               np.zeros(n, np.uint8))
    return S


@pytest.mark.parametrize("nb", [1000, 20000])
def test_seeding_follows_the_weibull_law(nb):
    dx = 31.25
    gran = ic.granite()
    k, m = gran["wk"], gran["wm"]
    n_iron = 137
    mat = np.r_[np.zeros(nb, np.int32), np.ones(n_iron, np.int32)]
    S = _system(mat.size, [gran, ic.iron()], mat, dx)
    nf = S.seed_flaws_multi(dx, 12345)
    start, eps = S.flaws()
    eps_act = S.field("eps_act")
    S.close()
    cnt = np.diff(start)
    Nf = math.ceil(nb * math.log(nb))
    # iron (no Weibull constants) holds no flaws; every granite particle holds >= 1
    assert np.all(cnt[nb:] == 0) and np.all(eps_act[nb:] == 1e30)
    assert np.all(cnt[:nb] >= 1)
    assert nf == eps.size and Nf <= nf <= Nf + np.count_nonzero(cnt[:nb] == 1)
    # cumulative law over the first N_f flaws: #(eps <= eps_j) = j = k N V eps_j^m
    V = nb * dx ** 3
    srt = np.sort(eps)
    j = np.arange(1, srt.size + 1)
    np.testing.assert_allclose(k * V * srt[:Nf] ** m, j[:Nf], rtol=1e-12)
    # the flaws beyond N_f (one per particle left empty) continue the same sequence
    np.testing.assert_allclose(srt, (j / (k * V)) ** (1.0 / m), rtol=1e-14)
    # eps_act is each particle's weakest flaw; lists are ascending
    assert np.all(eps_act[:nb] == eps[start[:nb]])
    assert all(np.all(np.diff(eps[start[i]:start[i + 1]]) > 0) for i in range(0, nb, 97))
    # owners uniform: counts ~ Poisson(ln N) (mean and variance near ln N)
    lam = Nf / nb
    assert abs(cnt[:nb].mean() - lam) < 0.15 + 1.0 / nb
    assert 0.7 * lam < cnt[:nb].var() < 1.3 * lam


def test_growth_follows_the_law():
    dx = 31.25
    gran = ic.granite()
    E, eta, h0 = gran["Emod"], 1.3, 1.3 * dx
    n = 7
    S = _system(n, [gran], np.zeros(n, np.int32), dx)
    # five flaws per particle at known thresholds
    thr = np.array([1e-5, 2e-5, 4e-5, 8e-5, 1.6e-4])
    start = np.arange(0, 5 * n + 1, 5, dtype=np.int64)
    S.set_flaws(start, np.tile(thr, n))
    S.set_field("eps_act", np.full(n, thr[0]))
    rho = np.full(n, 2680.0)
    # sigma_max / E: below every flaw, between flaws 2 and 3, above all, exactly
    # at a threshold (not counted: strict >), compressive, and two already damaged
    eps_local = np.array([0.5e-5, 3e-5, 1e-3, 4e-5, 5e-5, 3e-5, 9e-5])
    sig = eps_local * E
    sig[4] = -sig[4]
    D0 = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 0.35, 0.1])
    S.set_field("rho", rho)
    S.set_field("sigmax", sig)
    S.set_field("D", D0)
    cg = 0.4 * math.sqrt(E / 2680.0)
    Rs = 0.5 * h0 / eta
    nact = np.array([int(np.count_nonzero(eps_local[i] > thr)) if sig[i] > 0 else 0 for i in range(n)])
    assert list(nact) == [0, 2, 5, 2, 0, 2, 4]
    for dt in (1e-4, 1e-2):  # a short step (growth law), then a long one (the cap binds)
        S.grow_damage(dt)
        D1 = S.field("D")
        for i in range(n):
            if nact[i] == 0:
                want = D0[i]
            else:
                grown = (D0[i] ** (1 / 3) + nact[i] ** (1 / 3) * cg / Rs * dt) ** 3
                want = max(D0[i], min(nact[i] / 5.0, grown))
            assert D1[i] == pytest.approx(want, rel=1e-12, abs=1e-300), (dt, i, D1[i], want)
        assert np.all(D1 >= D0)  # D never decreases
        D0 = D1
    # after the long step every particle with active flaws sits at n_act / n_f
    np.testing.assert_allclose(D0[nact > 0], nact[nact > 0] / 5.0, rtol=1e-14)
    S.close()
