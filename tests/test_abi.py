"""The C ABI library: loads, exports every symbol include/*.h declares, host-only
entry points agree with the oracle / the reference's golden values, and the
device path fails loudly (no CPU fallback) when no GPU is present.  CPU only."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from deorbit_gb300 import ic

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:int|void|const char\s*\*)\s+(sph_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("sph_create", "sph_init", "sph_timestep", "sph_step", "sph_read_field",
                     "sph_impact_add_particles", "sph_impact_seed_damage", "sph_run"):
        assert required in names


def test_library_exports_every_declared_symbol(cuda_lib):
    missing = [n for n in declared_functions() if not hasattr(cuda_lib, n)]
    assert not missing, missing


def test_standard_materials_match_reference(cuda_lib):
    from deorbit_gb300 import sph
    gold = np.load(os.path.join(ROOT, "tests", "golden", "eos.npz"))
    for which in range(4):
        m = sph.standard(which)
        got = np.array([getattr(m, k) for k in ic.MAT_FIELDS])
        assert np.array_equal(got, gold[f"std{which}"]), which
    with pytest.raises(sph.SphError):
        sph.standard(9)


def test_params_default_is_reference_default(cuda_lib):
    from deorbit_gb300 import sph
    p = sph.params()
    assert (p.eta, p.h_init, p.alpha, p.beta, p.eps, p.alpha_u, p.cfl, p.eps_as, p.as_n, p.damage_on) == \
           (1.3, 0.01, 1.0, 2.0, 0.01, 0.0, 0.2, 0.0, 4, 0)


def test_host_seeding_matches_golden_and_oracle(cuda_lib, oracle_lib):
    from deorbit_gb300 import sph
    O = oracle_lib
    gold = np.load(os.path.join(ROOT, "tests", "golden", "seed_damage.npz"))
    mats = [sph.basalt(), sph.iron()]
    eps = sph.seed_flaws_single(gold["mat"], mats, float(gold["dx"]), int(gold["seed"]))
    assert np.array_equal(eps, gold["eps_act"])
    # multi-flaw extension: same procedure as the oracle's
    mat = (np.arange(3000) % 4 == 0).astype(np.int32)
    ptr, e2, act = sph.seed_flaws_multi(mat, [ic._material_struct(sph.Material, ic.granite()),
                                             ic._material_struct(sph.Material, ic.iron())], 31.25, 7)
    S = O.OracleSystem()
    S.add_material(ic._material_struct(O.Material, ic.granite()))
    S.add_material(ic._material_struct(O.Material, ic.iron()))
    S.set_params(h_init=40.0)
    S.add_many(np.zeros((3000, 3)), np.zeros((3000, 3)), 1.0, 0.0, mat)
    S.seed_flaws_multi(31.25, 7)
    optr, oeps = S.flaws()
    assert np.array_equal(ptr, optr) and np.array_equal(e2, oeps)
    assert np.array_equal(act, S.field("eps_act"))
    # every brittle particle holds at least one flaw, ~ln N on average
    cnt = np.diff(ptr)
    assert np.all(cnt[mat == 0] >= 1) and np.all(cnt[mat == 1] == 0)
    nb = int((mat == 0).sum())
    assert abs(cnt[mat == 0].mean() - np.log(nb)) < 1.5


def test_bad_arguments_return_status(cuda_lib):
    from deorbit_gb300 import sph
    L = sph.lib()
    assert L.sph_material_standard(7, None) == -1
    out = np.zeros(4)
    mat = np.array([0, 5, 0, 0], np.int32)
    arr = (sph.Material * 1)(sph.basalt())
    rc = L.sph_seed_flaws_single(4, mat.ctypes.data_as(C.POINTER(C.c_int32)), arr, 1, 1.0, 1,
                                 out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == -1 and b"material" in L.sph_last_error()


def test_device_path_fails_loudly_without_gpu(cuda_lib):
    """No CPU fallback: creating a context needs a CUDA device."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from deorbit_gb300 import sph
    with pytest.raises(sph.SphError) as e:
        sph.Context(sph.FP64)
    assert e.value.code == -2


def test_step_fields_rejects_bad_arguments_before_device_work(cuda_lib):
    """sph_step_fields checks its arguments before it touches a device: a
    non-finite dt, negative counts, missing name or buffer arrays and a null
    context each return SPH_ERR_ARG with a message."""
    from deorbit_gb300 import sph
    L = sph.lib()
    names = (C.c_char_p * 1)(b"x")
    buf = np.zeros(4)
    ptrs = (C.POINTER(C.c_double) * 1)(buf.ctypes.data_as(C.POINTER(C.c_double)))
    cases = [
        (float("inf"), 1, names, ptrs, 1, names, ptrs, b"dt"),
        (float("nan"), 1, names, ptrs, 1, names, ptrs, b"dt"),
        (-1.0, -1, names, ptrs, 1, names, ptrs, b"nin"),
        (-1.0, 1, names, ptrs, -2, names, ptrs, b"nout"),
        (-1.0, 1, None, ptrs, 1, names, ptrs, b"in_names"),
        (-1.0, 1, names, ptrs, 1, names, None, b"outs"),
        (0.5, 1, names, ptrs, 1, names, ptrs, b"null context"),
    ]
    for dt, nin, inn, ins, nout, outn, outs, msg in cases:
        rc = L.sph_step_fields(None, 0, dt, nin, inn, ins, nout, outn, outs, None)
        assert rc == -1 and msg in L.sph_last_error(), (dt, nin, nout, L.sph_last_error())
