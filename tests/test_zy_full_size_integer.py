"""Integer outputs bit for bit against the oracle at full size: the
1,048,576-particle grazing impact (strength + damage, multi-flaw), after init
and two steps of the mixed form (the headline form) and of the FP64 form.

The device state (positions and smoothing lengths, read back in original
order) is handed to the oracle, which builds its reference cell grid
(sph.hpp:142-162) and neighbour sets (for_neighbors, sph.hpp:163-182) from it;
the device builds the same structures from the same state.  Asserted equal:
  * the reference grid (cell counts per axis and widths) and its CSR: cell
    pointers and, inside every cell, the particle ids in ascending order;
  * the density sets {j : r < 2 h_i} (self included) and the force sets
    {j != i : r < 2 hbar, r != 0} of every particle;
  * the multi-flaw CSR the device holds.
"""
import dataclasses

import numpy as np
import pytest

from deorbit_gb300 import ic
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grazing():
    return ic.grazing()


def _sorted_sets(counts, ids):
    """Every set sorted ascending (the oracle lists in visiting order)."""
    seg = np.repeat(np.arange(counts.size, dtype=np.int64), counts)
    return ids[np.lexsort((ids, seg))]


@pytest.mark.parametrize("precision", [1, 0])
def test_full_size_cells_and_neighbours_bit_exact(cuda_lib, grazing, precision):
    from deorbit_gb300 import sph
    sc = grazing
    ctx = sph.Context(precision)
    b = ic.to_context(ctx, sc)
    ctx.init()
    ctx.run(2)
    state = {k: ctx.read(b, k) for k in ("x", "y", "z", "hh")}
    # the device rebuilds its grid from exactly the state handed to the oracle
    for k, v in state.items():
        ctx.write(b, k, v)
    nc, cw, start, ids = ctx.ref_cells(b)
    cnt_d, nb_d = ctx.neighbors(b, 0)
    cnt_f, nb_f = ctx.neighbors(b, 1)
    ptr, eps = ctx.flaws(b)
    ctx.close()

    orc = O.from_scenario(dataclasses.replace(sc, flaws=None), threads=16)
    for k, v in state.items():
        orc.set_field(k, v)
    orc.build_cells()
    onc, ocw, _ = orc.grid()
    ostart, oids = orc.cell_csr()
    assert np.array_equal(nc, onc) and np.array_equal(cw, ocw)
    assert np.array_equal(start, ostart)
    assert np.array_equal(ids, oids)
    for kind, (cnt, nb) in ((0, (cnt_d, nb_d)), (1, (cnt_f, nb_f))):
        ocnt, onb = orc.neighbors(kind)
        assert np.array_equal(cnt, ocnt), kind
        assert np.array_equal(nb, _sorted_sets(ocnt, onb)), kind
        assert cnt.mean() > 40, (kind, cnt.mean())
    orc.close()

    # the multi-flaw CSR the device holds equals the oracle's seeding
    orc = O.OracleSystem()
    for d in sc.materials:
        orc.add_material(O.material_from_dict(d))
    orc.add_many(sc.pos, sc.vel, sc.mass, sc.u, sc.mat, sc.fixed)
    orc.seed_flaws_multi(sc.dx, sc.flaws[1])
    ostart, oeps = orc.flaws()
    orc.close()
    assert np.array_equal(ptr, ostart)
    assert np.array_equal(eps, oeps if precision == 0 else oeps.astype(np.float32).astype(np.float64))
