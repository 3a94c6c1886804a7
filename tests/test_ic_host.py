"""The workload generators (deorbit_gb300/ic.py) on the CPU: exact particle
counts of the 1,048,576- and graded-lattice workloads, the 256-impact sweep's
size distribution, and that every generator is a pure function of its seed."""
import numpy as np

from deorbit_gb300 import ic


def same(a, b):
    return (a.n == b.n and np.array_equal(a.pos, b.pos) and np.array_equal(a.vel, b.vel)
            and np.array_equal(a.mass, b.mass) and np.array_equal(a.mat, b.mat))


def test_grazing_has_exactly_2_20_particles():
    sc = ic.grazing()
    assert sc.n == 1 << 20 and sc.pos.shape == (sc.n, 3)
    assert set(np.unique(sc.mat)) == {0, 1}           # granite target, iron impactor
    imp = sc.mat == 1
    assert np.all(np.linalg.norm(sc.vel[imp], axis=1) > 7999.0) and np.all(sc.vel[~imp] == 0.0)
    assert sc.params["damage_on"] == 1


def test_graded_lattice_exact_count_and_grading():
    sc = ic.large_graded(n_total=200_000)
    assert sc.n == 200_000
    tgt = sc.mat == 0
    h0 = sc.h0[tgt]
    z = sc.pos[tgt, 2]
    # spacing grows with depth: the deepest layer is the coarsest
    assert h0[np.argmin(z)] > 2.0 * h0[np.argmax(z)]
    assert np.all(np.diff(h0[np.argsort(-z)]) >= -1e-9 * h0.max())


def test_batch_sweep_sizes():
    scs = ic.batch_impacts(256)
    n = np.array([s.n for s in scs])
    assert len(scs) == 256 and n.min() >= 0.9 * 5000 and n.max() <= 1.1 * 80000
    # log-uniform: about half of the impacts below the geometric mean of the range
    below = np.mean(np.log(n) < 0.5 * (np.log(5000) + np.log(80000)))
    assert 0.35 < below < 0.65


def test_generators_are_pure_functions_of_the_seed():
    assert same(ic.grazing(n_total=20_000), ic.grazing(n_total=20_000))
    assert not same(ic.grazing(n_total=20_000), ic.grazing(n_total=20_000, seed=7))
    a, b = ic.batch_impacts(8), ic.batch_impacts(8)
    assert all(same(x, y) for x, y in zip(a, b))
    assert same(ic.large_graded(n_total=50_000), ic.large_graded(n_total=50_000))
