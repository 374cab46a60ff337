"""GPU neighbour list vs the oracle: identical neighbour sequences (order included), brute-force sets."""
import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _random_box(rng, full_periodic=False):
    ext = 1.0 + 9.0 * rng.random(3)
    per = np.ones(3, np.int32) if full_periodic else (rng.random(3) < 0.5).astype(np.int32)
    n = int(rng.integers(100, 1001))
    return ext, per, rng.random((n, 3)) * ext


def _same_lists(a, b):
    ca, ia, da = a
    cb, ib, db = b
    assert np.array_equal(ca, cb)
    assert np.array_equal(ia, ib)
    assert np.array_equal(da, db)  # bit-exact dr, same visiting order


@pytest.mark.parametrize("seed", [1334, 7])
def test_fuzz_boxes_match_oracle_exactly(gpu, oracle, seed):
    # The reference's fuzz (tests/neigh/list.cpp:167-208): random boxes, mixed periodicity, rc = min/3.
    rng = np.random.default_rng(seed)
    for _ in range(20):
        ext, per, pos = _random_box(rng)
        rc = ext.min() / 3
        g = gpu.List(ext, per, rc)
        g.rebuild(pos)
        o = oracle.List(ext, per, rc)
        o.rebuild(pos, 1)
        assert g.num_ghosts == o.num_ghosts
        _same_lists(g.neighbours(rc), o.neighbours(rc))
        # and the set equals the O(N^2) minimum-image brute force
        cg, ig, _ = g.neighbours(rc)
        cb, ib, _ = oracle.brute_neighbours(ext, per, pos, rc)
        assert np.array_equal(cg, cb)
        off = np.r_[0, np.cumsum(cg)]
        for a in range(len(cg)):
            assert np.array_equal(np.sort(ig[off[a]:off[a + 1]]), ib[off[a]:off[a + 1]])


def test_update_matches_oracle_exactly(gpu, oracle):
    # tests/neigh/list.cpp:210-250: list at rc + 2 skin, displacement 0.99 skin, then compare.
    rng = np.random.default_rng(11)
    for _ in range(6):
        ext, per, pos = _random_box(rng, full_periodic=True)
        rc, skin = ext.min() / 3, 0.1
        g = gpu.List(ext, per, rc + 2 * skin)
        o = oracle.List(ext, per, rc + 2 * skin)
        g.rebuild(pos)
        o.rebuild(pos, 1)
        d = rng.random(pos.shape)
        d = d / np.linalg.norm(d, axis=1, keepdims=True) * (skin * 0.99)
        for _k in range(3):
            g.update(d / 3)
            o.update(d / 3)
        _same_lists(g.neighbours(rc), o.neighbours(rc))
        cb, ib, _ = oracle.brute_neighbours(ext, per, pos - d, rc)
        assert np.array_equal(g.neighbours(rc)[0], cb)


def test_vacancy_cell_and_kat_cells(gpu, oracle, odata):
    for s in (W.kat_lattice(), W.fe_vacancy_cell()):
        rc = odata.r_cut + 0.3
        g = gpu.List(s.extents, s.periodic, rc)
        o = oracle.List(s.extents, s.periodic, rc)
        g.rebuild(s.pos)
        o.rebuild(s.pos, 1)
        _same_lists(g.neighbours(odata.r_cut), o.neighbours(odata.r_cut))


def test_empty_and_errors(gpu):
    g = gpu.List([10.0, 10.0, 10.0], [1, 1, 1], 3.0)
    g.rebuild(np.zeros((0, 3)))
    assert g.size() == 0
    with pytest.raises(gpu.FlyGPUError):
        gpu.List([2.0, 10.0, 10.0], [1, 1, 1], 3.0)  # r_cut larger than an extent (hypergrid.hpp:46-48)
    with pytest.raises(gpu.FlyGPUError):
        g.neighbours(3.5)  # r_cut above the list's cut-off (list.hpp:141-143)


def test_dense_clump_regrows_capacity(gpu, oracle):
    # The first neighbour capacity is sized from the mean density; a clump far denser than the mean
    # overflows it, and the rebuild regrows the capacity once (as List grows its vectors, list.cpp:91-94).
    rng = np.random.default_rng(3)
    ext = np.array([20.0, 20.0, 20.0])
    per = np.array([1, 0, 1], np.int32)
    background = rng.random((1500, 3)) * ext
    v = rng.normal(size=(200, 3))
    clump = 10.0 + v / np.linalg.norm(v, axis=1, keepdims=True) * 1.5 * rng.random((200, 1)) ** (1 / 3)
    pos = np.concatenate([background, clump])
    rc = 3.0
    g = gpu.List(ext, per, rc)
    o = oracle.List(ext, per, rc)
    g.rebuild(pos)
    o.rebuild(pos, 1)
    _same_lists(g.neighbours(rc), o.neighbours(rc))


def test_tightest_periodic_box(gpu, oracle):
    # Extents just above the cut-off in every periodic direction: the most ghosts per atom a valid
    # box allows (about 26 per atom, under the reference's MAX_GHOST_RATIO capacity, list.hpp:78).
    rng = np.random.default_rng(9)
    rc = 3.0
    ext = np.full(3, rc * 1.02)
    per = np.ones(3, np.int32)
    pos = rng.random((40, 3)) * ext
    g = gpu.List(ext, per, rc)
    o = oracle.List(ext, per, rc)
    g.rebuild(pos)
    o.rebuild(pos, 1)
    assert g.num_ghosts == o.num_ghosts
    assert g.num_ghosts > 20 * 40
    _same_lists(g.neighbours(rc), o.neighbours(rc))
