"""Edge cases of the batched search path: an error in one search ends that search alone, descriptions
the reference would reject are rejected before any launch, and a cluster whose state does not fit a
CTA's shared memory (so it runs from global memory) still matches the oracle."""
import dataclasses

import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu

E_TOL = 1e-3  # eV
SAME_SADDLE_A = 0.05


@pytest.fixture(scope="module")
def S(gpu):
    from openfly_gb300 import search

    return search


def _opts(S, O=None):
    g = S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000)
    o = O.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000) if O is not None else None
    return g, o


def _stacked(cl, k, radius):
    """The cluster with its k atoms nearest the centre moved into a ball of `radius` around it."""
    s = cl.sys
    d = np.linalg.norm(s.pos - s.pos[cl.centre], axis=1)
    near = np.argsort(d)[:k]
    rng = np.random.default_rng(k)
    v = rng.normal(size=(k, 3))
    pos = s.pos.copy()
    pos[near] = s.pos[cl.centre] + v / np.linalg.norm(v, axis=1, keepdims=True) * radius * rng.random((k, 1))
    return dataclasses.replace(cl, sys=dataclasses.replace(s, pos=pos))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_errors_stay_with_their_search(gpu, geam, S, precision):
    # A search whose density leaves the embedding table (atoms stacked at one point) ends with
    # SPLINE_OOB and one whose neighbour count exceeds the per-search capacity ends with
    # NLIST_OVERFLOW; kernels never trap, and the other searches of the batch are untouched.
    prec = gpu.FP64 if precision == "fp64" else gpu.MIXED
    rng = np.random.default_rng(21)
    good = [W.cluster(rng, 8.0) for _ in range(3)]
    oob = _stacked(W.cluster(rng, 8.0), 20, 0.01)
    crowd = _stacked(W.cluster(rng, 9.0), 120, 2.0)
    opt, _ = _opts(S)
    t = S.Tuning(2, 128, 2)
    mix = S.Batch(geam, [S.from_cluster(c) for c in (good[0], oob, good[1], crowd, good[2])], precision=prec,
                  dimer=opt)
    mix.run(t)
    res, pos, _ = mix.results()
    assert [r["status"] for r in res] == [gpu.OK, gpu.SPLINE_OOB, gpu.OK, gpu.NLIST_OVERFLOW, gpu.OK], res
    alone = S.Batch(geam, [S.from_cluster(c) for c in good], precision=prec, dimer=opt)
    alone.run(t)
    ra, pa, _ = alone.results()
    for a, b, k in zip(ra, pa, (0, 2, 4)):
        assert a == res[k]
        assert np.array_equal(b, pos[k])


def test_invalid_descriptions_are_rejected(gpu, geam, S):
    rng = np.random.default_rng(4)
    cl = W.cluster(rng, 7.0)
    opt, _ = _opts(S)
    s = cl.sys
    frozen_all = S.Search(s.pos, s.types, np.ones_like(s.frozen), s.extents, s.periodic, axis=np.zeros_like(s.pos))
    bad_type = S.Search(s.pos, np.full_like(s.types, 7), s.frozen, s.extents, s.periodic, axis=cl.axis)
    small_periodic = S.Search(s.pos, s.types, s.frozen, np.full(3, 8.0), np.ones(3, np.int32), axis=cl.axis)
    big = W.cluster(rng, 23.0)  # more than 4096 atoms
    assert big.sys.n > 4096
    too_big = S.from_cluster(big)
    for req in (frozen_all, bad_type, small_periodic, too_big):
        with pytest.raises(gpu.FlyGPUError) as e:
            S.Batch(geam, [S.from_cluster(cl), req], precision=gpu.MIXED, dimer=opt)
        assert e.value.status == gpu.INVALID_ARG


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_unstaged_cluster_matches_oracle(gpu, oracle, odata, geam, S, precision):
    # ~990 atoms, ~230 of them mobile: the search's vectors (39 x 3 x 230 doubles) exceed the 100 KB a
    # CTA stages, so the kernel works on them in global memory.
    O = oracle
    prec = gpu.FP64 if precision == "fp64" else gpu.MIXED
    cl = W.cluster(np.random.default_rng(31), 14.0)
    na = int((cl.sys.frozen == 0).sum())
    assert 39 * 3 * na * 8 > 100 * 1024
    gopt, oopt = _opts(S, O)
    b = S.Batch(geam, [S.from_cluster(cl)], precision=prec, dimer=gopt)
    b.run(S.Tuning(2, 256, 1))
    res, pos, _ = b.results()
    s = cl.sys
    ref = O.dimer_find_sp(odata, oopt, s.extents, s.periodic, s.pos, cl.axis, s.types, s.frozen)
    assert res[0]["status"] == gpu.OK
    assert res[0]["exit_code"] == ref["exit"]
    if ref["exit"] == 0 and np.abs(pos[0] - ref["x"]).max() < SAME_SADDLE_A:
        nl = O.List(s.extents, s.periodic, odata.r_cut)
        nl.rebuild(ref["x"], 1)
        assert abs(res[0]["energy"] - O.eam_energy(odata, nl, s.types)) < E_TOL
