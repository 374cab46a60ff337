"""Host-side logic without a GPU: the synthetic workloads match the stated configurations, the bench's
step schedule follows the reference's skin rule, and the pathway helpers agree with the oracle's
restatements of Master's glue (find.cpp:148-243, utility/lattice.hpp:203-226)."""
import numpy as np
import pytest

from openfly_gb300 import workloads as W


def test_fe_h_crystal_sizes():
    # 2 n^3 bcc sites, 0.1 % vacated, H = 0.05 % of the Fe count, periodic, sigma 0.05 A
    s = W.fe_h_crystal(n_cells=12)
    sites = 2 * 12 ** 3
    n_vac = int(round(0.001 * sites))
    n_fe = sites - n_vac
    assert int((s.types == 0).sum()) == n_fe
    assert int((s.types == 1).sum()) == int(round(0.0005 * n_fe))
    assert s.periodic.tolist() == [1, 1, 1]
    assert not s.frozen.any()
    assert np.all((s.pos >= -1.0) & (s.pos <= s.extents + 1.0))


def test_search_clusters():
    cl = W.search_clusters(n=64, seed=3)
    sizes = [c.sys.n for c in cl]
    assert 50 <= min(sizes) and max(sizes) <= 520
    for c in cl[:8]:
        s = c.sys
        assert s.periodic.tolist() == [0, 0, 0]
        assert np.all(s.pos > 0) and np.all(s.pos < s.extents)  # enclosed with a margin
        mobile = s.frozen == 0
        assert mobile.any() and (~mobile).any()
        assert np.isclose(np.linalg.norm(c.axis), 1.0)
        assert not c.axis[~mobile].any()  # the axis lives on mobile atoms only


def test_served_requests():
    reqs = W.served_requests(n_env=6, seed=5)
    envs = {e for e, _ in reqs}
    assert len(envs) == 6
    per = [sum(1 for e, _ in reqs if e == k) for k in envs]
    assert min(per) >= 8 and max(per) <= 32
    for _, c in reqs[:5]:
        assert c.sys.frozen.any() and (c.sys.frozen == 0).any()


def test_bench_schedule_follows_the_skin_rule():
    import bench

    sched = bench.schedule(100)
    acc, rebuilds = 0.0, 0
    for j, sign, rb in sched:
        acc += bench.STEP_DISP
        if acc > 0.5 * bench.SKIN:
            assert rb
            acc = 0.0
            rebuilds += 1
        else:
            assert not rb
    assert rebuilds == sum(1 for *_, rb in sched if rb) > 0
    assert [sign for _, sign, _ in sched[:4]] == [1.0, -1.0, 1.0, -1.0]


@pytest.mark.parametrize("seed", [1, 2])
def test_furthest_atom_matches_oracle(oracle, seed):
    from openfly_gb300 import search as S

    rng = np.random.default_rng(seed)
    ext = 5.0 + 10.0 * rng.random(3)
    per = (rng.random(3) < 0.5).astype(np.int32)
    pos = rng.random((200, 3)) * ext
    for i in (0, 17, 199):
        assert S.furthest_atom(pos, ext, per, i) == oracle.furthest_atom(pos, ext, per, i)


def test_centroid_align():
    from openfly_gb300 import search as S

    rng = np.random.default_rng(7)
    x, w = rng.normal(size=(50, 3)), rng.normal(size=(50, 3)) + 3.0
    y = S.centroid_align(x, w)
    assert np.allclose(S.centroid(y), S.centroid(w), atol=1e-12)
    assert np.allclose(y - x, (S.centroid(w) - S.centroid(x))[None, :])


def test_master_options_defaults():
    # saddle/find.hpp:112,120,129,138,163,184
    from openfly_gb300 import search as S

    o = S.MasterOptions()
    assert (o.basin_tol, o.stationary_tol, o.capture_r_tol, o.capture_E_tol) == (0.05, 0.025, 0.05, 0.01)
    assert (o.hessian_eigen_zero_tol, o.nudge_frac) == (1e-6, 0.01)
    assert S.MasterOptions(basin_tol=0.2).stationary_tol == 0.1  # stationary_tol = basin_tol / 2


def test_mode_classification():
    # the eigenvalue loops of find.cpp:851-865 and :1116-1126: negative below -tol, zero within tol,
    # the log of the rest summed
    from openfly_gb300 import search as S

    freq = np.array([-2.0, -1e-7, 0.0, 5e-7, 1.0, np.e])
    neg, zeros, logp = S._modes(freq, 1e-6)
    assert (neg, zeros) == (1, 3)
    assert np.isclose(logp, 1.0)


def test_bench_replica_value_and_traffic_table():
    import bench

    # N replicas, each n atoms x K steps, over the slowest rank's time (whole-job weak-scaling throughput)
    assert bench.replica_value(1000, 4, 10, 2.0) == pytest.approx(1000 * 4 * 10 / 2e-3)
    # the committed per-atom DRAM traffic of the binary32 passes, scaled to the bench's atom count
    t = bench.traffic_from_profile("k_force32", 1_000_000)
    assert t is not None and 200e6 < t < 400e6
    assert bench.traffic_from_profile("no_such_kernel", 10) is None


def test_desc_array_equals_per_search_descriptors():
    # the column-wise SearchDesc builder of batches, server submissions and Hessian batches gives the
    # per-search desc() contents, pointed-to bytes included (dimer and minimise modes, a saddle history,
    # an in_min, a binary32 position array that needs converting)
    import ctypes as C

    from openfly_gb300 import search as S

    cl = W.search_clusters(n=24, seed=3)
    reqs = [S.from_cluster(c) for c in cl]
    reqs[3].hist = [reqs[3].pos + 0.1, reqs[3].pos - 0.2]
    reqs[3].in_min = reqs[3].pos + 0.05
    reqs[3].theta_tol = 0.3
    reqs[5] = S.from_cluster(cl[5], mode=S.MINIMISE)
    reqs[7].pos = reqs[7].pos.astype(np.float32)
    k1, k2 = [], []
    a = (S.SearchDesc * len(reqs))(*[s.desc(k1) for s in reqs])
    b = S.desc_array(reqs, k2)

    def deref(d, field, cnt, ctype):
        p = getattr(d, field)
        return None if not p else bytes((ctype * cnt).from_address(p))

    for x, y in zip(a, b):
        n = x.n
        for fld in ("n", "mode", "n_hist", "theta_tol"):
            assert getattr(x, fld) == getattr(y, fld)
        assert list(x.extents) == list(y.extents) and list(x.periodic) == list(y.periodic)
        for fld, cnt, ct in (("pos", 3 * n, C.c_double), ("axis", 3 * n, C.c_double), ("types", n, C.c_uint32),
                             ("frozen", n, C.c_uint8), ("in_min", 3 * n, C.c_double),
                             ("hist", 3 * n * max(1, x.n_hist), C.c_double)):
            assert deref(x, fld, cnt, ct) == deref(y, fld, cnt, ct), fld
    assert len(S.desc_array([], [])) == 1
