"""Master::perturb and Master::find_batch on the device vs the oracle's single-thread restatement.

perturb (find.cpp:1147-1214) draws from the reference's xoshiro256** stream through libstdc++'s normal
distribution: positions, axis, the stddev drawn and the stream's state afterwards are bit-identical to the
oracle's (which calls libstdc++'s std::normal_distribution itself) on a periodic cell and on a cluster with
a frozen shell, the neighbours taken from the device list in List::for_neighbours order.

find_batch (find.cpp:684-755): spline-out-of-bounds failures are injected host-side, with a copy of the
potential whose F(rho) grid ends just above the densities of the minimum, so some perturbed starts lie
outside the table. The retries, the perturbed starts of the attempts that ran (bit for bit) and the
stream's final state equal the oracle's; exit codes agree; a batch whose searches keep failing raises after
three retries in both.
"""
import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(gpu):
    from openfly_gb300 import search

    return search


def _truncated_table(path, n_rho_keep):
    """wen.eam.fs with every F(rho) grid cut to its first n_rho_keep samples (a multiple of 5)."""
    lines = open(W.TABLE).read().splitlines()
    head = lines[4].split()
    n_rho, n_r, n_types = int(head[0]), int(head[2]), int(lines[3].split()[0])
    out = lines[:4] + [" ".join([str(n_rho_keep)] + head[1:])]
    k = 5
    for _ in range(n_types):
        out.append(lines[k])
        out += lines[k + 1:k + 1 + n_rho_keep // 5]
        k += 1 + n_rho // 5
        out += lines[k:k + n_types * (n_r // 5)]
        k += n_types * (n_r // 5)
    out += lines[k:]
    open(path, "w").write("\n".join(out) + "\n")
    return path


@pytest.fixture(scope="module")
def minimum(oracle, odata):
    """The vacancy cell relaxed to its minimum (binary64 oracle LBFGS::minimise)."""
    s = W.fe_vacancy_cell()
    opt = oracle.LBFGSOptions.defaults(f2norm=1e-8)
    failed, _, x, _ = oracle.lbfgs_minimise(odata, opt, s.extents, s.periodic, s.pos, s.types, s.frozen)
    assert not failed
    return W.System(np.asarray(x).reshape(-1, 3), s.types, s.frozen, s.extents, s.periodic, dict(s.meta))


def _check_perturb(gpu, oracle, S, sys_, centre, seeds):
    nl = gpu.List(sys_.extents, sys_.periodic, 4.0)
    nl.rebuild(sys_.pos)
    onl = oracle.List(sys_.extents, sys_.periodic, 4.0)
    onl.rebuild(sys_.pos, 1)
    for seed in seeds:
        g = S.Xoshiro(seed)
        st = np.array(seed, np.uint64)
        for _ in range(3):  # consecutive perturbations continue the same stream
            p, a, sd = S.perturb(nl, centre, sys_.pos, sys_.frozen, g, 0.6, 4.0)
            po, ao, sdo, st = oracle.perturb(onl, centre, sys_.pos, sys_.frozen, 0.6, 4.0, st)
            assert sd == sdo
            assert np.array_equal(p, po)
            assert np.array_equal(a, ao)
            assert g.state == tuple(int(x) for x in st)


def test_perturb_bit_identical_to_oracle(gpu, oracle, S, minimum):
    _check_perturb(gpu, oracle, S, minimum, minimum.meta["centre"], ([1, 3, 3, 4], [7, 7, 7, 7], [2 ** 63, 5, 9, 1]))
    c = W.cluster(np.random.default_rng(8), 10.0, n_vac=1, n_h=1)
    _check_perturb(gpu, oracle, S, c.sys, c.centre, ([1, 3, 3, 4], [3, 1, 4, 1]))


def _geo(pos, centre):
    d = np.linalg.norm(pos - pos[centre], axis=1)
    return np.concatenate([[centre], np.flatnonzero((d < 4.0) & (np.arange(len(pos)) != centre))])


def test_find_batch_retries_match_oracle(gpu, oracle, S, minimum, tmp_path):
    path = _truncated_table(str(tmp_path / "short_f.eam.fs"), 1800)  # F(rho) up to rho ~ 36
    eam, od = gpu.EAM(path), oracle.EAMData(path)
    m, c = minimum, minimum.meta["centre"]
    nl = gpu.List(m.extents, m.periodic, 4.0)
    nl.rebuild(m.pos)
    onl = oracle.List(m.extents, m.periodic, 4.0)
    onl.rebuild(m.pos, 1)
    gdim = S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=300)
    odim = oracle.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=300)
    glb, olb = S.LBFGSOptions.defaults(), oracle.LBFGSOptions.defaults()
    geo = _geo(m.pos, c)
    masses = [od.mass(int(t)) for t in m.types]
    seed = [1, 3, 3, 4]
    ocache, gcache = [], []
    ref, st = oracle.find_batch(od, odim, olb, 0, m.extents, m.periodic, m.pos, m.types, m.frozen, c, onl, ocache, 6,
                                np.array(seed, np.uint64), geo, masses, 3)
    g = S.Xoshiro(seed)
    out = S.find_batch(eam, 0, S.Search(m.pos, m.types, m.frozen, m.extents, m.periodic), c, nl, gcache, 6, g, geo,
                       precision=gpu.FP64, dimer=gdim, lbfgs=glb, zero_modes=3)
    assert sum(r["retries"] for r in ref) > 0  # the injected failures happened
    assert [o["retries"] for o in out] == [r["retries"] for r in ref]
    for o, r in zip(out, ref):
        assert np.array_equal(o["start"][0], r["start"][0])
        assert np.array_equal(o["start"][1], r["start"][1])
    assert g.state == tuple(int(x) for x in st)
    same = sum(o["exit_code"] == r["exit"] for o, r in zip(out, ref))
    assert same >= len(ref) - 1, ([o["exit_code"] for o in out], [r["exit"] for r in ref])


def test_find_batch_raises_after_three_retries(gpu, oracle, S, minimum, tmp_path):
    path = _truncated_table(str(tmp_path / "shorter_f.eam.fs"), 1400)  # F(rho) up to rho ~ 28
    eam, od = gpu.EAM(path), oracle.EAMData(path)
    m, c = minimum, minimum.meta["centre"]
    nl = gpu.List(m.extents, m.periodic, 4.0)
    nl.rebuild(m.pos)
    onl = oracle.List(m.extents, m.periodic, 4.0)
    onl.rebuild(m.pos, 1)
    opts = S.MasterOptions(stddev=1.5)
    with pytest.raises(RuntimeError, match="Consecutive spline-out-of-bounds"):
        oracle.find_batch(od, oracle.DimerOptions.defaults(), oracle.LBFGSOptions.defaults(), 0, m.extents, m.periodic,
                          m.pos, m.types, m.frozen, c, onl, [], 2, np.array([1, 3, 3, 4], np.uint64), _geo(m.pos, c),
                          [od.mass(0)] * m.n, 3, stddev=1.5)
    with pytest.raises(RuntimeError, match="Consecutive spline-out-of-bounds"):
        S.find_batch(eam, 0, S.Search(m.pos, m.types, m.frozen, m.extents, m.periodic), c, nl, [], 2,
                     S.Xoshiro([1, 3, 3, 4]), _geo(m.pos, c), opts=opts, precision=gpu.FP64, zero_modes=3)
