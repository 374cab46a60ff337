"""GPU EAM Hessian, mass weighting and eigenvalues through the C ABI, against the reference's known
answers and the oracle. The Hessian and the mass-weighted matrix are bit-exact; the eigenvalues come
from a different symmetric eigensolver than the oracle's and agree within EIG_TOL of the spectral
radius."""
import numpy as np
import pytest

from openfly_gb300 import workloads as W

from test_hessian import KAT_H00, KAT_H00_TOL, near

pytestmark = pytest.mark.gpu

EIG_TOL = 1e-10  # |lambda_gpu - lambda_oracle| <= EIG_TOL * max |lambda|


def _pair(gpu, oracle, odata, s, rc):
    g = gpu.List(s.extents, s.periodic, rc)
    g.rebuild(s.pos)
    o = oracle.List(s.extents, s.periodic, rc)
    o.rebuild(s.pos, 1)
    return g, o


def _masses(odata, types):
    return np.array([odata.mass(int(t)) for t in types])


def test_kat_block_away_from_minimum(gpu, geam):
    # tests/potential/EAM/eam.cpp:98-146
    s = W.kat_lattice()
    g = gpu.List(s.extents, s.periodic, geam.r_cut())
    g.rebuild(s.pos)
    h = geam.hessian(s.types, s.frozen, g)
    assert np.linalg.norm(h[:3, :3] - KAT_H00) < KAT_H00_TOL


def test_kat_zero_modes_at_minimum(gpu, geam):
    # tests/potential/EAM/eam.cpp:148-188 (unweighted: unit masses)
    s = W.kat_lattice(erase=False)
    g = gpu.List(s.extents, s.periodic, geam.r_cut())
    g.rebuild(s.pos)
    ev = geam.hessian_eigenvalues(s.types, s.frozen, g, masses=np.ones(geam.n_types))
    assert all(near(e, 0.0) for e in ev[:3])
    assert not any(near(e, 0.0) for e in ev[3:])


def _systems():
    rng = np.random.default_rng(21)
    tight = W.bcc_sites(2, 2, 2, W.A_FE) + rng.normal(0, 0.05, (16, 3))
    L = 2 * W.A_FE
    return [
        ("cluster", W.cluster(np.random.default_rng(3), 9.0, n_vac=1, n_h=2).sys, 0.0),
        ("vacancy_cell", W.fe_vacancy_cell(), 0.3),
        ("tight", W.System(tight, np.zeros(16, np.uint32), np.zeros(16, np.uint8), np.full(3, L),
                           np.ones(3, np.int32), {}), 0.0),
    ]


@pytest.mark.parametrize("name,s,skin", _systems(), ids=lambda v: v if isinstance(v, str) else "")
def test_hessian_bit_exact_vs_oracle(gpu, oracle, geam, odata, name, s, skin):
    # periodic images of an atom inside its own cut-off (the "tight" 2x2x2 cell) exercise the
    # self-image overlap term and repeated neighbours g of one atom a
    g, o = _pair(gpu, oracle, odata, s, odata.r_cut + skin)
    h = geam.hessian(s.types, s.frozen, g)
    ref = oracle.eam_hessian(odata, o, s.types, s.frozen, threads=4)
    assert np.array_equal(h, ref), np.abs(h - ref).max()


def test_hessian_in_place_column_path_vs_oracle(gpu, oracle, geam, odata):
    # 2420 atoms: a column block (3n rows of 3 doubles) no longer fits in one CTA's shared memory, so the
    # column pass accumulates in place in the matrix; same contributions, same order, same bits
    rng = np.random.default_rng(8)
    pos = W.bcc_sites(11, 11, 10, W.A_FE) + rng.normal(0, 0.04, (2420, 3))
    ext = np.array([11, 11, 10], float) * W.A_FE
    centre = ext / 2
    frozen = (np.linalg.norm(pos - centre, axis=1) > 5.0).astype(np.uint8)
    assert 20 < int((frozen == 0).sum()) < 100
    s = W.System(pos, np.zeros(2420, np.uint32), frozen, ext, np.ones(3, np.int32), {})
    g, o = _pair(gpu, oracle, odata, s, odata.r_cut)
    h = geam.hessian(s.types, s.frozen, g)
    ref = oracle.eam_hessian(odata, o, s.types, s.frozen, threads=4)
    assert np.array_equal(h, ref), np.abs(h - ref).max()


@pytest.mark.parametrize("name,s,skin", _systems(), ids=lambda v: v if isinstance(v, str) else "")
def test_mass_weighted_eigenvalues_vs_oracle(gpu, oracle, geam, odata, name, s, skin):
    g, o = _pair(gpu, oracle, odata, s, odata.r_cut + skin)
    ev, w = geam.hessian_eigenvalues(s.types, s.frozen, g, weighted=True)
    ref_h = oracle.eam_hessian(odata, o, s.types, s.frozen, threads=4)
    m = _masses(odata, s.types)
    assert np.array_equal(w, oracle.mass_weight(ref_h, m))
    ref = oracle.hessian_eigenvalues(ref_h, m)
    assert np.all(np.diff(ev) >= 0)
    assert np.abs(ev - ref).max() <= EIG_TOL * np.abs(ref).max()
    # frozen atoms contribute 3 zero modes each (find.cpp:1103-1110)
    n_frozen = int(s.frozen.sum())
    if n_frozen:
        tol = 1e-6  # Master::Options::hessian_eigen_zero_tol (saddle/find.hpp:163)
        assert int((np.abs(ev) <= tol).sum()) >= 3 * n_frozen


def test_hessian_more_than_128_neighbours_vs_oracle(gpu, oracle, geam, odata):
    # a bcc lattice compressed to 0.75 of its constant: some atoms have more than 128 neighbours within
    # the cut-off, so the column pass takes their coefficients in more than one chunk
    rng = np.random.default_rng(1)
    a = 0.75 * W.A_FE
    pos = W.bcc_sites(5, 5, 5, a) + rng.normal(0, 0.02, (250, 3))
    frozen = np.zeros(250, np.uint8)
    frozen[:200] = 1
    s = W.System(pos, np.zeros(250, np.uint32), frozen, np.full(3, 5 * a), np.ones(3, np.int32), {})
    g, o = _pair(gpu, oracle, odata, s, odata.r_cut)
    assert int(o.neighbours(odata.r_cut)[0].max()) > 128
    h = geam.hessian(s.types, s.frozen, g)
    ref = oracle.eam_hessian(odata, o, s.types, s.frozen, threads=4)
    assert np.array_equal(h, ref), np.abs(h - ref).max()


@pytest.mark.parametrize("radius,lo,hi", [(8.0, 460, 640), (8.9, 650, 900)], ids=["cluster16", "global_rows"])
def test_large_active_block_eigenvalues_vs_oracle(gpu, oracle, geam, odata, radius, lo, hi):
    # active blocks past the 8-CTA shared-memory size (M > ~460 coordinates: a 16-CTA cluster) and past
    # the 16-CTA one (M > ~640: rows in the global matrix)
    rng = np.random.default_rng(5)
    pos = W.bcc_sites(8, 8, 8, W.A_FE) + rng.normal(0, 0.04, (1024, 3))
    ext = np.full(3, 8 * W.A_FE)
    frozen = (np.linalg.norm(pos - ext / 2, axis=1) > radius).astype(np.uint8)
    M = 3 * int((frozen == 0).sum())
    assert lo < M < hi, M
    s = W.System(pos, np.zeros(1024, np.uint32), frozen, ext, np.ones(3, np.int32), {})
    g, o = _pair(gpu, oracle, odata, s, odata.r_cut)
    ev, w = geam.hessian_eigenvalues(s.types, s.frozen, g, weighted=True)
    ref = oracle.hessian_eigenvalues(oracle.eam_hessian(odata, o, s.types, s.frozen, threads=4), _masses(odata, s.types))
    assert np.all(np.diff(ev) >= 0)
    assert np.abs(ev - ref).max() <= EIG_TOL * np.abs(ref).max()


def test_explicit_masses(gpu, oracle, geam, odata):
    s = W.cluster(np.random.default_rng(8), 8.0, n_h=1).sys
    g, o = _pair(gpu, oracle, odata, s, odata.r_cut)
    per_type = np.array([50.0, 2.0])
    ev, w = geam.hessian_eigenvalues(s.types, s.frozen, g, masses=per_type, weighted=True)
    ref_h = oracle.eam_hessian(odata, o, s.types, s.frozen)
    assert np.array_equal(w, oracle.mass_weight(ref_h, per_type[s.types]))


def test_spline_out_of_bounds_is_reported(gpu, geam):
    pos = np.full((200, 3), 5.0) + np.random.default_rng(0).normal(0, 1e-3, (200, 3))
    g = gpu.List([10.0, 10.0, 10.0], [0, 0, 0], geam.r_cut())
    g.rebuild(pos)
    with pytest.raises(gpu.SplineOutOfBounds):
        geam.hessian(np.zeros(200, np.uint32), np.zeros(200, np.uint8), g)
    ok = np.array([[1.0, 1.0, 1.0], [3.5, 1.0, 1.0]])
    g.rebuild(ok)
    h = geam.hessian(np.zeros(2, np.uint32), np.zeros(2, np.uint8), g)
    assert h.shape == (6, 6) and np.isfinite(h).all()


def test_batch_matches_single_calls_and_oracle(gpu, oracle, geam, odata):
    # flygpu_hessian_eigenvalues_batch: 10 clusters of mixed sizes on 4 worker streams
    from openfly_gb300 import search as S

    clusters = W.search_clusters(n=10, seed=31)
    systems = [S.from_cluster(c) for c in clusters]
    batch = S.hessian_eigenvalues_batch(geam, systems, workers=4)
    assert len(batch) == len(systems)
    for c, ev in zip(clusters, batch):
        s = c.sys
        g, o = _pair(gpu, oracle, odata, s, odata.r_cut)
        assert np.array_equal(ev, geam.hessian_eigenvalues(s.types, s.frozen, g))
        ref = oracle.hessian_eigenvalues(oracle.eam_hessian(odata, o, s.types, s.frozen), _masses(odata, s.types))
        assert np.abs(ev - ref).max() <= EIG_TOL * np.abs(ref).max()


def test_batch_reports_the_failing_system(gpu, geam):
    from openfly_gb300 import search as S

    systems = [S.from_cluster(c) for c in W.search_clusters(n=3, seed=2)]
    systems[1].types = np.full(systems[1].n, 7, np.uint32)  # no such type in the potential
    with pytest.raises(gpu.FlyGPUError, match="system 1"):
        S.hessian_eigenvalues_batch(geam, systems, workers=2)
