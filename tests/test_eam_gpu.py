"""GPU EAM energy/gradient vs the reference's known answers and the oracle."""
import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# MIXED precision bound (binary32 pair terms, binary64 accumulation) against the binary64 oracle,
# stated as a norm-wise relative gradient error and a per-atom energy error.
MIXED_GRAD_REL = 2e-5
MIXED_E_PER_ATOM = 2e-6


def _pair(gpu, oracle, geam, odata, s, rc_list):
    g = gpu.List(s.extents, s.periodic, rc_list)
    g.rebuild(s.pos)
    o = oracle.List(s.extents, s.periodic, rc_list)
    o.rebuild(s.pos, 1)
    return g, o


def test_tables_bit_exact_vs_oracle(gpu, geam, odata):
    # DataEAM (data.cpp:67-153) + Spline (spline.cpp:27-103): every function's binary64 coefficients
    nt = geam.n_types
    for a in range(nt):
        assert np.array_equal(geam.table(0, a), odata.table(0, a))
        for b in range(nt):
            assert np.array_equal(geam.table(1, a, b), odata.table(1, a, b))
            assert np.array_equal(geam.table(2, a, b), odata.table(2, a, b))


def test_kat_fp64(gpu, oracle, geam, odata):
    # tests/potential/EAM/eam.cpp:119,125
    s = W.kat_lattice()
    g = gpu.List(s.extents, s.periodic, geam.r_cut())
    g.rebuild(s.pos)
    e, grad = geam.energy_gradient(s.types, s.frozen, g, gpu.FP64)
    assert abs(e - -2748.5339306065985) < 1e-9
    assert np.linalg.norm(grad[0] - np.full(3, -0.19182439085483005)) < 1e-10
    assert geam.energy(s.types, s.frozen, g) == e


def test_fp64_gradient_bit_exact_vs_oracle(gpu, oracle, geam, odata):
    for s in (W.kat_lattice(), W.fe_vacancy_cell(), W.fe_h_crystal(n_cells=6)):
        g, o = _pair(gpu, oracle, geam, odata, s, odata.r_cut + 0.17)
        grad = geam.gradient(s.types, s.frozen, g, gpu.FP64)
        ref = oracle.eam_gradient(odata, o, s.types, s.frozen)
        assert np.array_equal(grad, ref)
        e = geam.energy(s.types, s.frozen, g, gpu.FP64)
        e_ref = oracle.eam_energy(odata, o, s.types)
        assert abs(e - e_ref) <= 1e-12 * abs(e_ref)


def test_frozen_atoms_have_zero_gradient(gpu, oracle, geam, odata):
    c = W.cluster(np.random.default_rng(3), 9.0, n_vac=1, n_h=2)
    s = c.sys
    g, o = _pair(gpu, oracle, geam, odata, s, odata.r_cut + 0.2)
    grad = geam.gradient(s.types, s.frozen, g, gpu.FP64)
    assert np.all(grad[s.frozen == 1] == 0)
    assert np.array_equal(grad, oracle.eam_gradient(odata, o, s.types, s.frozen))


def test_update_then_gradient_bit_exact(gpu, oracle, geam, odata):
    s = W.fe_vacancy_cell()
    g, o = _pair(gpu, oracle, geam, odata, s, odata.r_cut + 0.3)
    rng = np.random.default_rng(5)
    for _ in range(4):
        d = rng.normal(0, 0.02, s.pos.shape)
        g.update(d)
        o.update(d)
        assert np.array_equal(geam.gradient(s.types, s.frozen, g), oracle.eam_gradient(odata, o, s.types, s.frozen))


def test_mixed_within_stated_tolerance(gpu, oracle, geam, odata):
    for s in (W.fe_vacancy_cell(), W.fe_h_crystal(n_cells=8)):
        g, o = _pair(gpu, oracle, geam, odata, s, odata.r_cut + 0.3)
        e, grad = geam.energy_gradient(s.types, s.frozen, g, gpu.MIXED)
        ref = oracle.eam_gradient(odata, o, s.types, s.frozen)
        e_ref = oracle.eam_energy(odata, o, s.types)
        rel = np.linalg.norm(grad - ref) / np.linalg.norm(ref)
        assert rel < MIXED_GRAD_REL, rel
        assert abs(e - e_ref) / s.n < MIXED_E_PER_ATOM


def test_spline_out_of_bounds_is_reported(gpu, geam):
    # Two atoms closer than any tabulated density argument keep r in range; an absurd density is
    # produced by stacking many atoms at one point, which drives rho beyond the F table.
    pos = np.full((200, 3), 5.0) + np.random.default_rng(0).normal(0, 1e-3, (200, 3))
    g = gpu.List([10.0, 10.0, 10.0], [0, 0, 0], geam.r_cut())
    g.rebuild(pos)
    with pytest.raises(gpu.SplineOutOfBounds):
        geam.gradient(np.zeros(200, np.uint32), np.zeros(200, np.uint8), g)
    # the handle stays usable afterwards
    ok = np.array([[1.0, 1.0, 1.0], [3.5, 1.0, 1.0]])
    g.rebuild(ok)
    geam.gradient(np.zeros(2, np.uint32), np.zeros(2, np.uint8), g)
