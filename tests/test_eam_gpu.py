"""GPU EAM energy/gradient vs the reference's known answers and the oracle."""
import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# MIXED precision bounds (binary32 pair terms, binary64 accumulation) against the binary64 oracle: the
# gradient within 1e-6 norm-wise relative (||g - g_ref|| / ||g_ref||), every component within 1e-6 eV/A
# absolute plus 1e-5 of its own size, and the energy within 2e-6 eV per atom.
MIXED_GRAD_REL = 1e-6
MIXED_COMP_ABS = 1e-6
MIXED_COMP_REL = 1e-5
MIXED_E_PER_ATOM = 2e-6


def mixed_errors(grad, ref):
    """Norm-wise relative error, worst component error in eV/A, worst component error relative to the
    component (over components of at least 1e-2 eV/A)."""
    err = np.abs(grad - ref)
    big = np.abs(ref) >= 1e-2
    return (np.linalg.norm(grad - ref) / np.linalg.norm(ref), float(err.max()),
            float((err[big] / np.abs(ref[big])).max()))


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


def _check_mixed(grad, ref, e, e_ref, n):
    rel, comp_abs, comp_rel = mixed_errors(grad, ref)
    assert rel < MIXED_GRAD_REL, rel
    assert np.all(np.abs(grad - ref) <= MIXED_COMP_ABS + MIXED_COMP_REL * np.abs(ref)), (comp_abs, comp_rel)
    assert abs(e - e_ref) / n < MIXED_E_PER_ATOM


def test_mixed_within_stated_tolerance(gpu, oracle, geam, odata):
    # the vacancy cell (sigma 0.02 A: small forces, the hardest relative case) and Fe-H crystals with
    # vacancies and H at sigma 0.05 A
    for s in (W.fe_vacancy_cell(), W.fe_h_crystal(n_cells=8), W.fe_h_crystal(n_cells=12, seed=5)):
        g, o = _pair(gpu, oracle, geam, odata, s, odata.r_cut + 0.3)
        e, grad = geam.energy_gradient(s.types, s.frozen, g, gpu.MIXED)
        ref = oracle.eam_gradient(odata, o, s.types, s.frozen)
        e_ref = oracle.eam_energy(odata, o, s.types)
        _check_mixed(grad, ref, e, e_ref, s.n)


def test_mixed_after_updates_and_in_a_cluster(gpu, oracle, geam, odata):
    # after update() (packed coordinates rewritten by the update kernel) and on a cluster with a frozen
    # shell in an open box
    s = W.fe_vacancy_cell(seed=9)
    g, o = _pair(gpu, oracle, geam, odata, s, odata.r_cut + 0.3)
    rng = np.random.default_rng(11)
    for _ in range(3):
        d = rng.normal(0, 0.01, s.pos.shape)
        g.update(d)
        o.update(d)
        e, grad = geam.energy_gradient(s.types, s.frozen, g, gpu.MIXED)
        _check_mixed(grad, oracle.eam_gradient(odata, o, s.types, s.frozen), e, oracle.eam_energy(odata, o, s.types), s.n)
    c = W.cluster(np.random.default_rng(4), 11.0, n_vac=2, n_h=2).sys
    g, o = _pair(gpu, oracle, geam, odata, c, odata.r_cut + 0.2)
    e, grad = geam.energy_gradient(c.types, c.frozen, g, gpu.MIXED)
    ref = oracle.eam_gradient(odata, o, c.types, c.frozen)
    assert np.all(grad[c.frozen == 1] == 0)
    _check_mixed(grad, ref, e, oracle.eam_energy(odata, o, c.types), c.n)


def _counting_table(path, rc=5.0):
    """A one-type eam/fs table with phi = 1, F(rho) = rho and v = 0 inside a 6 A grid and cut-off rc: the
    energy is then the number of ordered pairs within rc, so it shows every cut-off decision."""
    n_rho, d_rho, n_r, d_r = 5000, 0.01, 1000, 0.006

    def block(vals):
        return "\n".join(" ".join(f"{v:.17g}" for v in vals[k:k + 5]) for k in range(0, len(vals), 5))

    with open(path, "w") as f:
        f.write("counting table\n\n\n1 Fe\n")
        f.write(f"{n_rho} {d_rho} {n_r} {d_r} {rc}\n26 55.845 2.855 bcc\n")
        f.write(block([k * d_rho for k in range(n_rho)]) + "\n")
        f.write(block([1.0] * n_r) + "\n")
        f.write(block([0.0] * n_r) + "\n")
    return rc


def test_mixed_cutoff_decision_is_binary64(gpu, oracle, tmp_path):
    # Atoms placed within ~1e-13 A of r_cut of a centre atom, on either side: every pair must be in or
    # out exactly as the reference's binary64 (dx*dx + dy*dy) + dz*dz < rc*rc decides (list.hpp:139-154).
    # With the counting table the energy counts the pairs inside r_cut.
    path = str(tmp_path / "count.eam.fs")
    rc = _counting_table(path)
    eam, od = gpu.EAM(path), oracle.EAMData(path)
    rng = np.random.default_rng(21)
    centre = np.array([20.0, 20.0, 20.0])
    pos = [centre]
    for k in range(60):
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        pos.append(centre + rc * (1 + (k - 30) * 2.0 ** -48) * u)
    pos = np.array(pos)
    ext, per = [40.0, 40.0, 40.0], [0, 0, 0]
    types, frozen = np.zeros(len(pos), np.uint32), np.zeros(len(pos), np.uint8)
    g = gpu.List(ext, per, rc + 0.3)
    g.rebuild(pos)
    o = oracle.List(ext, per, rc + 0.3)
    o.rebuild(pos, 1)
    counts, _, _ = o.neighbours(rc)
    assert 0 < counts[0] < 60  # both outcomes occur among the near-r_cut pairs
    e_ref = oracle.eam_energy(od, o, types)
    assert abs(e_ref - counts.sum()) < 1e-6
    for prec in (gpu.MIXED, gpu.FP64):
        e, _ = eam.energy_gradient(types, frozen, g, prec)
        assert abs(e - e_ref) < 1e-6, (prec, e, e_ref)
    # after an update() that moves the shell by exact binary64 amounts the decisions still follow binary64
    d = np.zeros_like(pos)
    d[1:] = rng.normal(0, 1e-14, (len(pos) - 1, 3))
    g.update(d)
    o.update(d)
    e_ref = oracle.eam_energy(od, o, types)
    e, _ = eam.energy_gradient(types, frozen, g, gpu.MIXED)
    assert abs(e - e_ref) < 1e-6, (e, e_ref)


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
