"""The oracle's EAM Hessian and eigenvalue restatements (eam.cpp:122-233, system/hessian.hpp:86-143),
pinned to the reference's known answers and to finite differences of the pinned gradient. CPU only."""
import json
import os

import numpy as np

from openfly_gb300 import workloads as W

# tests/potential/EAM/eam.cpp:131-141, the (0, 0) block of the erased 7x7x7 cell and its tolerance, as
# extracted from the reference's test source into the golden fixture (tests/golden/make_golden.py)
_KATS = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_kats.json")))
KAT_H00 = np.array(_KATS["hessian_block_00"])
KAT_H00_TOL = _KATS["hessian_block_tol"]


def near(a, b, atol=1e-10, ftol=1e-4):
    """utility/core.hpp:539-542."""
    return abs(a - b) < atol or abs(a - b) <= ftol * max(abs(a), abs(b))


def _hess(oracle, odata, s, rc=None):
    o = oracle.List(s.extents, s.periodic, odata.r_cut if rc is None else rc)
    o.rebuild(s.pos, 1)
    return o, oracle.eam_hessian(odata, o, s.types, s.frozen, threads=4)


def test_kat_block_away_from_minimum(oracle, odata):
    # tests/potential/EAM/eam.cpp:98-146
    _, h = _hess(oracle, odata, W.kat_lattice())
    assert np.linalg.norm(h[:3, :3] - KAT_H00) < KAT_H00_TOL


def test_kat_zero_modes_at_minimum(oracle, odata):
    # tests/potential/EAM/eam.cpp:148-188: the perfect cell has exactly the 3 translational zero modes
    s = W.kat_lattice(erase=False)
    o, h = _hess(oracle, odata, s)
    assert np.linalg.norm(oracle.eam_gradient(odata, o, s.types, s.frozen)) < 1e-7
    ev = oracle.hessian_eigenvalues(h)
    assert all(near(e, 0.0) for e in ev[:3])
    assert not any(near(e, 0.0) for e in ev[3:])


def test_hessian_class_cases(oracle):
    # tests/system/hessian.cpp:22-49
    assert all(near(e, 0.0) for e in oracle.hessian_eigenvalues(np.zeros((6, 6))))
    one = np.ones((3, 3))
    assert near(oracle.hessian_eigenvalues(one).sum(), 3.0)


def test_lower_blocks_only_and_frozen_zero(oracle, odata):
    c = W.cluster(np.random.default_rng(11), 7.5, n_vac=1, n_h=1)
    s = c.sys
    _, h = _hess(oracle, odata, s)
    n = s.n
    blocks = h.reshape(n, 3, n, 3)
    iu = np.triu_indices(n, 1)
    assert not blocks[iu[0], :, iu[1], :].any()  # strictly upper blocks untouched
    fz = s.frozen == 1
    assert not blocks[fz].any() and not blocks[:, :, fz].any()


def test_matches_finite_differences_of_the_gradient(oracle, odata):
    # Two species, a vacancy and a frozen shell; central differences of the oracle gradient (itself
    # pinned to eam.cpp's known answers) against the symmetrised lower-block Hessian.
    c = W.cluster(np.random.default_rng(4), 8.0, shell=4.0, n_vac=1, n_h=2)
    s = c.sys
    _, h = _hess(oracle, odata, s)
    full = np.tril(h) + np.tril(h, -1).T
    mobile = np.flatnonzero(s.frozen == 0)
    step = 1e-5
    rng = np.random.default_rng(0)
    for a in rng.choice(mobile, 4, replace=False):
        for k in range(3):
            col = []
            for sign in (1.0, -1.0):
                p = s.pos.copy()
                p[a, k] += sign * step
                o = oracle.List(s.extents, s.periodic, odata.r_cut)
                o.rebuild(p, 1)
                col.append(oracle.eam_gradient(odata, o, s.types, s.frozen).ravel())
            fd = (col[0] - col[1]) / (2 * step)
            ref = full[:, 3 * a + k]
            assert np.linalg.norm(fd - ref) <= 1e-6 * np.linalg.norm(ref)


def test_mass_weight_scales_blocks(oracle):
    rng = np.random.default_rng(2)
    h = rng.normal(size=(6, 6))
    w = oracle.mass_weight(h, [4.0, 9.0])
    assert np.allclose(w[:3, :3], h[:3, :3] / 4.0)
    assert np.allclose(w[3:, :3], h[3:, :3] / 6.0)
    assert np.allclose(w[3:, 3:], h[3:, 3:] / 9.0)
