"""Catalogue local environments (geometry + fingerprint, env/geometry.hpp:391-407, env/heuristics.hpp:93-110):
the oracle's restatement against the reference's own Fingerprint test case (a hypercube, tests/env/
heuristics.cpp:31-100), then the GPU (flygpu_env_*) bit for bit against the oracle."""
import numpy as np
import pytest

from openfly_gb300 import workloads as W


def _hypercube_env(oracle):
    # the 8 corners of a unit cube (tests/env/heuristics.cpp:31-48) in a large non-periodic box
    pos = np.array([[x, y, z] for z in (0.0, 1.0) for y in (0.0, 1.0) for x in (0.0, 1.0)]) + 4.0
    ext = np.full(3, 10.0)
    nl = oracle.List(ext, np.zeros(3, np.int32), 2.0)
    nl.rebuild(pos, 1)
    counts, idx, dr = nl.neighbours(2.0)
    return oracle.local_environment(counts, idx, dr, np.zeros(8, np.uint32), np.zeros(8, np.uint8), 0)


def test_oracle_fingerprint_of_the_hypercube(oracle):
    q, col, ind, r0, rij = _hypercube_env(oracle)
    assert np.array_equal(np.sort(ind), np.arange(8)) and ind[0] == 0
    assert np.allclose(q.mean(axis=0), 0.0, atol=1e-15)  # centred (Geometry::centre)
    s2, s3 = np.sqrt(2.0), np.sqrt(3.0)
    assert np.array_equal(r0, [1.0, 1.0, 1.0, s2, s2, s2, s3])
    assert np.array_equal(rij, [1.0] * 9 + [s2] * 9 + [s3] * 3)


def test_oracle_fingerprint_is_invariant(oracle):
    # Fingerprint equivalence under rotation and reordering (tests/env/heuristics.cpp:81-101), here with
    # the neighbours shuffled and the cube rotated about its centre.
    q, col, ind, r0, rij = _hypercube_env(oracle)
    rng = np.random.default_rng(1)
    a = rng.normal(size=(3, 3))
    rot, _ = np.linalg.qr(a)
    perm = np.concatenate([[0], 1 + rng.permutation(7)])
    dr = (q[perm] - q[0]) @ rot.T
    counts = np.array([7])
    q2, _, _, r02, rij2 = oracle.local_environment(counts, np.arange(1, 8), dr[1:], np.zeros(8, np.uint32),
                                                   np.zeros(8, np.uint8), 0)
    assert np.allclose(r02, r0, atol=1e-12)
    assert np.allclose(rij2, rij, atol=1e-12)


def _compare(gpu, oracle, s, r_env, update=None):
    from openfly_gb300 import env as E

    rc = r_env + 0.3
    g = gpu.List(s.extents, s.periodic, rc)
    o = oracle.List(s.extents, s.periodic, rc)
    g.rebuild(s.pos)
    o.rebuild(s.pos, 1)
    if update is not None:
        g.update(update)
        o.update(update)
    envs = E.local_environments(g, r_env, s.types, s.frozen)
    counts, idx, dr = o.neighbours(r_env)
    for i in range(s.n):
        q, col, ind, r0, rij = oracle.local_environment(counts, idx, dr, s.types, s.frozen, i)
        gq, gcol, gind = envs.geometry(i)
        gr0, grij = envs.fingerprint(i)
        assert np.array_equal(gq, q), i
        assert np.array_equal(gcol, col) and np.array_equal(gind, ind), i
        assert np.array_equal(gr0, r0) and np.array_equal(grij, rij), i


@pytest.mark.gpu
def test_gpu_environments_bit_exact(gpu, oracle, odata):
    # periodic cell with a vacancy, and a non-periodic cluster with a frozen shell and H (colours 0..3)
    _compare(gpu, oracle, W.fe_vacancy_cell(), odata.r_cut)
    cl = W.cluster(np.random.default_rng(8), 9.0, n_h=2, n_vac=1)
    _compare(gpu, oracle, cl.sys, 4.0)


@pytest.mark.gpu
def test_gpu_environments_after_update(gpu, oracle, odata):
    s = W.fe_vacancy_cell()
    d = np.random.default_rng(2).normal(0.0, 0.02, s.pos.shape)
    _compare(gpu, oracle, s, odata.r_cut, update=d)
