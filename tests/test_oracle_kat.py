"""The oracle against the reference's own known answers (CPU only)."""
import json
import os

import numpy as np
import pytest

from openfly_gb300 import workloads as W


def near(a, b, atol=1e-10, ftol=1e-4):
    """fly::near (utility/core.hpp:539-542)."""
    return abs(a - b) < atol or abs(a - b) <= ftol * max(abs(a), abs(b))


def test_eam_parse_kat(odata):
    # tests/potential/EAM/data.cpp:35-43
    assert odata.n_types == 2
    assert near(odata.spline(0, 0, 0, 0, 0.0), -0.1414216239132407e00)
    assert near(odata.spline(0, 0, 0, 0, 1.9999999999999999e-02), -0.2000010747904311e00)
    assert odata.r_cut == pytest.approx(5.3)


def test_eam_compute_kat(oracle, odata):
    # tests/potential/EAM/eam.cpp:99-125: 685-atom bcc Fe, site 1 erased.
    s = W.kat_lattice()
    nl = oracle.List(s.extents, s.periodic, odata.r_cut)
    nl.rebuild(s.pos, 1)
    e0 = oracle.eam_energy(odata, nl, s.types)
    assert near(e0, -2748.5339306065985)
    assert abs(e0 - -2748.5339306065985) < 1e-9
    g = oracle.eam_gradient(odata, nl, s.types, s.frozen)
    assert np.linalg.norm(g[0] - np.full(3, -0.19182439085483005)) < 1e-10


def test_eam_minimum_kat(oracle, odata):
    # tests/potential/EAM/eam.cpp:149-167: perfect lattice is force free.
    s = W.kat_lattice(erase=False)
    nl = oracle.List(s.extents, s.periodic, odata.r_cut)
    nl.rebuild(s.pos, 1)
    assert np.linalg.norm(oracle.eam_gradient(odata, nl, s.types, s.frozen)) < 1e-7


def test_threads_do_not_change_gradient(oracle, odata):
    s = W.fe_vacancy_cell()
    nl = oracle.List(s.extents, s.periodic, odata.r_cut)
    nl.rebuild(s.pos, 4)
    g1 = oracle.eam_gradient(odata, nl, s.types, s.frozen, threads=1)
    g4 = oracle.eam_gradient(odata, nl, s.types, s.frozen, threads=4)
    assert np.array_equal(g1, g4)


def _sorted_pairs(counts, idx, dr):
    out, o = [], 0
    for c in counts:
        p = np.argsort(idx[o:o + c], kind="stable")
        out.append((idx[o:o + c][p], dr[o:o + c][p]))
        o += c
    return out


def _random_box(rng, full_periodic=False):
    # Orthorhombic analogue of gen_rand (tests/neigh/list.cpp:128-165).
    ext = 1.0 + 9.0 * rng.random(3)
    per = np.ones(3, np.int32) if full_periodic else (rng.random(3) < 0.5).astype(np.int32)
    n = int(rng.integers(100, 1001))
    return ext, per, rng.random((n, 3)) * ext


@pytest.mark.parametrize("seed", [1334, 1111])
def test_list_fuzz_vs_brute_force(oracle, seed):
    # tests/neigh/list.cpp:167-208 (fewer boxes; same sizes and cut-off rule).
    rng = np.random.default_rng(seed)
    for _ in range(12):
        ext, per, pos = _random_box(rng)
        rc = ext.min() / 3
        nl = oracle.List(ext, per, rc)
        nl.rebuild(pos, 1)
        a = _sorted_pairs(*nl.neighbours(rc))
        b = _sorted_pairs(*oracle.brute_neighbours(ext, per, pos, rc))
        for (ia, da), (ib, db) in zip(a, b):
            assert np.array_equal(ia, ib)
            assert np.all(np.linalg.norm(da - db, axis=1) < 1e-10)


def test_list_update_vs_brute_force(oracle):
    # tests/neigh/list.cpp:210-250: list at rc + 2 skin, displacements 0.99 skin.
    rng = np.random.default_rng(1)
    for _ in range(5):
        ext, per, pos = _random_box(rng, full_periodic=True)
        rc, skin = ext.min() / 3, 0.1
        nl = oracle.List(ext, per, rc + 2 * skin)
        nl.rebuild(pos, 2)
        d = rng.random((pos.shape[0], 3))
        d = d / np.linalg.norm(d, axis=1, keepdims=True) * (skin * 0.99)
        nl.update(d)
        a = _sorted_pairs(*nl.neighbours(rc))
        b = _sorted_pairs(*oracle.brute_neighbours(ext, per, pos - d, rc))
        for (ia, da), (ib, db) in zip(a, b):
            assert np.array_equal(ia, ib)
            assert np.all(np.linalg.norm(da - db, axis=1) < 1e-9)


KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def test_golden_fixture_values(oracle, odata):
    # tests/golden/reference_kats.json holds the values tests/golden/make_golden.py read out of the
    # reference's test sources; the oracle reproduces each.
    for x, fx in KATS["f_Fe"]:
        assert near(odata.spline(0, 0, 0, 0, x), fx)
    s = W.kat_lattice()
    nl = oracle.List(s.extents, s.periodic, odata.r_cut)
    nl.rebuild(s.pos, 2)
    assert near(oracle.eam_energy(odata, nl, s.types, 2), KATS["E0"])
    g = oracle.eam_gradient(odata, nl, s.types, s.frozen, 2)
    assert np.linalg.norm(g[0] - KATS["grad0_component"]) < KATS["grad0_tol"]


def test_adjacent_cells_kat(oracle):
    # tests/neigh/adjacent.cpp:23-95
    a = KATS["adjacent_5cubed"]
    assert oracle.adjacent([5, 5, 5], a["interior_cell"]) == a["interior"]
    assert len(oracle.adjacent([5, 5, 5], a["face_cell"])) == a["face_count"]
    assert len(oracle.adjacent([5, 5, 5], a["edge_cell"])) == a["edge_count"]
    assert len(oracle.adjacent([5, 5, 5], a["corner_cell"])) == a["corner_count"]


def test_hypergrid_cell_idx_kat(oracle):
    # tests/system/boxes/hypergrid.cpp:24-44
    h = KATS["hypergrid_10_rc3"]
    for k, x in h["x"].items():
        assert oracle.cell_idx([10.0, 10.0, 10.0], 3.0, [x, x, x]) == h["idx"][k]


def test_ghost_capacity_and_spline_oob(oracle, odata):
    # Spline::OutOfBounds (spline.hpp:141-143) surfaces as a status.
    with pytest.raises(oracle.OracleError) as e:
        odata.spline(1, 0, 0, 0, 1e6)
    assert e.value.status == oracle.SPLINE_OOB
    with pytest.raises(oracle.OracleError):
        odata.spline(1, 0, 0, 0, -1.0)
