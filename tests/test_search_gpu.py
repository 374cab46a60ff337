"""Batched and plain GPU searches vs the oracle's Dimer::find_sp / LBFGS::minimise.

A dimer search can branch to a different saddle on rounding-level differences (reduction order,
binary32 pair terms), as the reference's own results do across compilers and thread counts. So the
bar is stated per saddle: when both runs converge to the same saddle (final positions within
SAME_SADDLE_A of each other), their energies agree within 1 meV (the barrier-height bar); at least
90 % of searches end with the same exit code, and at least 80 % of jointly converged ones at the same
saddle.
"""
import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu

E_TOL = 1e-3  # eV
SAME_SADDLE_A = 0.05  # max per-atom distance between two final configurations of one saddle


@pytest.fixture(scope="module")
def search_mod(gpu):
    from openfly_gb300 import search

    return search


@pytest.fixture(scope="module")
def clusters():
    return W.search_clusters(n=32, seed=11)


@pytest.fixture(scope="module")
def oracle_refs(oracle, odata, clusters, search_mod):
    _, oopt = c3_options(search_mod, oracle)
    return [run_oracle(oracle, odata, oopt, c) for c in clusters]


def c3_options(S, O):
    gpu_opt = S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000)
    orc_opt = O.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000)
    return gpu_opt, orc_opt


def oracle_energy(O, odata, s, pos):
    nl = O.List(s.extents, s.periodic, odata.r_cut)
    nl.rebuild(pos, 1)
    return O.eam_energy(odata, nl, s.types)


def run_oracle(O, odata, opt, cl):
    s = cl.sys
    r = O.dimer_find_sp(odata, opt, s.extents, s.periodic, s.pos, cl.axis, s.types, s.frozen)
    r["energy"] = oracle_energy(O, odata, s, r["x"])
    return r


# Measured on the 32 test clusters: the same exit code for 100 % (binary64) and 97 % (binary32 pairs) of
# searches, and every jointly converged pair on the same saddle; the bars leave room for one or two
# chaotic searches more.
def compare(results, refs, label, positions=None, min_same_exit=0.9, min_same_saddle=0.8):
    same_exit = sum(a["exit_code"] == b["exit"] for a, b in zip(results, refs))
    assert same_exit >= min_same_exit * len(refs), (label, [(a["exit_code"], b["exit"]) for a, b in zip(results, refs)])
    both = [k for k, (a, b) in enumerate(zip(results, refs)) if a["exit_code"] == 0 and b["exit"] == 0]
    assert both, label
    if positions is None:
        same = both
    else:
        same = [k for k in both if np.abs(positions[k] - refs[k]["x"]).max() < SAME_SADDLE_A]
    assert len(same) >= min_same_saddle * len(both), (label, len(same), len(both))
    errs = [abs(results[k]["energy"] - refs[k]["energy"]) for k in same]
    assert max(errs) < E_TOL, (label, errs)
    return errs


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_dimer_matches_oracle(gpu, oracle, odata, geam, search_mod, clusters, oracle_refs, precision):
    S, O = search_mod, oracle
    gopt, oopt = c3_options(S, O)
    prec = gpu.FP64 if precision == "fp64" else gpu.MIXED
    b = S.Batch(geam, [S.from_cluster(c) for c in clusters], precision=prec, dimer=gopt)
    b.run(S.Tuning(4, 128, 2))
    res, pos, ax = b.results()
    assert all(r["status"] == 0 for r in res), res
    compare(res, oracle_refs, precision, positions=pos)
    # the reported energy is the energy of the returned positions
    for r, p, c in zip(res, pos, clusters):
        assert abs(r["energy"] - oracle_energy(O, odata, c.sys, p)) < 1e-4


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_two_phase_run_matches_oracle(gpu, oracle, odata, geam, search_mod, clusters, oracle_refs, precision):
    # Every search stops after one translation step in the throughput shape and resumes, from its saved
    # state, in the wide shape; one-phase runs (steps 0) are the single persistent launch.
    S, O = search_mod, oracle
    gopt, oopt = c3_options(S, O)
    prec = gpu.FP64 if precision == "fp64" else gpu.MIXED
    for steps in (1, 0):
        b = S.Batch(geam, [S.from_cluster(c) for c in clusters], precision=prec, dimer=gopt)
        b.set_stragglers(steps, S.Tuning(1, 256, 1, 0))
        b.run(S.Tuning(4, 128, 2))
        res, pos, ax = b.results()
        assert all(r["status"] == 0 for r in res), res
        compare(res, oracle_refs, f"{precision} stragglers {steps}", positions=pos)


def test_same_alone_and_in_mix(gpu, geam, search_mod, clusters):
    S = search_mod
    gopt = S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3)
    t = S.Tuning(4, 128, 2)
    mix = S.Batch(geam, [S.from_cluster(c) for c in clusters], precision=gpu.MIXED, dimer=gopt)
    mix.run(t)
    res_mix, pos_mix, _ = mix.results()
    for k in (0, 5, len(clusters) - 1):
        alone = S.Batch(geam, [S.from_cluster(clusters[k])], precision=gpu.MIXED, dimer=gopt)
        alone.run(t)
        r, p, _ = alone.results()
        assert r[0]["exit_code"] == res_mix[k]["exit_code"]
        assert r[0]["energy"] == res_mix[k]["energy"]
        assert np.array_equal(p[0], pos_mix[k])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_register_capped_variant_is_the_same_search(gpu, geam, search_mod, clusters, precision):
    # The 128-register kernel differs from the default one only in register allocation.
    S = search_mod
    prec = gpu.FP64 if precision == "fp64" else gpu.MIXED
    b = S.Batch(geam, [S.from_cluster(c) for c in clusters[:12]], precision=prec,
                dimer=S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3))
    out = []
    for regs in (0, 128):
        b.reset()
        b.run(S.Tuning(2, 128, 4, regs))
        out.append(b.results())
    (r0, p0, _), (r1, p1, _) = out
    assert r0 == r1
    assert all(np.array_equal(a, c) for a, c in zip(p0, p1))


def test_batch_rerun_after_reset_is_identical(gpu, geam, search_mod, clusters):
    S = search_mod
    b = S.Batch(geam, [S.from_cluster(c) for c in clusters[:6]], precision=gpu.MIXED,
                dimer=S.DimerOptions.defaults(n=6, f2norm=1e-3))
    b.run(S.Tuning(2, 128, 2))
    r1, p1, _ = b.results()
    b.reset()
    b.run(S.Tuning(2, 128, 2))
    r2, p2, _ = b.results()
    assert r1 == r2
    assert all(np.array_equal(a, c) for a, c in zip(p1, p2))


def test_plain_path_matches_oracle(gpu, oracle, odata, geam, search_mod, clusters, oracle_refs):
    # The drop-in path runs the reference's host loop over the GPU potential: same exit, same step
    # and gradient-call counts as the oracle, and converged saddles within 1 meV.
    S, O = search_mod, oracle
    gopt, oopt = c3_options(S, O)
    refs = list(zip(clusters, oracle_refs))
    pick = [p for p in refs if p[1]["exit"] == 0][:3] + [p for p in refs if p[1]["exit"] != 0][:2]
    res = []
    for c, ref in pick:
        r, _, _ = S.search_plain(geam, S.from_cluster(c), gpu.FP64, dimer=gopt)
        assert (r["exit_code"], r["steps"], r["grad_calls"]) == (ref["exit"], ref["steps"], ref["grad_calls"])
        res.append(r)
    compare(res, [p[1] for p in pick], "plain")


def test_vacancy_cell_periodic_search(gpu, oracle, odata, geam, search_mod):
    # 431-atom periodic cell, vacancy neighbour perturbed as Master::perturb does, f2norm 1e-3.
    S, O = search_mod, oracle
    s = W.fe_vacancy_cell()
    pos, axis = W.perturb(s, s.meta["centre"], np.random.default_rng(4))
    gopt, oopt = c3_options(S, O)
    ref = O.dimer_find_sp(odata, oopt, s.extents, s.periodic, pos, axis, s.types, s.frozen)
    ref["energy"] = oracle_energy(O, odata, s, ref["x"])
    srch = S.Search(pos, s.types, s.frozen, s.extents, s.periodic, axis=axis)
    plain, _, _ = S.search_plain(geam, srch, gpu.FP64, dimer=gopt)
    b = S.Batch(geam, [srch], precision=gpu.FP64, dimer=gopt)
    b.run(S.Tuning(4, 256, 1))
    batched = b.results()[0][0]
    for r in (plain, batched):
        assert r["exit_code"] == ref["exit"]
        if ref["exit"] == 0:
            assert abs(r["energy"] - ref["energy"]) < E_TOL


def _check_pathway(O, odata, s, p, ref, tag):
    assert (p is None) == (ref is None), tag
    if p is None:
        return
    for key in ("rev", "sp", "fwd"):
        assert np.abs(p[key] - ref[key]).max() < SAME_SADDLE_A, (tag, key)
    for key, e in (("rev", p["E_rev"]), ("fwd", p["E_fwd"])):
        assert abs(e - oracle_energy(O, odata, s, ref[key])) < E_TOL, (tag, key)
    assert abs(p["E_sp"] - oracle_energy(O, odata, s, ref["sp"])) < 1e-6, tag
    assert p["barrier"] == p["E_sp"] - p["E_rev"]


def test_pathways_match_oracle(gpu, oracle, odata, geam, search_mod, clusters):
    # Master::do_adj_min (find.cpp:1014-1090) against the oracle's restatement: the two relaxations from
    # the nudged saddle, the rev/fwd assignment, the centre-of-mass drift correction and the centre
    # check (no pathway when the atom moving most is not the centre), on converged saddles.
    S, O = search_mod, oracle
    gopt, _ = c3_options(S, O)
    b = S.Batch(geam, [S.from_cluster(c) for c in clusters], precision=gpu.FP64, dimer=gopt)
    b.run(S.Tuning(4, 128, 2))
    res, pos, ax = b.results()
    ok = [k for k, r in enumerate(res) if r["exit_code"] == 0][:6]
    assert ok
    sads = [S.Search(pos[k], clusters[k].sys.types, clusters[k].sys.frozen, clusters[k].sys.extents,
                     clusters[k].sys.periodic, axis=ax[k]) for k in ok]
    starts = [clusters[k].sys.pos for k in ok]
    centres = [clusters[k].centre for k in ok]
    lopt = S.LBFGSOptions.defaults(f2norm=1e-4)
    olopt = O.LBFGSOptions.defaults(f2norm=1e-4)
    for cen in (None, centres):
        paths = S.pathways(geam, sads, starts, centres=cen, precision=gpu.FP64, lbfgs=lopt)
        for i, (k, p) in enumerate(zip(ok, paths)):
            s = clusters[k].sys
            ref = O.adj_min(odata, olopt, s.extents, s.periodic, s.types, s.frozen, pos[k], ax[k], s.pos,
                            None if cen is None else cen[i])
            _check_pathway(O, odata, s, p, ref, (k, cen is not None))


def test_pathway_of_a_fully_mobile_cell(gpu, oracle, odata, geam, search_mod):
    # No frozen atom: the relaxations freeze the atom furthest from the centre (find.cpp:1026-1034).
    S, O = search_mod, oracle
    s = W.fe_vacancy_cell()
    centre = s.meta["centre"]
    pos, axis = W.perturb(s, centre, np.random.default_rng(4))
    gopt, _ = c3_options(S, O)
    b = S.Batch(geam, [S.Search(pos, s.types, s.frozen, s.extents, s.periodic, axis=axis)], precision=gpu.FP64,
                dimer=gopt)
    b.run(S.Tuning(4, 256, 1))
    res, sp, ax = b.results()
    if res[0]["exit_code"] != 0:
        pytest.skip("the vacancy-cell search did not converge")
    sad = S.Search(sp[0], s.types, s.frozen, s.extents, s.periodic, axis=ax[0])
    lopt = S.LBFGSOptions.defaults(f2norm=1e-4)
    olopt = O.LBFGSOptions.defaults(f2norm=1e-4)
    p = S.pathways(geam, [sad], [s.pos], centres=[centre], precision=gpu.FP64, lbfgs=lopt)[0]
    ref = O.adj_min(odata, olopt, s.extents, s.periodic, s.types, s.frozen, sp[0], ax[0], s.pos, centre)
    assert S.furthest_atom(s.pos, s.extents, s.periodic, centre) == O.furthest_atom(s.pos, s.extents, s.periodic,
                                                                                    centre)
    _check_pathway(O, odata, s, p, ref, "vacancy_cell")


def test_minimise_matches_oracle(gpu, oracle, odata, geam, search_mod, clusters):
    S, O = search_mod, oracle
    lopt = S.LBFGSOptions.defaults(f2norm=1e-4)
    olopt = O.LBFGSOptions.defaults(f2norm=1e-4)
    subset = clusters[:6]
    b = S.Batch(geam, [S.from_cluster(c, mode=S.MINIMISE) for c in subset], precision=gpu.FP64, lbfgs=lopt)
    b.run(S.Tuning(4, 128, 2))
    res, pos, _ = b.results()
    for r, p, c in zip(res, pos, subset):
        s = c.sys
        failed, iters, x, g = O.lbfgs_minimise(odata, olopt, s.extents, s.periodic, s.pos, s.types, s.frozen)
        assert r["exit_code"] == int(failed)
        assert abs(r["energy"] - oracle_energy(O, odata, s, x)) < E_TOL
