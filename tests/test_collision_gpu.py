"""Dimer::find_sp's history check (dimer.cpp:102-131) on the batch, the server and the plain path vs the
oracle. A search that climbs back towards a saddle already found from the same minimum stops with
Dimer::collision at a history-check step once cos(theta) between x - in_min and sp - in_min exceeds
cos(theta_tol), theta_tol as Master::find_batch sets it (find.cpp:692).

The device search keeps its vectors over mobile atoms only; the static atoms' shares of the check's
dots are constants of the search, added on the device, so the check is the reference's 3n one also when
a history saddle's frozen atoms (or the start's) differ from in_min. Cases below cover both.
"""
import time

import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu

COLLISION = -3


def theta_tol(tot: int) -> float:
    """Master::find_batch's collision angle after `tot` searches (find.cpp:692)."""
    return ((30 - 2.5) * np.exp(-0.02 * tot) + 2.5) / 360.0 * 2.0 * np.pi


@pytest.fixture(scope="module")
def S(gpu):
    from openfly_gb300 import search

    return search


def _opts(S, O):
    return (S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000),
            O.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000))


@pytest.fixture(scope="module")
def cases(oracle, odata):
    """(cluster, in_min, start, hist, oracle result) per case: a first oracle search gives a saddle; a
    second start (extra noise on the mobile atoms, same axis) gets it as history. Variants shift the
    history saddle's frozen atoms, or the start's static atoms, away from in_min."""
    O = oracle
    oopt = O.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000)
    rng = np.random.default_rng(3)
    out = []
    for c in W.search_clusters(n=40, seed=31):
        s = c.sys
        r1 = O.dimer_find_sp(odata, oopt, s.extents, s.periodic, s.pos, c.axis, s.types, s.frozen)
        if r1["exit"] != 0:
            continue
        mob, fz = s.frozen == 0, s.frozen == 1
        start = s.pos.copy()
        start[mob] += rng.normal(0, 0.02, (int(mob.sum()), 3))
        variants = [(start, r1["x"])]
        sp_f = r1["x"].copy()
        sp_f[fz] += rng.normal(0, 0.03, (int(fz.sum()), 3))  # history saddle's frozen atoms off in_min
        variants.append((start, sp_f))
        st_f = start.copy()
        st_f[fz] += rng.normal(0, 0.01, (int(fz.sum()), 3))  # the start's static atoms off in_min
        variants.append((st_f, r1["x"]))
        for st, sp in variants:
            r = O.dimer_find_sp(odata, oopt, s.extents, s.periodic, st, c.axis, s.types, s.frozen, in_min=s.pos,
                                hist=[sp], theta_tol=theta_tol(0))
            out.append((c, s.pos, st, [sp], r))
        if len(out) >= 18:
            break
    assert any(r["exit"] == COLLISION for *_, r in out)
    assert any(r["exit"] != COLLISION for *_, r in out)
    return out


def _search(S, c, in_min, start, hist):
    s = c.sys
    return S.Search(start, s.types, s.frozen, s.extents, s.periodic, axis=c.axis, in_min=in_min, hist=hist,
                    theta_tol=theta_tol(0))


def test_plain_path_collision_exit_matches_oracle_exactly(gpu, oracle, geam, S, cases):
    # the reference's host loop over the GPU potential: same exit and step count as the oracle
    gopt, _ = _opts(S, oracle)
    for c, im, st, hist, ref in cases:
        r, _, _ = S.search_plain(geam, _search(S, c, im, st, hist), gpu.FP64, dimer=gopt)
        assert (r["exit_code"], r["steps"]) == (ref["exit"], ref["steps"]), (r, ref["exit"], ref["steps"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_collision_exit_matches_oracle(gpu, oracle, geam, S, cases, precision):
    gopt, _ = _opts(S, oracle)
    prec = gpu.FP64 if precision == "fp64" else gpu.MIXED
    b = S.Batch(geam, [_search(S, c, im, st, h) for c, im, st, h, _ in cases], precision=prec, dimer=gopt)
    b.run(S.Tuning(4, 128, 2))
    res, _, _ = b.results(positions=False)
    assert all(r["status"] == 0 for r in res)
    refs = [ref for *_, ref in cases]
    same_exit = [r["exit_code"] == ref["exit"] for r, ref in zip(res, refs)]
    assert sum(same_exit) >= len(refs) - 1, [(r["exit_code"], ref["exit"]) for r, ref in zip(res, refs)]
    # a collision is detected at the same history-check step as the oracle's
    coll = [(r["steps"], ref["steps"]) for r, ref in zip(res, refs) if r["exit_code"] == ref["exit"] == COLLISION]
    assert coll
    assert sum(a == b_ for a, b_ in coll) >= 0.8 * len(coll), coll


def test_served_collision_exit_equals_batched(gpu, oracle, geam, S, cases):
    gopt, _ = _opts(S, oracle)
    t = S.Tuning(4, 128, 2)
    searches = [_search(S, c, im, st, h) for c, im, st, h, _ in cases]
    b = S.Batch(geam, searches, precision=gpu.MIXED, dimer=gopt)
    b.run(t)
    res, _, _ = b.results(positions=False)
    srv = S.Server(geam, precision=gpu.MIXED, hbm_budget_bytes=1 << 30, max_active=64, steps_per_tick=4, tuning=t,
                   dimer=gopt)
    ids = [srv.submit(x) for x in searches]
    got = {}
    t0 = time.time()
    while len(got) < len(ids) and time.time() - t0 < 120:
        for r in srv.poll(64, wait_ms=50):
            got[r["id"]] = r
    srv.close()
    assert len(got) == len(ids)
    for i, r in zip(ids, res):
        assert (got[i]["exit_code"], got[i]["steps"]) == (r["exit_code"], r["steps"])
        assert got[i]["energy"] == r["energy"]
