"""Continuous batching: every served result equals the same search run alone, whatever else is in
flight, however many steps a tick takes and however tight the HBM budget is."""
import time

import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(gpu):
    from openfly_gb300 import search

    return search


@pytest.fixture(scope="module")
def requests():
    return [c for _, c in W.served_requests(n_env=3, seed=5, per_env=(6, 8))]


def alone(S, gpu, geam, cl, opt, tuning):
    b = S.Batch(geam, [S.from_cluster(cl)], precision=gpu.MIXED, dimer=opt)
    b.run(tuning)
    r, p, a = b.results()
    return r[0], p[0], a[0]


def serve_all(S, gpu, geam, reqs, opt, tuning, budget=1 << 30, steps=8, stagger_s=0.0):
    srv = S.Server(geam, precision=gpu.MIXED, hbm_budget_bytes=budget, max_active=64, steps_per_tick=steps,
                   tuning=tuning, dimer=opt)
    ids = []
    for c in reqs:
        ids.append(srv.submit(S.from_cluster(c)))
        if stagger_s:
            time.sleep(stagger_s)
    got = {}
    t0 = time.time()
    while len(got) < len(ids) and time.time() - t0 < 120:
        for r in srv.poll(64, wait_ms=50):
            got[r["id"]] = (r, *srv.take(r["id"]))
    stats = srv.stats()
    srv.close()
    assert len(got) == len(ids)
    return [got[i] for i in ids], stats


def test_served_equals_alone(gpu, geam, S, requests):
    opt = S.DimerOptions.defaults(f2norm=1e-3, n=6)
    t = S.Tuning(4, 128, 2)
    served, stats = serve_all(S, gpu, geam, requests, opt, t, stagger_s=0.002)
    assert stats["completed"] == len(requests)
    assert stats["ticks"] > 1
    for k in range(0, len(requests), 4):
        r0, p0, a0 = alone(S, gpu, geam, requests[k], opt, t)
        r, p, a = served[k]
        assert r["status"] == 0
        assert (r["exit_code"], r["steps"], r["energy"]) == (r0["exit_code"], r0["steps"], r0["energy"])
        assert np.array_equal(p, p0) and np.array_equal(a, a0)


def test_tick_length_and_budget_do_not_change_results(gpu, geam, S, requests):
    opt = S.DimerOptions.defaults(f2norm=1e-3, n=6)
    t = S.Tuning(2, 128, 2)
    sub = requests[:8]
    a, _ = serve_all(S, gpu, geam, sub, opt, t, steps=1)
    b, _ = serve_all(S, gpu, geam, sub, opt, t, steps=16)
    # a budget that admits only a couple of requests at a time
    one = max(S.Batch(geam, [S.from_cluster(c)], dimer=opt).device_bytes for c in sub)
    c, _ = serve_all(S, gpu, geam, sub, opt, t, budget=2 * one)
    for x, y, z in zip(a, b, c):
        assert x[0]["energy"] == y[0]["energy"] == z[0]["energy"]
        assert np.array_equal(x[1], y[1]) and np.array_equal(x[1], z[1])


def test_request_over_budget_is_rejected(gpu, geam, S, requests):
    # a 1 KiB budget is below any request's device footprint (its neighbour columns alone are larger)
    srv = S.Server(geam, hbm_budget_bytes=1 << 10, max_active=4)
    with pytest.raises(gpu.FlyGPUError) as e:
        srv.submit(S.from_cluster(requests[0]))
    assert e.value.status == gpu.OOM
    srv.close()


def test_submit_many_is_all_or_nothing(gpu, geam, S, requests):
    # flygpu_server_submit_many: results equal single submissions; a bad descriptor queues none of them
    opt = S.DimerOptions.defaults(f2norm=1e-3, n=6)
    t = S.Tuning(4, 128, 2)
    sub = requests[:6]
    single, _ = serve_all(S, gpu, geam, sub, opt, t)
    srv = S.Server(geam, precision=gpu.MIXED, hbm_budget_bytes=1 << 30, max_active=64, tuning=t, dimer=opt)
    bad = [S.from_cluster(c) for c in sub]
    bad[3].types = np.full(bad[3].n, 200, np.uint32)  # no such type in the potential
    with pytest.raises(gpu.FlyGPUError, match="request 3"):
        srv.submit_many(bad)
    st = srv.stats()
    assert st["pending"] == 0 and st["active"] == 0 and st["completed"] == 0
    ids = srv.submit_many([S.from_cluster(c) for c in sub])
    assert ids == sorted(ids) and len(set(ids)) == len(sub)
    got = {}
    t0 = time.time()
    while len(got) < len(ids) and time.time() - t0 < 120:
        for r in srv.poll(64, wait_ms=50):
            got[r["id"]] = (r, *srv.take(r["id"]))
    srv.close()
    assert len(got) == len(ids)
    for i, x in zip(ids, single):
        assert got[i][0]["energy"] == x[0]["energy"]
        assert np.array_equal(got[i][1], x[1])


def test_server_rejects_a_shape_that_cannot_launch(gpu, geam, S, requests):
    # 1024 threads with the compiler's register allocation do not fit an SM: rejected when the server is
    # created, before its graph is captured; the thread is not left inside a capture, so a server with a
    # valid shape works afterwards.
    opt = S.DimerOptions.defaults(f2norm=1e-3, n=6)
    with pytest.raises(gpu.FlyGPUError) as e:
        S.Server(geam, precision=gpu.MIXED, tuning=S.Tuning(8, 1024, 1, 0), dimer=opt)
    assert e.value.status == gpu.INVALID_ARG
    served, stats = serve_all(S, gpu, geam, requests[:2], opt, S.Tuning(4, 128, 2))
    assert stats["completed"] == 2
    assert all(r[0]["status"] == 0 for r in served)
