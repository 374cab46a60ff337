#!/usr/bin/env python
"""Throughput of the openFLY saddle-search inner loop on GB300.

Workload (one "step"): on 80^3 bcc Fe (1,024,000 sites, 0.1 % vacancies, 0.05 % H on tetrahedral
sites, sigma = 0.05 A noise; 1,023,487 atoms), a neighbour-list update with a 0.3 A skin followed by
one EAM energy + gradient evaluation (binary32 pair terms, binary64 accumulation). Each step applies a
resident displacement field of at most 0.005 A per atom (alternating +D_j, -D_j); the list is rebuilt
whenever the accumulated maximum displacement exceeds skin / 2 (the reference's rule,
src/minimise/LBFGS/lbfgs.cpp:96-101), and those rebuilds are inside the timed region.

value: atom-evals/s with inputs resident in HBM (device-timed with CUDA events on the library's
stream). e2e: the same steps through the host C ABI (flygpu_list_update / flygpu_eam_energy_gradient
with pinned host buffers: H2D of the displacement, D2H of gradient and energy every step).

--impl reference times the reference's CPU path for the same workload: the oracle port (the reference
cannot be compiled here: Eigen, fmt and its other dependencies are absent) with every host thread.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SKIN = 0.3
SAME_SADDLE_A = 0.05  # per-atom distance under which two final configurations are one saddle
STEP_DISP = 0.005  # max per-atom displacement per step (A)
N_FIELDS = 4
ALGO_BYTES_DENSITY = 36  # per atom: 24 B position + 4 B type read, 8 B F' write
ALGO_BYTES_FORCE = 60    # per atom: 24 B position + 4 B type + 8 B F' read, 24 B gradient write
ALGO_BYTES_STEP = 168    # per atom and step: 96 B EAM (both passes) + 72 B list update


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def make_workload(cells: int):
    from openfly_gb300 import workloads as W

    s = W.fe_h_crystal(n_cells=cells)
    rng = np.random.default_rng(99)
    fields = []
    for _ in range(N_FIELDS):
        d = rng.normal(0.0, 1.0, s.pos.shape)
        d *= STEP_DISP / np.linalg.norm(d, axis=1).max()
        fields.append(d)
    return s, fields


# Accumulated displacement at the start of a timed window: the window's 16th step triggers the first
# rebuild and every 31st after it, so any window of 16 or more steps holds at least its share of rebuilds.
ACC_TIMED = 0.5 * SKIN - 15 * STEP_DISP


def schedule(steps: int, acc0: float = 0.0):
    """(field index, sign, rebuild-after-update?) per step, with the reference's skin rule, starting from an
    accumulated displacement acc0."""
    acc, out = acc0, []
    for k in range(steps):
        j, sign = (k // 2) % N_FIELDS, (1.0 if k % 2 == 0 else -1.0)
        acc += STEP_DISP
        rebuild = acc > 0.5 * SKIN
        if rebuild:
            acc = 0.0
        out.append((j, sign, rebuild))
    return out


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self, t0: float, t1: float) -> dict | None:
        """Summary of the samples whose timestamps fall in the timed region [t0, t1] (host time.time())."""
        if self.p is None:
            return None
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        import datetime

        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                ts = datetime.datetime.strptime(r[0].strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
                if not t0 <= ts <= t1:
                    continue
                sm.append(float(r[2]))
                mx = max(mx, float(r[3]))
                for name, v in zip(names, r[6:10]):
                    if v.strip() == "Active":
                        reasons.add(name)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def reduce_max(x: float, device=None) -> float:
    """Maximum of x over the ranks of the default process group (x itself without one)."""
    import torch
    import torch.distributed as tdist

    if not (tdist.is_available() and tdist.is_initialized()):
        return float(x)
    t = torch.tensor([x], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: int, world: int, steps: int, max_ms: float) -> float:
    """Whole-job throughput of `world` independent replicas: every rank's units over the slowest rank's
    time (weak scaling, no data-path collective)."""
    return units_per_rank * world * steps / (max_ms * 1e-3)


def measured_peak_hbm() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_from_profile(kernel: str, atoms: int) -> float | None:
    """DRAM bytes (read + write) of one launch of `kernel` at `atoms` atoms, from the committed ncu
    capture of a smaller Fe-H crystal (profiles/fe_h_crystal_dram_traffic.json), scaled by atom count: the
    traffic of a pass grows in proportion to the atoms it processes."""
    p = os.path.join(ROOT, "profiles", "fe_h_crystal_dram_traffic.json")
    if os.path.exists(p):
        k = json.load(open(p)).get(kernel)
        if k:
            return k["bytes_per_atom"] * atoms
    return None


# ----------------------------------------------------------------------------- CPU (oracle) leg

def cpu_crystal_steps(s, fields, steps: int, threads: int, acc0: float = ACC_TIMED):
    """The reference's CPU path (oracle port) on the same steps; returns (seconds, steps, rebuilds)."""
    from oracle import pyoracle as O
    from openfly_gb300 import workloads as W

    data = O.EAMData(W.TABLE)
    nl = O.List(s.extents, s.periodic, data.r_cut + SKIN)
    nl.rebuild(s.pos, threads)
    sched = schedule(steps, acc0)
    pos_alt = [s.pos - f for f in fields]
    t0 = time.perf_counter()
    rebuilds = 0
    for j, sign, rb in sched:
        if rb:
            nl.rebuild(pos_alt[j] if sign > 0 else s.pos, threads)
            rebuilds += 1
        else:
            nl.update(sign * fields[j])
        O.eam_energy(data, nl, s.types, threads)
        O.eam_gradient(data, nl, s.types, s.frozen, threads)
    return time.perf_counter() - t0, len(sched), rebuilds


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    s, fields = make_workload(args.cells)
    from oracle import pyoracle as O

    O.build()
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    # warm-up then K timed steps, each a full step of the workload on every host thread
    cpu_crystal_steps(s, fields, max(1, args.warmup), threads)
    secs, k, rb = cpu_crystal_steps(s, fields, args.steps, threads)
    value = s.n * k / secs
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "atom-evals/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / k, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(s, args, reference=True),
        "cpu_baseline": {"value": value, "unit": "atom-evals/s", "cores": threads, "kind": "port",
                         "sample": f"{k} full steps ({rb} rebuilds) of the {s.n}-atom workload"},
        "e2e": {"value": value, "unit": "atom-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


METRIC = "saddle searches/s + p50/p99 latency vs one-at-a-time GPU @<=1 meV; atom-evals/s"


def config_dict(s, args, reference: bool = False):
    c = {"workload": f"{args.cells}^3 bcc Fe, 0.1% vacancies, 0.05% H, sigma 0.05 A; per step "
                     f"List::update (skin {SKIN} A, rebuild by the reference's skin rule) + EAM energy+gradient",
         "atoms": s.n, "cells": args.cells}
    if reference:
        c.update({"precision": "binary64 (the reference's arithmetic, oracle port)",
                  "parallelism": "host threads of rank 0"})
    else:
        c.update({"precision": "binary32 pairs / binary64 accumulation",
                  "l2": "inputs larger than L2 (positions, packed slots, neighbour columns ~0.4 GB)",
                  "parallelism": f"replicas x{args.gpus}"})
    return c


# ----------------------------------------------------------------------------- search metrics

def serve_run(S, eam, stream, tune, opt, args, rate) -> dict:
    """The served stream through flygpu_server: submit `stream` with Poisson arrivals at `rate` per second (all at
    once when rate is None) and poll completions on another thread; searches/s over the wall time from
    the first submission to the last completion, latency from submission to completion."""
    import threading

    srv = S.Server(eam, hbm_budget_bytes=40 << 30, max_active=2048, steps_per_tick=args.steps_per_tick,
                   tuning=tune, dimer=opt)
    rng = np.random.default_rng(1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(stream))) if rate else np.zeros(len(stream))
    done: list = []
    stop = threading.Event()

    def poller():
        while len(done) < len(stream) and not (stop.is_set() and len(done) >= len(stream)):
            done.extend(srv.poll(512, wait_ms=20))
            if stop.is_set() and srv.stats()["pending"] == 0 and srv.stats()["active"] == 0 and len(done) >= len(stream):
                break

    th = threading.Thread(target=poller)
    th.start()
    t0 = time.perf_counter()
    for k, r in enumerate(stream):
        while time.perf_counter() - t0 < arrivals[k]:
            pass
        srv.submit(r)
    stop.set()
    th.join(timeout=600)
    elapsed = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat = np.array([d["latency_ms"] for d in done])
    ex = [d["exit_code"] for d in done]
    return {"requests": len(stream), "completed": len(done), "arrival_rate_per_s": rate if rate else "all at once",
            "searches_per_s": len(done) / elapsed, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "steps_per_tick": args.steps_per_tick, "ticks": st["ticks"],
            "converged": ex.count(0), "hbm_budget_bytes": 40 << 30}


def search_metrics(fly, args) -> dict:
    """Configs 3 and 4: batched searches/s (one persistent launch over 4096 clusters), the plain
    one-search-at-a-time drop-in GPU path on a sample, binary32-pair vs binary64 saddle energies, and
    the served path's searches/s with p50/p99 latency under Poisson arrivals."""

    import torch

    from openfly_gb300 import search as S
    from openfly_gb300 import workloads as W

    eam = fly.EAM(W.TABLE)
    opt = S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000)
    clusters = W.search_clusters(n=args.searches, seed=7)
    reqs = [S.from_cluster(c) for c in clusters]
    out = {"batched": {"searches": len(reqs), "mean_atoms": float(np.mean([r.n for r in reqs])),
                       "options": "m=6 (translation and rotation), |F| < 1e-3 eV/A, <= 1000 steps"}}
    l0 = fly.launch_count()
    runs, pos_final = {}, {}
    for prec, name in ((fly.MIXED, "mixed"), (fly.FP64, "fp64")):
        b = S.Batch(eam, reqs, precision=prec, dimer=opt)
        tune = b.autotune()
        best = None
        for _ in range(2):
            b.reset()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            t0 = time.perf_counter()
            b.run(tune)
            res, _, _ = b.results(positions=False)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        runs[name] = res
        pos_final[name] = b.results(positions=True)[1]  # untimed: final configurations for the same-saddle test
        del b
        # end to end: the batch built from the host descriptions (packing and upload), run and read back
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b2 = S.Batch(eam, reqs, precision=prec, dimer=opt)
        b2.run(tune)
        res2, _, _ = b2.results(positions=True)
        e2e_s = time.perf_counter() - t0
        del b2
        ex = [r["exit_code"] for r in res]
        out["batched"][name] = {"searches_per_s": len(reqs) / best, "seconds": best, "tuning": tune.as_dict(),
                                "converged": ex.count(0), "convex": ex.count(-1), "iter_max": ex.count(-2),
                                "saddles_per_s": ex.count(0) / best,
                                "e2e": {"searches_per_s": len(reqs) / e2e_s, "seconds": e2e_s,
                                        "saddles_per_s": sum(r["exit_code"] == 0 for r in res2) / e2e_s,
                                        "note": "flygpu_batch_create (host packing + upload) + run + results with "
                                                "final positions and axes, timed together"},
                                "errors": sum(r["status"] != 0 for r in res),
                                "grad_calls_mean": float(np.mean([r["grad_calls"] for r in res]))}
    # Both precisions converged and ended on the same saddle (every atom within SAME_SADDLE_A): the
    # barrier-height error is measured there; a pair that took different saddles is counted, not measured.
    conv = [k for k, (a, b_) in enumerate(zip(runs["mixed"], runs["fp64"]))
            if a["exit_code"] == 0 and b_["exit_code"] == 0]
    same = [k for k in conv if np.abs(pos_final["mixed"][k] - pos_final["fp64"][k]).max() < SAME_SADDLE_A]
    err = np.abs(np.array([runs["mixed"][k]["energy"] - runs["fp64"][k]["energy"] for k in same])) * 1e3
    out["batched"]["saddle_energy_err_mixed_vs_fp64_meV"] = {
        "n": int(err.size), "both_converged": len(conv), "same_saddle_A": SAME_SADDLE_A,
        "max": float(err.max()) if err.size else None,
        "p99": float(np.percentile(err, 99)) if err.size else None,
        "within_1meV_fraction": float(np.mean(err < 1.0)) if err.size else None,
        "same_exit_fraction": float(np.mean([a["exit_code"] == b_["exit_code"]
                                             for a, b_ in zip(runs["mixed"], runs["fp64"])]))}
    # plain drop-in path, one search at a time, on an evenly spread sample
    sample = reqs[:: max(1, len(reqs) // args.plain_sample)][: args.plain_sample]
    lat = []
    t0 = time.perf_counter()
    for r in sample:
        t1 = time.perf_counter()
        S.search_plain(eam, r, fly.MIXED, dimer=opt)
        lat.append(1e3 * (time.perf_counter() - t1))
    plain = len(sample) / (time.perf_counter() - t0)
    out["batched"]["plain_one_at_a_time"] = {"searches_per_s": plain, "sample": len(sample),
                                             "p50_ms": float(np.percentile(lat, 50)),
                                             "p99_ms": float(np.percentile(lat, 99))}
    out["batched"]["batched_over_plain"] = out["batched"]["mixed"]["searches_per_s"] / plain
    # served stream: Poisson arrivals at --arrival-rate, then every request at once (capacity)
    stream = [S.from_cluster(c) for _, c in W.served_requests()]
    # served in a latency shape: the batch's lanes per atom, 512 threads at one CTA per SM with the
    # 128-register variant (a served request waits on its own chain, not on the batch's tail; at this
    # arrival rate a few dozen requests are in flight, so SMs are not the scarce resource)
    t3 = out["batched"]["mixed"]["tuning"]
    tune = S.Tuning(t3["lanes_per_atom"], 512, 1, 128)
    out["served"] = serve_run(S, eam, stream, tune, opt, args, args.arrival_rate)
    out["served"]["tuning"] = tune.as_dict()
    out["served"]["plain_service_p50_ms"] = out["batched"]["plain_one_at_a_time"]["p50_ms"]
    out["served"]["plain_service_p99_ms"] = out["batched"]["plain_one_at_a_time"]["p99_ms"]
    out["served"]["saturated"] = serve_run(S, eam, stream, tune, opt, args, None)
    out["mechanisms"] = mechanism_metrics(fly, eam, S, W)
    out["gpu_launches"] = int(fly.launch_count() - l0)
    # kept for the CPU leg's comparison with the oracle (not printed)
    out["_oracle_sample"] = (clusters[:ORACLE_SAMPLE], {k: v[:ORACLE_SAMPLE] for k, v in runs.items()},
                             {k: v[:ORACLE_SAMPLE] for k, v in pos_final.items()})
    return out


ORACLE_SAMPLE = 96  # batched searches also run by the oracle in the CPU leg


def oracle_search_agreement(sample, threads: int) -> dict:
    """The first ORACLE_SAMPLE batched searches against the oracle's Dimer::find_sp on the same inputs:
    the fraction with the reference's exit code, the fraction of jointly converged pairs on the same saddle
    (every atom within SAME_SADDLE_A) and their saddle-energy differences, per precision."""
    from oracle import pyoracle as O
    from openfly_gb300 import workloads as W

    clusters, runs, pos = sample
    od = O.EAMData(W.TABLE)
    oopt = O.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000)
    sys_ = [c.sys for c in clusters]
    offs = np.concatenate([[0], np.cumsum([x.n for x in sys_])]).astype(np.int64)
    t0 = time.perf_counter()
    ex, st, x, _ = O.dimer_batch(od, oopt, offs, np.stack([x.extents for x in sys_]), np.stack([x.periodic for x in sys_]),
                                 np.concatenate([x.pos for x in sys_]), np.concatenate([c.axis for c in clusters]),
                                 np.concatenate([x.types for x in sys_]), np.concatenate([x.frozen for x in sys_]),
                                 np.array([int(x.frozen.sum()) for x in sys_], np.int32), threads)
    secs = time.perf_counter() - t0
    out = {"searches": len(clusters), "oracle_seconds": secs, "oracle_threads": threads, "same_saddle_A": SAME_SADDLE_A}
    for name in runs:
        same_exit = [int(r["exit_code"]) == int(e) for r, e in zip(runs[name], ex)]
        both = [k for k, (r, e) in enumerate(zip(runs[name], ex)) if r["exit_code"] == 0 and e == 0]
        same = []
        for k in both:
            xo = x[offs[k]:offs[k + 1]]
            if np.abs(pos[name][k] - xo).max() < SAME_SADDLE_A:
                same.append(k)
        errs = []
        for k in same:
            s = sys_[k]
            nl = O.List(s.extents, s.periodic, od.r_cut)
            nl.rebuild(x[offs[k]:offs[k + 1]], 1)
            errs.append(abs(runs[name][k]["energy"] - O.eam_energy(od, nl, s.types)) * 1e3)
        out[name] = {"same_exit_fraction": float(np.mean(same_exit)), "both_converged": len(both),
                     "same_saddle_fraction": len(same) / len(both) if both else None,
                     "saddle_energy_err_meV_max": float(max(errs)) if errs else None}
    return out


def mechanism_metrics(fly, eam, S, W, n: int = 256) -> dict:
    """Master's post-search pipeline on n search clusters, as Master runs it: each cluster relaxed to its
    minimum, perturbed around its centre (Master::perturb) and climbed to a saddle (binary32 pairs, one
    batched launch each); then search.mechanisms (saddle_2_mech: do_adj_min, the checks, energies,
    prefactors and recon_relax, all relaxations batched) on the converged saddles, timed on its own.
    Each saddle's geometry is centred on the atom that moves most in its pathway."""
    clusters = W.search_clusters(n=n, seed=19)
    lb = S.LBFGSOptions.defaults(f2norm=1e-6)
    relax = S.Batch(eam, [S.from_cluster(c, mode=S.MINIMISE) for c in clusters], precision=fly.MIXED, lbfgs=lb)
    relax.run()
    _, minima, _ = relax.results()
    rng = np.random.default_rng(5)
    starts = []
    for c, x in zip(clusters, minima):
        s = c.sys
        p, a = W.perturb(W.System(x, s.types, s.frozen, s.extents, s.periodic), c.centre, rng)
        starts.append(S.Search(p, s.types, s.frozen, s.extents, s.periodic, axis=a, in_min=x))
    opt = S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000)
    b = S.Batch(eam, starts, precision=fly.MIXED, dimer=opt)
    b.run()
    res, pos, ax = b.results()
    found = [(c, x, S.Search(xs, c.sys.types, c.sys.frozen, c.sys.extents, c.sys.periodic, axis=a))
             for c, x, r, xs, a in zip(clusters, minima, res, pos, ax) if r["status"] == 0 and r["exit_code"] == 0]
    paths = S.pathways(eam, [s for *_, s in found], [x for _, x, _ in found], None, precision=fly.MIXED, lbfgs=lb)
    sel, geos = [], []
    for (c, x, s), p in zip(found, paths):
        if p is not None:
            mm = int(np.argmax(((p["rev"] - p["fwd"]) ** 2).sum(axis=1)))
            d = np.linalg.norm(x - x[mm], axis=1)
            geos.append(np.concatenate([[mm], np.flatnonzero((d < 4.0) & (np.arange(c.sys.n) != mm))]))
            sel.append((c, x, s))
    t0 = time.perf_counter()
    try:
        mech = S.mechanisms(eam, [s for *_, s in sel], [x for _, x, _ in sel], geos, precision=fly.MIXED, dimer=opt,
                            lbfgs=lb)
        err = None
    except RuntimeError as e:  # a verify() of the reference (kept as the reference raises it)
        mech, err = [], str(e)
    dt = time.perf_counter() - t0
    built = [m for m in mech if m is not None]
    return {"clusters": n, "saddles": len(sel), "mechanisms": len(built), "seconds": dt,
            "saddles_per_s": len(sel) / dt if dt > 0 else None,
            "poisoned": sum(1 for m in built if m["poison_sp"] or m["poison_fwd"]), "raised": err,
            "note": "search.mechanisms: saddle_2_mech for every saddle; relaxations, Hessians and recon batched"}


# ----------------------------------------------------------------------------- GPU leg

def ours(args):
    import torch

    import openfly_gb300 as fly
    from openfly_gb300 import workloads as W
    from openfly_gb300.build import build

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch.distributed as tdist

        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if rank == 0 or not dist:
        build()
    if dist:
        tdist.barrier()
    dev = torch.device("cuda", local)
    # A stream of our own: the list launches every kernel on it and the timing events are recorded on it
    # (handle 0 would make the library create a private non-blocking stream the events do not see).
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)

    s, fields = make_workload(args.cells)
    n = s.n
    eam = fly.EAM(W.TABLE)
    nl = fly.List(s.extents, s.periodic, eam.r_cut() + SKIN, stream=stream.cuda_stream)
    d_fields = [torch.from_numpy(f.reshape(-1)).to(dev) for f in fields]
    d_neg = [-f for f in d_fields]
    d_pos0 = torch.from_numpy(s.pos.reshape(-1)).to(dev)
    d_pos_alt = [d_pos0 - f for f in d_fields]
    d_types = torch.from_numpy(s.types.astype(np.int32)).to(dev)
    d_frozen = torch.from_numpy(s.frozen).to(dev)
    d_grad = torch.empty(3 * n, dtype=torch.float64, device=dev)
    d_e = torch.empty(1, dtype=torch.float64, device=dev)
    nl.rebuild_device(d_pos0, n)
    eam.energy_gradient_device(nl, d_e, d_grad, d_types=d_types, d_frozen=d_frozen, precision=fly.MIXED)
    nl.sync()
    # untimed: both precisions' gradients and energies at the workload's positions, for the parity
    # block the CPU leg fills in against the oracle's binary64 gradient on the same positions
    par = {"mixed": (float(d_e.item()), d_grad.cpu().numpy().reshape(-1, 3))}
    eam.energy_gradient_device(nl, d_e, d_grad, precision=fly.FP64)
    nl.sync()
    par["fp64"] = (float(d_e.item()), d_grad.cpu().numpy().reshape(-1, 3))

    def step(j, sign, rb):
        if rb:
            nl.rebuild_device(d_pos_alt[j] if sign > 0 else d_pos0, n)
        else:
            nl.update_device(d_fields[j] if sign > 0 else d_neg[j])
        eam.energy_gradient_device(nl, d_e, d_grad, precision=fly.MIXED)

    clocks = Clocks(local)  # started early: nvidia-smi takes a moment to produce its first sample
    time.sleep(0.5)
    for j, sign, rb in schedule(args.warmup):
        step(j, sign, rb)
    nl.sync()
    sched = schedule(args.steps, ACC_TIMED)
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    nl.set_timing(True)
    launches0 = fly.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_clk0 = time.time()
    ev0.record(stream)
    for j, sign, rb in sched:
        step(j, sign, rb)
    ev1.record(stream)
    torch.cuda.synchronize()
    t_clk1 = time.time()
    launches = fly.launch_count() - launches0
    ktimes = nl.kernel_times()
    clk = clocks.stop(t_clk0, t_clk1)
    nl.sync()
    ms = reduce_max(ev0.elapsed_time(ev1), dev)
    value = replica_value(n, world, args.steps, ms)

    # e2e through the host C ABI with pinned host buffers
    h_fields = [torch.from_numpy(f.reshape(-1)).pin_memory() for f in fields]
    h_neg = [(-f).pin_memory() for f in h_fields]
    h_pos0 = torch.from_numpy(s.pos.reshape(-1)).pin_memory()
    h_pos_alt = [(h_pos0 - f).pin_memory() for f in h_fields]
    h_grad = torch.empty(3 * n, dtype=torch.float64).pin_memory()
    h_types, h_frozen = s.types, s.frozen
    nl.rebuild(h_pos0.numpy())
    eam.energy_gradient(h_types, h_frozen, nl, fly.MIXED, out=h_grad.numpy())

    def step_host(j, sign, rb):
        if rb:
            nl.rebuild((h_pos_alt[j] if sign > 0 else h_pos0).numpy())
        else:
            nl.update((h_fields[j] if sign > 0 else h_neg[j]).numpy())
        return eam.energy_gradient(None, None, nl, fly.MIXED, out=h_grad.numpy())[0]

    for j, sign, rb in schedule(args.warmup):
        step_host(j, sign, rb)
    if dist:
        tdist.barrier()
    t0 = time.perf_counter()
    for j, sign, rb in sched:
        step_host(j, sign, rb)
    e2e_s = reduce_max(time.perf_counter() - t0, dev)
    n_rb = sum(1 for _, _, rb in sched if rb)
    h2d = 24 * n  # a displacement field, or the positions on rebuild steps
    d2h = 24 * n + 8

    # the bit-exact binary64 path (the reference's arithmetic and summation order) on the same steps
    def step64(j, sign, rb):
        if rb:
            nl.rebuild_device(d_pos_alt[j] if sign > 0 else d_pos0, n)
        else:
            nl.update_device(d_fields[j] if sign > 0 else d_neg[j])
        eam.energy_gradient_device(nl, d_e, d_grad, precision=fly.FP64)

    nl.rebuild_device(d_pos0, n)
    for j, sign, rb in schedule(args.warmup):
        step64(j, sign, rb)
    sched64 = schedule(min(args.steps, 40), ACC_TIMED)
    torch.cuda.synchronize()
    ev2, ev3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev2.record(stream)
    for j, sign, rb in sched64:
        step64(j, sign, rb)
    ev3.record(stream)
    torch.cuda.synchronize()
    ms64 = reduce_max(ev2.elapsed_time(ev3), dev)

    def step64_host(j, sign, rb):
        if rb:
            nl.rebuild((h_pos_alt[j] if sign > 0 else h_pos0).numpy())
        else:
            nl.update((h_fields[j] if sign > 0 else h_neg[j]).numpy())
        return eam.energy_gradient(None, None, nl, fly.FP64, out=h_grad.numpy())[0]

    nl.rebuild(h_pos0.numpy())
    for j, sign, rb in schedule(args.warmup):
        step64_host(j, sign, rb)
    t0 = time.perf_counter()
    for j, sign, rb in sched64:
        step64_host(j, sign, rb)
    e2e64_s = reduce_max(time.perf_counter() - t0, dev)
    fp64_line = {"value": replica_value(n, world, len(sched64), ms64), "unit": "atom-evals/s",
                 "steps": len(sched64), "ms_per_step": ms64 / len(sched64),
                 "rebuilds": sum(1 for *_, rb in sched64 if rb),
                 "e2e": {"value": n * world * len(sched64) / e2e64_s, "unit": "atom-evals/s",
                         "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
                 "note": "binary64 EAM in the reference's operation order (bit-identical to the oracle); e2e through "
                         "the host C ABI with pinned buffers, as the headline's e2e"}

    # catalogue local environments (geometry + fingerprint of every atom) from the same list
    from openfly_gb300 import env as E

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sizes = E.local_environments(nl, eam.r_cut(), s.types, s.frozen, copy=False)
    env_s = time.perf_counter() - t0
    env_line = {"atoms": n, "r_env_A": eam.r_cut(), "seconds": env_s, "atoms_per_s": n / env_s,
                "r_ij_values": int(sizes["rij_values"]),
                "note": "flygpu_env_build: every geometry and sorted fingerprint on the device (bit-exact binary64)"}

    # whole-system relaxation (LBFGS::minimise with every vector on the device), 30 iterations
    from openfly_gb300 import search as SS

    lmin = SS.LBFGSOptions.defaults(iter_max=30, f2norm=1e-9)
    t0 = time.perf_counter()
    rmin, _ = SS.minimise_system(eam, SS.Search(s.pos, s.types, s.frozen, s.extents, s.periodic, mode=SS.MINIMISE),
                                 fly.MIXED, lbfgs=lmin)
    min_s = time.perf_counter() - t0
    min_line = {"atoms": n, "iterations": rmin["steps"], "grad_calls": rmin["grad_calls"], "seconds": min_s,
                "ms_per_iteration": 1e3 * min_s / max(1, rmin["steps"]), "precision": "mixed", "history": lmin.n,
                "note": "flygpu_minimise from the crystal's positions, list build and host transfers included"}

    hess_line = hessian_prefactor(fly, eam)

    # roofline of the dominant kernel
    peak, peak_kind = measured_peak_hbm()
    f_ms, f_cnt = ktimes["force"]
    d_ms, d_cnt = ktimes["density"]
    dom = "force" if f_ms >= d_ms else "density"
    dom_ms, dom_cnt = ktimes[dom]
    per_atom = ALGO_BYTES_FORCE if dom == "force" else ALGO_BYTES_DENSITY
    achieved = per_atom * n / (dom_ms / dom_cnt * 1e-3) / 1e9
    traffic = traffic_from_profile("k_force32" if dom == "force" else "k_density32", n)

    line = {
        "metric": METRIC, "value": value, "unit": "atom-evals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 pair terms / f64 accumulation", "data": "synthetic",
        "config": config_dict(s, args),
        "e2e": {"value": n * world * args.steps / e2e_s, "unit": "atom-evals/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_atom": per_atom},
        "kernel_ms_per_step": {k: v[0] / max(1, args.steps) for k, v in ktimes.items()},
        "rebuilds_in_window": n_rb,
        "step_algorithmic_GBps": ALGO_BYTES_STEP * n * args.steps / (ms * 1e-3) / 1e9,
        "gpu_launches": int(launches),
        "clocks": clk,
        "fp64_exact": fp64_line,
        "catalogue_envs": env_line,
        "minimise_system": min_line,
        "hessian_prefactor": hess_line,
    }
    if rank == 0 and not args.no_searches:
        line["searches"] = search_metrics(fly, args)
    if rank == 0 and not args.no_cpu and world == 1:
        threads = os.cpu_count() or 1
        os.environ.setdefault("OMP_NUM_THREADS", str(threads))
        cpu_crystal_steps(s, fields, 1, threads)  # warm-up: OpenMP threads and first-touch pages
        secs, k, rb = cpu_crystal_steps(s, fields, args.cpu_steps, threads)
        line["cpu_baseline"] = {"value": n * k / secs, "unit": "atom-evals/s", "cores": threads, "kind": "port",
                                "sample": f"{k} steps ({rb} rebuild) of the same {n}-atom workload, oracle port, "
                                          f"{threads} OpenMP threads"}
        line["parity"] = parity_block(s, par, threads)
        if "searches" in line:
            line["searches"]["batched"]["vs_oracle"] = oracle_search_agreement(line["searches"].pop("_oracle_sample"),
                                                                               threads)
        from oracle import pyoracle as O

        olmin = O.LBFGSOptions.defaults(iter_max=3, f2norm=1e-9)
        t0 = time.perf_counter()
        _, it_cpu, _, _ = O.lbfgs_minimise(O.EAMData(W.TABLE), olmin, s.extents, s.periodic, s.pos, s.types, s.frozen)
        line["minimise_system"]["cpu_ms_per_iteration"] = 1e3 * (time.perf_counter() - t0) / max(1, it_cpu)
        line["minimise_system"]["cpu_sample"] = f"oracle LBFGS::minimise, {it_cpu} iterations, {threads} threads"
        hs = HESS_SYSTEM()
        od = O.EAMData(W.TABLE)
        ol = O.List(hs.extents, hs.periodic, od.r_cut)
        t0 = time.perf_counter()
        ol.rebuild(hs.pos, 1)
        hmat = O.eam_hessian(od, ol, hs.types, hs.frozen, threads=1)
        t1 = time.perf_counter()
        hm = [od.mass(int(t)) for t in hs.types]
        O.hessian_eigenvalues(hmat, hm)
        t2 = time.perf_counter()
        act = np.repeat(hs.frozen == 0, 3)
        O.hessian_eigenvalues(O.mass_weight(hmat, hm)[np.ix_(act, act)])
        t3 = time.perf_counter()
        line["hessian_prefactor"]["cpu_ms"] = {"hessian": 1e3 * (t1 - t0), "eigenvalues": 1e3 * (t2 - t1),
                                               "eigenvalues_active_block": 1e3 * (t3 - t2)}
        line["hessian_prefactor"]["cpu_sample"] = ("oracle EAM::hessian on 1 thread (the reference's call, find.cpp:840), "
                                                   "then numpy eigvalsh (LAPACK, all host threads) of the full matrix "
                                                   "and, separately, of the active block")

    if rank == 0:
        if "searches" in line:
            line["searches"].pop("_oracle_sample", None)
        print(json.dumps(line), flush=True)
    if dist:
        tdist.destroy_process_group()


def parity_block(s, par, threads: int) -> dict:
    """The headline workload's gradient and energy against the oracle's binary64 EAM::gradient / energy on
    the same positions (the CPU leg's oracle port): binary32 pairs within the stated tolerance, binary64
    bit for bit."""
    from oracle import pyoracle as O
    from openfly_gb300 import workloads as W

    od = O.EAMData(W.TABLE)
    ol = O.List(s.extents, s.periodic, od.r_cut + SKIN)
    ol.rebuild(s.pos, threads)
    ref = O.eam_gradient(od, ol, s.types, s.frozen, threads)
    e_ref = O.eam_energy(od, ol, s.types, threads)
    e32, g32 = par["mixed"]
    e64, g64 = par["fp64"]
    err = np.abs(g32 - ref)
    big = np.abs(ref) >= 1e-2
    return {"atoms": s.n, "against": "oracle binary64 EAM::gradient/energy on the same positions",
            "mixed": {"grad_norm_rel": float(np.linalg.norm(g32 - ref) / np.linalg.norm(ref)),
                      "grad_max_abs_eV_per_A": float(err.max()),
                      "grad_max_component_rel": float((err[big] / np.abs(ref[big])).max()),
                      "grad_p99_component_rel": float(np.percentile(err[big] / np.abs(ref[big]), 99)),
                      "energy_err_eV_per_atom": abs(e32 - e_ref) / s.n,
                      "tolerance": "norm-wise relative 1e-6 (component relative over components >= 1e-2 eV/A)"},
            "fp64": {"grad_bit_identical": bool(np.array_equal(g64, ref)),
                     "energy_rel": abs(e64 - e_ref) / abs(e_ref)}}


def HESS_SYSTEM():
    """The prefactor workload: a saddle-search sized cluster (vacancy + 2 H, frozen shell): 610 atoms, 114 mobile."""
    from openfly_gb300 import workloads as W

    return W.cluster(np.random.default_rng(77), 12.0, n_vac=1, n_h=2).sys


def hessian_prefactor(fly, eam, reps: int = 5) -> dict:
    """EAM::hessian + Hessian::mass_weight + Hessian::eigenvalues of one saddle-sized cluster through the
    C ABI (list build, host copies and the eigensolve included), as Master's prefactor step runs them."""
    hs = HESS_SYSTEM()
    nl = fly.List(hs.extents, hs.periodic, eam.r_cut())
    nl.rebuild(hs.pos)
    eam.hessian_eigenvalues(hs.types, hs.frozen, nl)  # warm-up (scratch allocations)
    t0 = time.perf_counter()
    for _ in range(reps):
        nl.rebuild(hs.pos)
        ev = eam.hessian_eigenvalues(hs.types, hs.frozen, nl)
    ms = 1e3 * (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        eam.hessian(hs.types, hs.frozen, nl)
    ms_h = 1e3 * (time.perf_counter() - t0) / reps
    tol = 1e-6
    # a batch of 32 search-sized clusters: one call on 8 worker streams, and the same systems one call each
    from openfly_gb300 import search as S
    from openfly_gb300 import workloads as W

    systems = [S.from_cluster(c) for c in W.search_clusters(n=32, seed=77)]
    S.hessian_eigenvalues_batch(eam, systems[:8])  # warm-up of the worker handles
    t0 = time.perf_counter()
    S.hessian_eigenvalues_batch(eam, systems, workers=8)
    ms_b = 1e3 * (time.perf_counter() - t0) / len(systems)
    t0 = time.perf_counter()
    for x in systems:
        nl1 = fly.List(x.extents, x.periodic, eam.r_cut())
        nl1.rebuild(x.pos)
        eam.hessian_eigenvalues(x.types, x.frozen, nl1)
    ms_s = 1e3 * (time.perf_counter() - t0) / len(systems)
    return {"atoms": hs.n, "frozen": int(hs.frozen.sum()), "matrix_dim": 3 * hs.n, "ms_per_system": ms,
            "ms_hessian_to_host": ms_h, "zero_modes": int((np.abs(ev) <= tol).sum()),
            "batch": {"systems": len(systems), "mean_atoms": float(np.mean([x.n for x in systems])), "workers": 8,
                      "ms_per_system": ms_b, "one_call_each_ms_per_system": ms_s},
            "note": "flygpu_hessian_eigenvalues: binary64 Hessian (bit-exact), mass weighting, the library's own dense eigensolver (cluster Householder tridiagonalisation + Sturm multisection) on the active block"}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=600)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cells", type=int, default=80, help="bcc cells per side (80 -> 1,024,000 sites)")
    ap.add_argument("--cpu-steps", type=int, default=5, help="steps of the bounded CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-searches", action="store_true", help="skip the search metrics (configs 3 and 4)")
    ap.add_argument("--searches", type=int, default=4096, help="clusters in the batched search run")
    ap.add_argument("--plain-sample", type=int, default=32, help="searches timed on the plain path")
    ap.add_argument("--arrival-rate", type=float, default=3000.0, help="served requests per second (Poisson)")
    ap.add_argument("--steps-per-tick", type=int, default=4, help="translation steps per serving tick")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        reference_arm(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
