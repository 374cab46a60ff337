"""Small, fixed cases of the library's kernels for profilers (ncu captures of one kernel at a time).

    python -m openfly_gb300.cases --search-batch N [--max-search-steps S] [--precision mixed|fp64]
        one batched launch over N search clusters (2 lanes per atom, 128 threads, 2 CTAs per SM)
    python -m openfly_gb300.cases --search-tail
        the 4096-cluster search batch run once; the searches that needed more than 100 translation steps
        then run alone in the wide shape (4 lanes, 256 threads, 1 CTA per SM) as one launch
    python -m openfly_gb300.cases --prefactor
        the Hessian prefactor step: one 610-atom search cluster (EAM::hessian, mass weighting,
        eigenvalues) five times, then a batch of 32 clusters

Each prints one JSON line describing what ran. These are not benchmarks: bench.py is.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def search_batch(n: int, max_steps: int, precision: str) -> dict:
    import openfly_gb300 as fly
    from openfly_gb300 import search as S
    from openfly_gb300 import workloads as W

    eam = fly.EAM(W.TABLE)
    opt = S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=max_steps)
    prec = fly.MIXED if precision == "mixed" else fly.FP64
    b = S.Batch(eam, [S.from_cluster(c) for c in W.search_clusters(n=n, seed=7)], precision=prec, dimer=opt)
    t0 = time.perf_counter()
    b.run(S.Tuning(2, 128, 2, 0))
    res, _, _ = b.results(positions=False)
    return {"search_batch": len(res), "precision": precision, "seconds": time.perf_counter() - t0,
            "grad_calls": int(sum(r["grad_calls"] for r in res)), "errors": int(sum(r["status"] != 0 for r in res))}


def search_tail(n: int = 4096) -> dict:
    import openfly_gb300 as fly
    from openfly_gb300 import search as S
    from openfly_gb300 import workloads as W

    eam = fly.EAM(W.TABLE)
    opt = S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-3, max_steps=1000)
    cl = W.search_clusters(n=n, seed=7)
    b = S.Batch(eam, [S.from_cluster(c) for c in cl], precision=fly.MIXED, dimer=opt)
    b.set_stragglers(0)
    b.run(S.Tuning(8, 256, 2, 128))
    res, _, _ = b.results(positions=False)
    tail = [k for k, r in enumerate(res) if r["steps"] > 100]
    bt = S.Batch(eam, [S.from_cluster(cl[k]) for k in tail], precision=fly.MIXED, dimer=opt)
    bt.set_stragglers(0)
    t0 = time.perf_counter()
    bt.run(S.Tuning(4, 256, 1, 0))
    r2, _, _ = bt.results(positions=False)
    return {"search_tail": len(tail), "seconds": time.perf_counter() - t0,
            "max_grad_calls": int(max(r["grad_calls"] for r in r2))}


def prefactor(reps: int = 5) -> dict:
    import openfly_gb300 as fly
    from openfly_gb300 import search as S
    from openfly_gb300 import workloads as W

    eam = fly.EAM(W.TABLE)
    hs = W.cluster(np.random.default_rng(77), 12.0, n_vac=1, n_h=2).sys
    nl = fly.List(hs.extents, hs.periodic, eam.r_cut())
    nl.rebuild(hs.pos)
    eam.hessian_eigenvalues(hs.types, hs.frozen, nl)
    t0 = time.perf_counter()
    for _ in range(reps):
        nl.rebuild(hs.pos)
        eam.hessian_eigenvalues(hs.types, hs.frozen, nl)
    one = 1e3 * (time.perf_counter() - t0) / reps
    systems = [S.from_cluster(c) for c in W.search_clusters(n=32, seed=77)]
    S.hessian_eigenvalues_batch(eam, systems[:8])
    t0 = time.perf_counter()
    S.hessian_eigenvalues_batch(eam, systems, workers=8)
    return {"prefactor_atoms": hs.n, "ms_per_system": one,
            "batch_ms_per_system": 1e3 * (time.perf_counter() - t0) / len(systems)}


def main() -> None:
    from openfly_gb300.build import build

    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--search-batch", type=int, default=0)
    ap.add_argument("--max-search-steps", type=int, default=1000)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--search-tail", action="store_true")
    ap.add_argument("--prefactor", action="store_true")
    a = ap.parse_args()
    build()
    if a.search_batch > 0:
        out = search_batch(a.search_batch, a.max_search_steps, a.precision)
    elif a.search_tail:
        out = search_tail()
    elif a.prefactor:
        out = prefactor()
    else:
        ap.error("choose a case")
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
