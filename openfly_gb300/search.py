"""Saddle searches and minimisations through libflygpu.

  DimerOptions / LBFGSOptions   Dimer::Options + Rotor::Options (saddle/dimer.hpp:56-98,
                                saddle/rotor.hpp:47-60), LBFGS::Options (minimise/LBFGS/lbfgs.hpp:56-80)
  Batch                         many searches in one persistent launch (Master::find_batch's fan-out,
                                saddle/find.cpp:684-732)
  search_plain                  one search the drop-in way: host search loop, GPU List + EAM
  Server                        continuous batching of searches (openfly_gb300.serve)
  Xoshiro / perturb             Master's random stream and Master::perturb (find.cpp:1147-1214)
  find_batch                    Master::find_batch (find.cpp:684-755): perturb, batched searches with the
                                saddle cache as history, retries on Spline::OutOfBounds, mechanisms, caching
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import EAM, FP64, MIXED, check, lib

DIMER, MINIMISE = 0, 1
EXIT_SUCCESS, EXIT_CONVEX, EXIT_ITER_MAX, EXIT_COLLISION, EXIT_UNINIT = 0, -1, -2, -3, -4


class DimerOptions(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("max_steps", C.c_int), ("hist_check_freq", C.c_int), ("use_history", C.c_int),
        ("f2norm", C.c_double), ("skin_frac", C.c_double), ("proj_tol", C.c_double), ("max_trust", C.c_double),
        ("min_trust", C.c_double), ("grow_trust", C.c_double), ("shrink_trust", C.c_double),
        ("convex_max", C.c_double),
        ("rot_n", C.c_int), ("iter_max_rot", C.c_int), ("relax_in_convex", C.c_int), ("pad_", C.c_int),
        ("delta_r", C.c_double), ("theta_tol", C.c_double),
    ]

    @classmethod
    def defaults(cls, **kw) -> "DimerOptions":
        o = cls()
        _setup()
        lib().flygpu_dimer_options_default(C.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        return o


class LBFGSOptions(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("iter_max", C.c_int), ("f2norm", C.c_double), ("skin_frac", C.c_double),
        ("proj_tol", C.c_double), ("max_trust", C.c_double), ("min_trust", C.c_double),
        ("grow_trust", C.c_double), ("shrink_trust", C.c_double),
    ]

    @classmethod
    def defaults(cls, **kw) -> "LBFGSOptions":
        o = cls()
        _setup()
        lib().flygpu_lbfgs_options_default(C.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        return o


class SearchDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("pos", C.c_void_p), ("axis", C.c_void_p), ("types", C.c_void_p),
        ("frozen", C.c_void_p), ("extents", C.c_double * 3), ("periodic", C.c_int * 3), ("mode", C.c_int),
        ("n_hist", C.c_int), ("hist", C.c_void_p), ("in_min", C.c_void_p), ("theta_tol", C.c_double),
    ]


def desc_array(searches: list, keep: list):
    """The SearchDesc array of many searches, filled column by column (one numpy assignment per field
    instead of one ctypes assignment per field and search); the descriptors point into the searches' own
    arrays, or into converted copies kept alive by ``keep``. The same contents as
    ``(SearchDesc * n)(*[s.desc(keep) for s in searches])``."""
    n = len(searches)
    out = (SearchDesc * max(1, n))()
    if n == 0:
        return out
    f = {name: getattr(SearchDesc, name).offset for name, _ in SearchDesc._fields_}
    names = ["n", "pos", "axis", "types", "frozen", "extents", "periodic", "mode", "n_hist", "hist", "in_min",
             "theta_tol"]
    dt = np.dtype({"names": names,
                   "formats": [np.int64, np.uint64, np.uint64, np.uint64, np.uint64, (np.float64, 3), (np.int32, 3),
                               np.int32, np.int32, np.uint64, np.uint64, np.float64],
                   "offsets": [f[k] for k in names], "itemsize": C.sizeof(SearchDesc)})
    rec = np.frombuffer(out, dtype=dt, count=n)

    def col(arrays):
        keep.extend(arrays)
        return np.fromiter((0 if a is None else a.ctypes.data for a in arrays), dtype=np.uint64, count=n)

    pos = [np.ascontiguousarray(x.pos, dtype=np.float64) for x in searches]
    rec["n"] = np.fromiter((p.size // 3 for p in pos), dtype=np.int64, count=n)
    rec["pos"] = col(pos)
    rec["axis"] = col([None if x.axis is None else np.ascontiguousarray(x.axis, dtype=np.float64) for x in searches])
    rec["types"] = col([np.ascontiguousarray(x.types, dtype=np.uint32) for x in searches])
    rec["frozen"] = col([np.ascontiguousarray(x.frozen, dtype=np.uint8) for x in searches])
    rec["extents"] = np.array([np.asarray(x.extents, dtype=np.float64).reshape(3) for x in searches])
    rec["periodic"] = np.array([np.asarray(x.periodic).reshape(3) for x in searches]).astype(np.int32)
    rec["mode"] = np.fromiter((x.mode for x in searches), dtype=np.int32, count=n)
    rec["theta_tol"] = np.fromiter((x.theta_tol for x in searches), dtype=np.float64, count=n)
    rec["n_hist"] = 0
    rec["hist"] = 0
    rec["in_min"] = 0
    for k, x in enumerate(searches):  # the rare per-search extras
        if x.hist or x.in_min is not None:
            d = x.desc(keep)
            rec["n_hist"][k], rec["hist"][k] = d.n_hist, d.hist or 0
            rec["in_min"][k] = d.in_min or 0
    return out


class SearchResult(C.Structure):
    _fields_ = [
        ("exit_code", C.c_int), ("status", C.c_int), ("steps", C.c_int), ("pad_", C.c_int),
        ("grad_calls", C.c_int64), ("curvature", C.c_double), ("energy", C.c_double),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad_"}


class Tuning(C.Structure):
    _fields_ = [("lanes_per_atom", C.c_int), ("threads", C.c_int), ("blocks_per_sm", C.c_int),
                ("max_registers", C.c_int)]

    def as_dict(self) -> dict:
        return {"lanes_per_atom": self.lanes_per_atom, "threads": self.threads, "blocks_per_sm": self.blocks_per_sm,
                "max_registers": self.max_registers}


_ready = False


def _setup() -> None:
    global _ready
    if _ready:
        return
    L = lib()
    V = C.c_void_p
    L.flygpu_dimer_options_default.argtypes = [V]
    L.flygpu_lbfgs_options_default.argtypes = [V]
    L.flygpu_batch_create.argtypes = [V, V, V, C.c_int, V, C.c_int, V, C.POINTER(V)]
    L.flygpu_batch_destroy.argtypes = [V]
    L.flygpu_batch_run.argtypes = [V, V]
    L.flygpu_batch_autotune.argtypes = [V, V]
    L.flygpu_batch_reset.argtypes = [V]
    L.flygpu_batch_set_stragglers.argtypes = [V, C.c_int, V]
    L.flygpu_batch_results.argtypes = [V, V, V, V]
    L.flygpu_batch_device_bytes.restype = C.c_int64
    L.flygpu_batch_device_bytes.argtypes = [V]
    L.flygpu_search_plain.argtypes = [V, V, V, C.c_int, V, V, V, V]
    L.flygpu_xoshiro_seed.argtypes = [V, V]
    L.flygpu_xoshiro_next.restype = C.c_uint64
    L.flygpu_xoshiro_next.argtypes = [V]
    L.flygpu_xoshiro_long_jump.argtypes = [V]
    L.flygpu_normal_draws.argtypes = [V, C.c_double, C.c_double, C.c_int64, V]
    L.flygpu_perturb.argtypes = [V, C.c_int64, V, V, C.c_int64, C.c_double, C.c_double, V, V, V, V]
    _ready = True


@dataclass
class Search:
    """One search request: the arguments of Dimer::find_sp (or LBFGS::minimise) for one system."""

    pos: np.ndarray
    types: np.ndarray
    frozen: np.ndarray
    extents: np.ndarray
    periodic: np.ndarray
    axis: np.ndarray | None = None
    mode: int = DIMER
    hist: list | None = None
    in_min: np.ndarray | None = None
    theta_tol: float = 0.0

    def desc(self, keep: list) -> SearchDesc:
        """A SearchDesc pointing into arrays kept alive by ``keep``."""
        def arr(a, dt):
            a = np.ascontiguousarray(a, dtype=dt).reshape(-1)
            keep.append(a)
            return a.ctypes.data

        d = SearchDesc()
        d.n = int(np.asarray(self.pos).reshape(-1, 3).shape[0])
        d.pos = arr(self.pos, np.float64)
        d.axis = arr(self.axis, np.float64) if self.axis is not None else None
        d.types = arr(self.types, np.uint32)
        d.frozen = arr(self.frozen, np.uint8)
        for k in range(3):
            d.extents[k] = float(self.extents[k])
            d.periodic[k] = int(self.periodic[k])
        d.mode = self.mode
        if self.hist:
            h = np.ascontiguousarray(np.stack([np.asarray(x, np.float64).reshape(-1) for x in self.hist]))
            keep.append(h)
            d.n_hist, d.hist = h.shape[0], h.ctypes.data
        d.in_min = arr(self.in_min, np.float64) if self.in_min is not None else None
        d.theta_tol = self.theta_tol
        return d

    @property
    def n(self) -> int:
        return int(np.asarray(self.pos).reshape(-1, 3).shape[0])


def from_cluster(cl, mode: int = DIMER) -> Search:
    s = cl.sys
    return Search(s.pos, s.types, s.frozen, s.extents, s.periodic, axis=cl.axis if mode == DIMER else None,
                  mode=mode)


class Batch:
    """Many searches resident on the GPU, run by one persistent launch."""

    def __init__(self, eam: EAM, searches: list[Search], precision: int = MIXED,
                 dimer: DimerOptions | None = None, lbfgs: LBFGSOptions | None = None, stream: int | None = None):
        _setup()
        self.searches = searches
        keep: list = []
        descs = desc_array(searches, keep)
        h = C.c_void_p()
        self.dimer = dimer or DimerOptions.defaults()
        self.lbfgs = lbfgs or LBFGSOptions.defaults()
        check(lib().flygpu_batch_create(eam.h, C.byref(self.dimer), C.byref(self.lbfgs), precision, descs,
                                        len(searches), stream, C.byref(h)), "Batch")
        self.h = h
        self.eam = eam

    def __del__(self):
        if getattr(self, "h", None):
            lib().flygpu_batch_destroy(self.h)
            self.h = None

    def run(self, tuning: Tuning | None = None) -> None:
        check(lib().flygpu_batch_run(self.h, C.byref(tuning) if tuning is not None else None), "Batch.run")

    def autotune(self) -> Tuning:
        t = Tuning()
        check(lib().flygpu_batch_autotune(self.h, C.byref(t)), "Batch.autotune")
        return t

    def reset(self) -> None:
        check(lib().flygpu_batch_reset(self.h), "Batch.reset")

    def set_stragglers(self, steps: int, wide: Tuning | None = None) -> None:
        """Two-phase runs (flygpu_batch_set_stragglers): `steps` translation steps for the whole batch in
        the throughput shape, then the unfinished searches in the `wide` shape; steps <= 0: one launch."""
        check(lib().flygpu_batch_set_stragglers(self.h, int(steps), C.byref(wide) if wide is not None else None),
              "Batch.set_stragglers")

    @property
    def device_bytes(self) -> int:
        return lib().flygpu_batch_device_bytes(self.h)

    def results(self, positions: bool = True):
        """(list of result dicts, list of (n,3) positions, list of (n,3) axes); waits for the batch."""
        n = len(self.searches)
        res = (SearchResult * n)()
        tot = sum(s.n for s in self.searches)
        pos = np.zeros(3 * tot) if positions else None
        ax = np.zeros(3 * tot) if positions else None
        check(lib().flygpu_batch_results(self.h, res, pos.ctypes.data if positions else None,
                                         ax.ctypes.data if positions else None), "Batch.results")
        out_p, out_a, o = [], [], 0
        if positions:
            for s in self.searches:
                out_p.append(pos[3 * o:3 * (o + s.n)].reshape(-1, 3))
                out_a.append(ax[3 * o:3 * (o + s.n)].reshape(-1, 3))
                o += s.n
        return [r.as_dict() for r in res], out_p, out_a


class Served(C.Structure):
    _fields_ = [("id", C.c_uint64), ("result", SearchResult), ("latency_ms", C.c_double), ("queue_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("pending", C.c_int64), ("active", C.c_int64), ("completed", C.c_int64), ("ticks", C.c_int64),
                ("hbm_used", C.c_int64), ("hbm_budget", C.c_int64)]


class Server:
    """Continuous batching of searches (flygpu_server): submit as requests arrive, poll completions."""

    def __init__(self, eam: EAM, precision: int = MIXED, hbm_budget_bytes: int = 40 << 30, max_active: int = 1024,
                 steps_per_tick: int = 8, tuning: Tuning | None = None, dimer: DimerOptions | None = None,
                 lbfgs: LBFGSOptions | None = None):
        _setup()
        L = lib()
        V = C.c_void_p
        L.flygpu_server_create.argtypes = [V, V, V, C.c_int, C.c_int64, C.c_int, C.c_int, V, C.POINTER(V)]
        L.flygpu_server_destroy.argtypes = [V]
        L.flygpu_server_submit.argtypes = [V, V, C.POINTER(C.c_uint64)]
        L.flygpu_server_submit_many.argtypes = [V, V, C.c_int, V]
        L.flygpu_server_poll.argtypes = [V, C.c_int, C.c_int, V, C.POINTER(C.c_int)]
        L.flygpu_server_take.argtypes = [V, C.c_uint64, V, V]
        L.flygpu_server_get_stats.argtypes = [V, V]
        self.dimer = dimer or DimerOptions.defaults()
        self.lbfgs = lbfgs or LBFGSOptions.defaults()
        self.tuning = tuning
        h = C.c_void_p()
        check(L.flygpu_server_create(eam.h, C.byref(self.dimer), C.byref(self.lbfgs), precision, hbm_budget_bytes,
                                     max_active, steps_per_tick, C.byref(tuning) if tuning is not None else None,
                                     C.byref(h)), "Server")
        self.h = h
        self.eam = eam
        self.n_atoms: dict[int, int] = {}

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().flygpu_server_destroy(self.h)
            self.h = None

    __del__ = close

    def submit(self, s: Search) -> int:
        keep: list = []
        d = s.desc(keep)
        rid = C.c_uint64()
        check(lib().flygpu_server_submit(self.h, C.byref(d), C.byref(rid)), "Server.submit")
        self.n_atoms[rid.value] = s.n
        return rid.value

    def submit_many(self, searches: list[Search]) -> list[int]:
        """flygpu_server_submit_many: all of them or none; returns their ids in order."""
        keep: list = []
        descs = desc_array(searches, keep)
        ids = np.zeros(max(1, len(searches)), dtype=np.uint64)
        check(lib().flygpu_server_submit_many(self.h, descs, len(searches), ids.ctypes.data), "Server.submit_many")
        out = [int(i) for i in ids[: len(searches)]]
        for rid, x in zip(out, searches):
            self.n_atoms[rid] = x.n
        return out

    def poll(self, max_n: int = 256, wait_ms: int = 0) -> list[dict]:
        buf = (Served * max_n)()
        n = C.c_int()
        check(lib().flygpu_server_poll(self.h, max_n, wait_ms, buf, C.byref(n)), "Server.poll")
        out = []
        for k in range(n.value):
            r = buf[k]
            d = r.result.as_dict()
            d.update(id=r.id, latency_ms=r.latency_ms, queue_ms=r.queue_ms)
            out.append(d)
        return out

    def take(self, rid: int):
        """(positions (n,3), axis (n,3)) of a polled request; forgets it."""
        n = self.n_atoms.pop(rid)
        pos, ax = np.zeros(3 * n), np.zeros(3 * n)
        check(lib().flygpu_server_take(self.h, rid, pos.ctypes.data, ax.ctypes.data), "Server.take")
        return pos.reshape(-1, 3), ax.reshape(-1, 3)

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().flygpu_server_get_stats(self.h, C.byref(st)), "Server.stats")
        return {k: getattr(st, k) for k, _ in st._fields_}


def centroid(x: np.ndarray) -> np.ndarray:
    """utility/lattice.hpp:203-209: the mean position (a sequential sum over atoms, then / N)."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    return np.cumsum(x, axis=0)[-1] / x.shape[0]


def centroid_align(x: np.ndarray, with_: np.ndarray) -> np.ndarray:
    """utility/lattice.hpp:214-226: x translated so that its centroid is the centroid of ``with_``."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    return x + (centroid(with_) - centroid(x))


class XoshiroState(C.Structure):
    _fields_ = [("s", C.c_uint64 * 4)]


class Xoshiro:
    """Master's random stream (saddle/find.hpp:314): xoshiro256** 1.0 (utility/random.hpp:42-162) through
    flygpu_xoshiro_*. Host only; needs no GPU."""

    def __init__(self, seed):
        _setup()
        self.st = XoshiroState()
        check(lib().flygpu_xoshiro_seed(C.byref(self.st), (C.c_uint64 * 4)(*[int(x) for x in seed])), "Xoshiro")

    @property
    def state(self) -> tuple:
        return tuple(int(x) for x in self.st.s)

    def copy(self) -> "Xoshiro":
        return Xoshiro(self.state)

    def assign(self, other: "Xoshiro") -> None:
        for k in range(4):
            self.st.s[k] = other.st.s[k]

    def next(self) -> int:
        return int(lib().flygpu_xoshiro_next(C.byref(self.st)))

    def long_jump(self) -> None:
        lib().flygpu_xoshiro_long_jump(C.byref(self.st))

    def normal(self, mean: float, stddev: float, count: int) -> np.ndarray:
        """count draws of one std::normal_distribution<double>(mean, stddev) object (libstdc++'s)."""
        out = np.zeros(count)
        check(lib().flygpu_normal_draws(C.byref(self.st), mean, stddev, count, out.ctypes.data), "normal")
        return out


def perturb(nl_pert, centre: int, in_pos, frozen, prng: Xoshiro, stddev: float = 0.6, r_pert: float = 4.0):
    """Master::perturb (find.cpp:1147-1214) through flygpu_perturb: nl_pert is a List of cut-off >= r_pert
    rebuilt on in_pos. Returns (positions (n,3), unit axis (n,3), stddev drawn); advances prng."""
    _setup()
    x = np.ascontiguousarray(in_pos, dtype=np.float64).reshape(-1)
    fz = np.ascontiguousarray(frozen, dtype=np.uint8)
    n = x.size // 3
    out, ax = np.zeros(3 * n), np.zeros(3 * n)
    sd = C.c_double()
    check(lib().flygpu_perturb(nl_pert.h, int(centre), x.ctypes.data, fz.ctypes.data, n, stddev, r_pert,
                               C.byref(prng.st), out.ctypes.data, ax.ctypes.data, C.byref(sd)), "perturb")
    return out.reshape(-1, 3), ax.reshape(-1, 3), sd.value


def theta_tol(tot: int) -> float:
    """Master::find_batch's collision angle after `tot` searches around one centre (find.cpp:692)."""
    return ((30 - 2.5) * np.exp(-0.02 * tot) + 2.5) / 360.0 * 2.0 * np.pi


def find_batch(eam: EAM, tot: int, minimum: Search, centre: int, nl_pert, cache: list, batch_size: int,
               prng: Xoshiro, geo, opts: "MasterOptions | None" = None, precision: int = MIXED,
               dimer: DimerOptions | None = None, lbfgs: LBFGSOptions | None = None, masses=None,
               zero_modes: int | None = None, tuning: Tuning | None = None, max_retries: int = 3) -> list:
    """Master::find_batch (find.cpp:684-755) over one batched launch.

    For each of batch_size searches: perturb the minimum around `centre` (`perturb`, drawing from prng),
    centroid_align onto the minimum when no atom is frozen, then run every search in one Batch with the
    saddle cache as history and the collision angle theta_tol(tot) (find_sp, find.cpp:983-1009). A search
    that ends in Spline::OutOfBounds is perturbed again and rerun, and after max_retries retries a
    RuntimeError is raised (find.cpp:706-722). The draws are those of the reference run on one thread: a
    retry's perturbation is drawn right after the failed one, so when search k needs one, the searches
    after k are perturbed again from that point of the stream and rerun with it. Each successful saddle
    goes through saddle_2_mech (`mechanisms`, geometry `geo`); a success that yields no mechanism is
    appended to cache, as the reference caches it for later collision checks (find.cpp:734-745); failed
    searches are not cached. zero_modes is the minimum's zero-mode count (None: computed from its Hessian,
    `minimum_modes`). The catalogue step that follows (add_mech) is the caller's.

    Returns one dict per search: exit_code, result (the search's result dict), pos, axis (final), start
    (perturbed positions and axis of the attempt that ran), retries, mech (None or the mechanism)."""
    from . import SPLINE_OOB

    opts = opts or MasterOptions()
    dimer = dimer or DimerOptions.defaults()
    x0 = np.asarray(minimum.pos, np.float64).reshape(-1, 3)
    frozen = np.asarray(minimum.frozen, np.uint8)
    nothing_frozen = int(frozen.sum()) == 0
    hist = [np.asarray(h, np.float64).reshape(-1, 3) for h in cache] or None
    tt = theta_tol(tot)
    starts: list = [None] * batch_size
    out: list = [None] * batch_size
    retries = [0] * batch_size
    after = [None] * batch_size  # the stream's state after each search's latest perturbation
    g, first = prng.copy(), 0
    while first < batch_size:
        for j in range(first, batch_size):
            p, a, _ = perturb(nl_pert, centre, x0, frozen, g, opts.stddev, opts.r_pert)
            if nothing_frozen:
                p = centroid_align(p, x0)
            starts[j] = (p, a)
            after[j] = g.copy()
        run = list(range(first, batch_size))
        b = Batch(eam, [Search(starts[j][0], minimum.types, frozen, minimum.extents, minimum.periodic,
                               axis=starts[j][1], in_min=x0, hist=hist, theta_tol=tt) for j in run],
                  precision=precision, dimer=dimer, lbfgs=lbfgs)
        b.run(tuning)
        res, pos, ax = b.results()
        for k, j in enumerate(run):
            out[j] = (res[k], pos[k], ax[k])
        oob = [j for j in run if out[j][0]["status"] == SPLINE_OOB]
        bad = [j for j in run if out[j][0]["status"] not in (0, SPLINE_OOB)]
        if bad:
            check(out[bad[0]][0]["status"], f"find_batch search {bad[0]}")
        if not oob:
            break
        j = oob[0]
        retries[j] += 1
        if retries[j] > max_retries:
            raise RuntimeError(f"Consecutive spline-out-of-bounds @{centre}")
        g, first = after[j].copy(), j
    prng.assign(g)
    succ = [j for j in range(batch_size) if out[j][0]["exit_code"] == EXIT_SUCCESS]
    mechs: list = [None] * batch_size
    if succ:
        ms = mechanisms(eam, [Search(out[j][1], minimum.types, frozen, minimum.extents, minimum.periodic,
                                     axis=out[j][2]) for j in succ],
                        [x0] * len(succ), [np.asarray(geo)] * len(succ), masses=masses, opts=opts, precision=precision,
                        dimer=dimer, lbfgs=lbfgs, zero_modes=None if zero_modes is None else [zero_modes] * len(succ),
                        tuning=tuning)
        for j, m in zip(succ, ms):
            mechs[j] = m
    for j in succ:
        if mechs[j] is None:
            cache.append(out[j][1].copy())
    return [dict(exit_code=out[j][0]["exit_code"], result=out[j][0], pos=out[j][1], axis=out[j][2], start=starts[j],
                 retries=retries[j], mech=mechs[j]) for j in range(batch_size)]


def furthest_atom(pos: np.ndarray, extents, periodic, i: int) -> int:
    """The entry for atom i of Master's separation list (find.cpp:224-243): the first atom at the largest
    minimum-image distance from i."""
    d = np.asarray(pos, np.float64).reshape(-1, 3) - np.asarray(pos, np.float64).reshape(-1, 3)[i]
    for k in range(3):
        if periodic[k]:
            d[:, k] -= extents[k] * np.rint(d[:, k] / extents[k])
    r = np.linalg.norm(d, axis=1)
    return int(np.argmax(r)) if r.max() > 0 else 0  # argmax returns the first maximum, as the strict > loop


def pathways(eam: EAM, saddles: list[Search], minima: list[np.ndarray], centres: list[int] | None = None,
             precision: int = MIXED, nudge_frac: float = 0.01, lbfgs: LBFGSOptions | None = None,
             tuning: Tuning | None = None):
    """Master::do_adj_min (find.cpp:1014-1090) for many saddles at once, the relaxations in one batched
    launch of the device minimiser. For each saddle (positions = the converged dimer, axis = its final
    axis) both states nudged by +/- nudge_frac of its distance from the initial minimum along the axis
    are relaxed with LBFGS::minimise; a system with no frozen atom has the atom furthest from its centre
    frozen for the relaxations (find.cpp:1026-1034). Then, as the reference: no pathway (None) if a
    relaxation fails; the relaxed state nearer the initial minimum is 'rev' (find.cpp:1054-1058); the
    centre-of-mass drift of rev is removed from rev, the saddle and fwd (find.cpp:1062-1075); and, when
    centres are given, no pathway unless the atom moving most between rev and fwd is the centre
    (find.cpp:148-173, 1082-1087). Returns per saddle None or a dict: rev, sp, fwd (n,3), their energies
    E_rev, E_sp, E_fwd (eV; translation leaves them unchanged), barrier = E_sp - E_rev, and the
    minimisers' exit codes."""
    reqs = []
    for k, (s, x0) in enumerate(zip(saddles, minima)):
        x = np.asarray(s.pos, np.float64).reshape(-1, 3)
        ax = np.asarray(s.axis, np.float64).reshape(-1, 3)
        x0 = np.asarray(x0, np.float64).reshape(-1, 3)
        disp = np.linalg.norm(x - x0)
        fz = np.asarray(s.frozen, np.uint8).copy()
        if int(fz.sum()) == 0 and centres is not None:
            fz[furthest_atom(x0, s.extents, s.periodic, centres[k])] = 1
        for sign in (1.0, -1.0):
            reqs.append(Search(x + sign * ax * disp * nudge_frac, s.types, fz, s.extents, s.periodic, mode=MINIMISE))
    b = Batch(eam, reqs, precision=precision, lbfgs=lbfgs)
    b.run(tuning)
    res, pos, _ = b.results()
    sp = Batch(eam, [Search(s.pos, s.types, s.frozen, s.extents, s.periodic, mode=MINIMISE) for s in saddles],
               precision=precision, lbfgs=LBFGSOptions.defaults(iter_max=0))
    sp.run(tuning)
    e_sp = [r["energy"] for r in sp.results(positions=False)[0]]
    out = []
    for k, (s, x0) in enumerate(zip(saddles, minima)):
        fwd, rev = pos[2 * k], pos[2 * k + 1]
        rf, rr = res[2 * k], res[2 * k + 1]
        if rf["status"] != 0 or rr["status"] != 0 or rf["exit_code"] != 0 or rr["exit_code"] != 0:
            out.append(None)
            continue
        x0 = np.asarray(x0, np.float64).reshape(-1, 3)
        if np.linalg.norm(rev - x0) > np.linalg.norm(fwd - x0):
            fwd, rev, rf, rr = rev, fwd, rr, rf
        drift = centroid(rev) - centroid(x0)
        rev, x_sp, fwd = rev - drift, np.asarray(s.pos, np.float64).reshape(-1, 3) - drift, fwd - drift
        if centres is not None:
            r = ((rev - fwd) ** 2).sum(axis=1)
            if (int(np.argmax(r)) if r.max() > 0 else 0) != centres[k]:
                out.append(None)
                continue
        out.append(dict(rev=rev, sp=x_sp, fwd=fwd, E_rev=rr["energy"], E_sp=e_sp[k], E_fwd=rf["energy"],
                        barrier=e_sp[k] - rr["energy"], exit_rev=rr["exit_code"], exit_fwd=rf["exit_code"]))
    return out


def minimise_system(eam: EAM, s: Search, precision: int = FP64, lbfgs: LBFGSOptions | None = None):
    """LBFGS::minimise of one system of any size with every vector on the device (flygpu_minimise); returns
    (result dict, final positions (n,3)). For a whole-system relaxation, not a batch of small ones."""
    _setup()
    L = lib()
    if not getattr(L, "_minimise_ready", False):
        V = C.c_void_p
        L.flygpu_minimise.argtypes = [V, V, C.c_int, C.c_int64, V, V, V, V, V, V, V, V]
        L._minimise_ready = True
    pos = np.ascontiguousarray(s.pos, dtype=np.float64).reshape(-1)
    ty = np.ascontiguousarray(s.types, dtype=np.uint32)
    fz = np.ascontiguousarray(s.frozen, dtype=np.uint8)
    ext = np.ascontiguousarray(s.extents, dtype=np.float64)
    per = np.ascontiguousarray(s.periodic, dtype=np.int32)
    out = np.zeros_like(pos)
    r = SearchResult()
    lbfgs = lbfgs or LBFGSOptions.defaults()
    check(L.flygpu_minimise(eam.h, C.byref(lbfgs), precision, pos.size // 3, pos.ctypes.data, ty.ctypes.data,
                            fz.ctypes.data, ext.ctypes.data, per.ctypes.data, None, out.ctypes.data, C.byref(r)),
          "minimise_system")
    return r.as_dict(), out.reshape(-1, 3)


def hessian_eigenvalues_batch(eam: EAM, systems: list, masses=None, workers: int = 8) -> list:
    """The prefactor step (EAM::hessian + Hessian::mass_weight + Hessian::eigenvalues, find.cpp:838-871) for
    many systems in one call (flygpu_hessian_eigenvalues_batch); returns each system's ascending
    eigenvalues (3n,). systems: Search objects (positions, types, frozen, box; the search fields are not
    used); masses per type (None: the potential file's)."""
    _setup()
    keep: list = []
    descs = desc_array(systems, keep)
    sizes = [3 * s.n for s in systems]
    eig = np.zeros(max(1, sum(sizes)), dtype=np.float64)
    m = None if masses is None else np.ascontiguousarray(masses, dtype=np.float64)
    check(lib().flygpu_hessian_eigenvalues_batch(eam.h, descs, len(systems), None if m is None else m.ctypes.data,
                                                 workers, eig.ctypes.data), "Hessian batch")
    return list(np.split(eig[: sum(sizes)], np.cumsum(sizes)[:-1])) if systems else []


def search_plain(eam: EAM, s: Search, precision: int = FP64, dimer: DimerOptions | None = None,
                 lbfgs: LBFGSOptions | None = None):
    """One search the drop-in way; returns (result dict, positions (n,3), axis (n,3))."""
    _setup()
    keep: list = []
    d = s.desc(keep)
    pos = np.zeros(3 * s.n)
    ax = np.zeros(3 * s.n)
    r = SearchResult()
    dimer = dimer or DimerOptions.defaults()
    lbfgs = lbfgs or LBFGSOptions.defaults()
    check(lib().flygpu_search_plain(eam.h, C.byref(dimer), C.byref(lbfgs), precision, C.byref(d), pos.ctypes.data,
                                    ax.ctypes.data, C.byref(r)), "search_plain")
    return r.as_dict(), pos.reshape(-1, 3), ax.reshape(-1, 3)


AMU_KG = 1.6605390666050e-27  # the atomic mass unit in kg, as find.cpp:288 writes it


class MasterOptions:
    """The Master::Options fields the mechanism step reads (saddle/find.hpp:100-160), with the reference's
    defaults."""

    def __init__(self, basin_tol: float = 0.05, stationary_tol: float | None = None, capture_r_tol: float = 0.05,
                 capture_E_tol: float = 0.01, hessian_eigen_zero_tol: float = 1e-6, nudge_frac: float = 0.01,
                 r_pert: float = 4.0, stddev: float = 0.6):
        self.r_pert = r_pert  # find.hpp:97
        self.stddev = stddev  # find.hpp:101
        self.basin_tol = basin_tol
        self.stationary_tol = basin_tol / 2 if stationary_tol is None else stationary_tol
        self.capture_r_tol = capture_r_tol
        self.capture_E_tol = capture_E_tol
        self.hessian_eigen_zero_tol = hessian_eigen_zero_tol
        self.nudge_frac = nudge_frac


def _modes(freq: np.ndarray, tol: float):
    """Counts of the sorted eigenvalues: (negative, zero, sum of log of the positive ones)."""
    neg = int((freq < -tol).sum())
    pos = freq[freq > tol]
    return neg, int(freq.size - neg - pos.size), float(np.sum(np.log(pos)))


def minimum_modes(eam: EAM, minima: list[Search], masses=None, opts: MasterOptions | None = None) -> list[dict]:
    """Master::calc_minima_hess (find.cpp:1094-1144) for each minimum: the log product of the non-zero
    mass-weighted Hessian eigenvalues and the number of zero modes. Raises, as the reference's verify,
    on a negative mode or a zero-mode count other than 3 per frozen atom (3 when none is frozen)."""
    opts = opts or MasterOptions()
    out = []
    for s, freq in zip(minima, hessian_eigenvalues_batch(eam, minima, masses)):
        neg, zeros, logp = _modes(freq, opts.hessian_eigen_zero_tol)
        if neg:
            raise RuntimeError(f"Mode 0 has eigenvalue = {freq[0]}")
        n_frozen = int(np.asarray(s.frozen).sum())
        expect = 3 * n_frozen if n_frozen > 0 else 3
        if zeros != expect:
            raise RuntimeError(f"Expecting {expect} zero modes but found {zeros}")
        out.append(dict(log_prod_eigen=logp, zero_modes=zeros, count_frozen=n_frozen))
    return out


def mechanisms(eam: EAM, saddles: list[Search], minima: list[np.ndarray], geos: list, masses=None,
               opts: MasterOptions | None = None, precision: int = MIXED, dimer: DimerOptions | None = None,
               lbfgs: LBFGSOptions | None = None, zero_modes: list[int] | None = None,
               tuning: Tuning | None = None) -> list:
    """Master::saddle_2_mech (find.cpp:757-981) for many saddles, every relaxation batched on the device.

    For saddle k (positions = the converged dimer, axis = its axis, types/frozen = the initial minimum's)
    with initial minimum minima[k] and local geometry geos[k] (atom indices, the centre first):
    do_adj_min (`pathways`); no mechanism if rev lies more than basin_tol from the initial minimum,
    fwd within basin_tol of rev, or the saddle within stationary_tol of rev or fwd (:771-797); the
    barrier E_sp - E_rev (which must be positive) and delta E_fwd - E_rev; the saddle and final-state
    displacements and the normalised axis on the geometry's atoms (:807-836); the prefactor from the
    saddle's mass-weighted Hessian (:838-871): exactly one negative mode (a second one: no mechanism),
    the zero modes counted against zero_modes[k] (default: the initial minimum's, `minimum_modes`) and
    kinetic_pre = sum of the log of the positive eigenvalues, and with the minimum's log product the
    prefactor sqrt(exp(log_prod_min - kinetic_pre) / (2 pi amu)) in Hz (find.cpp:286-292; None when
    zero_modes is given); and recon_relax (:77-125, :874-956): the
    mechanism rebuilt on rev, the minimum relaxed with LBFGS::minimise and the saddle with Dimer::find_sp,
    each compared (after centroid alignment) with the pathway's fwd and saddle within capture_r_tol and
    capture_E_tol (poison_fwd / poison_sp). Raises where the reference throws (a non-positive barrier, no
    negative mode, a wrong zero-mode count, a poisoned final state with a barrier under 0.5 eV).
    Returns per saddle None or a dict of the mechanism."""
    opts = opts or MasterOptions()
    dimer = dimer or DimerOptions.defaults()
    lbfgs = lbfgs or LBFGSOptions.defaults()
    centres = [int(g[0]) for g in geos]
    paths = pathways(eam, saddles, minima, centres, precision=precision, nudge_frac=opts.nudge_frac, lbfgs=lbfgs,
                     tuning=tuning)
    keep = []
    for k, p in enumerate(paths):
        if p is None:
            continue
        x0 = np.asarray(minima[k], np.float64).reshape(-1, 3)
        rev, sp, fwd = p["rev"], p["sp"], p["fwd"]
        if (np.linalg.norm(rev - x0) > opts.basin_tol or np.linalg.norm(fwd - rev) < opts.basin_tol
                or np.linalg.norm(rev - sp) < opts.stationary_tol or np.linalg.norm(fwd - sp) < opts.stationary_tol):
            continue
        if not p["E_sp"] > p["E_rev"]:
            raise RuntimeError(f"Bad internal state Esp={p['E_sp']} but E0={p['E_rev']}!")
        keep.append(k)
    log_prod = {}
    if zero_modes is None and keep:
        mins = [Search(minima[k], saddles[k].types, saddles[k].frozen, saddles[k].extents, saddles[k].periodic)
                for k in keep]
        mm = minimum_modes(eam, mins, masses, opts)
        zero_modes = {k: m["zero_modes"] for k, m in zip(keep, mm)}
        log_prod = {k: m["log_prod_eigen"] for k, m in zip(keep, mm)}
    elif zero_modes is not None:
        zero_modes = {k: zero_modes[k] for k in keep}
    # prefactors at the saddles (one batched call)
    sps = [Search(paths[k]["sp"], saddles[k].types, saddles[k].frozen, saddles[k].extents, saddles[k].periodic)
           for k in keep]
    freqs = dict(zip(keep, hessian_eigenvalues_batch(eam, sps, masses))) if keep else {}
    mech = {}
    for k in keep:
        p, geo = paths[k], np.asarray(geos[k], np.int64)
        freq = freqs[k]
        tol = opts.hessian_eigen_zero_tol
        if not freq[0] < -tol:
            raise RuntimeError(f"Saddle-point with minimum mode={freq[0]}")
        neg, zeros, logp = _modes(freq[1:], tol)
        if neg:
            continue  # second-order saddle point or higher
        if zeros != zero_modes[k]:
            raise RuntimeError(f"Expecting {zero_modes[k]} zero modes but hessian has {zeros}")
        ax = np.asarray(saddles[k].axis, np.float64).reshape(-1, 3)[geo]
        mech[k] = dict(barrier=p["E_sp"] - p["E_rev"], delta=p["E_fwd"] - p["E_rev"],
                       delta_sp=p["sp"][geo] - p["rev"][geo], delta_fwd=p["fwd"][geo] - p["rev"][geo],
                       axis=ax / np.sqrt((ax * ax).sum()), kinetic_pre=logp, geo=geo,
                       prefactor_hz=(float(np.sqrt(np.exp(log_prod[k] - logp) / (2 * np.pi * AMU_KG)))
                                     if k in log_prod else None),
                       rev=p["rev"], sp=p["sp"], fwd=p["fwd"], E_rev=p["E_rev"], E_sp=p["E_sp"], E_fwd=p["E_fwd"])
    # recon_relax: rebuild every mechanism on its rev and relax both states (one batched launch)
    reqs, slots = [], []
    for k, m in mech.items():
        s, ref = saddles[k], m["rev"]
        re_min, re_sp = ref.copy(), ref.copy()
        re_min[m["geo"]] += m["delta_fwd"]
        re_sp[m["geo"]] += m["delta_sp"]
        if int(np.asarray(s.frozen).sum()) == 0:
            re_sp = centroid_align(re_sp, ref)
        axis = np.zeros_like(ref)
        axis[m["geo"]] = m["axis"]
        m["re_min"], m["re_sp"] = re_min, re_sp
        slots.append(k)
        reqs.append(Search(re_min, s.types, s.frozen, s.extents, s.periodic, mode=MINIMISE))
        reqs.append(Search(re_sp, s.types, s.frozen, s.extents, s.periodic, axis=axis, in_min=ref))
    if reqs:
        b = Batch(eam, reqs, precision=precision, dimer=dimer, lbfgs=lbfgs)
        b.run(tuning)
        res, pos, _ = b.results()
    out = [None] * len(saddles)
    for j, k in enumerate(slots):
        m = mech[k]
        for which, r, x, ref_x, e_ref in (("fwd", res[2 * j], pos[2 * j], m["fwd"], m["E_fwd"]),
                                            ("sp", res[2 * j + 1], pos[2 * j + 1], m["sp"], m["E_sp"])):
            if r["status"] != 0 or r["exit_code"] != 0:
                m["poison_" + which], m["err_" + which] = True, None
                continue
            m["err_" + which] = float(np.linalg.norm(x - m["re_min" if which == "fwd" else "re_sp"]))
            aligned = centroid_align(x, ref_x)
            m["poison_" + which] = bool(np.linalg.norm(aligned - ref_x) > opts.capture_r_tol
                                        or abs(r["energy"] - e_ref) > opts.capture_E_tol)
        if m["poison_fwd"] and m["barrier"] < 0.5:
            raise RuntimeError(f"Mechanism @{int(m['geo'][0])} with energy barrier = {m['barrier']}eV is poisoned! "
                               f"err_sp={m['err_sp']}, err_min={m['err_fwd']}")
        out[k] = m
    return out
