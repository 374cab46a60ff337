"""ctypes wrapper over the CPU oracle (oracle/flyoracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU legs of bench.py as
the checker. The product package never imports this module.

Beyond the C++ restatements it restates in Python the host-side glue of Master (saddle/find.cpp):
do_adj_min (:1014-1090, `adj_min`), saddle_2_mech with recon_relax (:757-981, :77-125, `mechanism`),
calc_minima_hess (:1094-1144, `minimum_modes`), the catalogue's local environments
(env/catalogue.cpp:66-78, `local_environment`) and Hessian::mass_weight / eigenvalues
(system/hessian.hpp:86-93,136-143).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libflyoracle.so")

OK, INVALID, SPLINE_OOB, GHOST_OVERFLOW = 0, 1, 2, 3


class OracleError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"oracle {what} failed with status {status}")
        self.status = status


def build() -> str:
    """Compile the oracle with its Makefile (a few seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


class DimerOptions(C.Structure):
    """Dimer::Options (dimer.hpp:56-98) followed by Rotor::Options (rotor.hpp:47-60)."""

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
        o = cls(n=10, max_steps=1000, hist_check_freq=5, use_history=1, f2norm=1e-5, skin_frac=1.1, proj_tol=0.0,
                max_trust=0.5, min_trust=0.05, grow_trust=1.5, shrink_trust=0.5, convex_max=3.0, rot_n=6,
                iter_max_rot=20, relax_in_convex=1, pad_=0, delta_r=0.001, theta_tol=np.pi / 360.0)
        for k, v in kw.items():
            setattr(o, k, v)
        return o


class LBFGSOptions(C.Structure):
    """LBFGS::Options (lbfgs.hpp:56-80)."""

    _fields_ = [
        ("n", C.c_int), ("iter_max", C.c_int), ("f2norm", C.c_double), ("skin_frac", C.c_double),
        ("proj_tol", C.c_double), ("max_trust", C.c_double), ("min_trust", C.c_double),
        ("grow_trust", C.c_double), ("shrink_trust", C.c_double),
    ]

    @classmethod
    def defaults(cls, **kw) -> "LBFGSOptions":
        o = cls(n=10, iter_max=2000, f2norm=1e-6, skin_frac=1.1, proj_tol=0.0, max_trust=0.5, min_trust=0.01,
                grow_trust=1.5, shrink_trust=0.5)
        for k, v in kw.items():
            setattr(o, k, v)
        return o


_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_lp = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_bp = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_SO):
            build()
        L = C.CDLL(_SO)
        V = C.c_void_p
        L.orc_eam_load.restype = V
        L.orc_eam_load.argtypes = [C.c_char_p]
        L.orc_eam_free.argtypes = [V]
        L.orc_eam_rcut.restype = C.c_double
        L.orc_eam_rcut.argtypes = [V]
        L.orc_eam_ntypes.argtypes = [V]
        L.orc_eam_mass.restype = C.c_double
        L.orc_eam_mass.argtypes = [V, C.c_int]
        L.orc_spline_eval.argtypes = [V, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_double)]
        L.orc_spline_table.restype = C.c_long
        L.orc_spline_table.argtypes = [V, C.c_int, C.c_int, C.c_int, V, C.c_long]
        L.orc_list_new.restype = V
        L.orc_list_new.argtypes = [_dp, _ip, C.c_double]
        L.orc_list_free.argtypes = [V]
        L.orc_list_rebuild.argtypes = [V, _dp, C.c_long, C.c_int]
        L.orc_list_update.argtypes = [V, _dp]
        L.orc_list_num_ghosts.restype = C.c_long
        L.orc_list_num_ghosts.argtypes = [V]
        L.orc_list_shape.argtypes = [V, _ip]
        L.orc_list_slots.restype = C.c_long
        L.orc_list_slots.argtypes = [V, V, V, C.c_long]
        L.orc_list_neighbours.restype = C.c_long
        L.orc_list_neighbours.argtypes = [V, C.c_double, _ip, V, V, C.c_long]
        L.orc_list_raw.restype = C.c_long
        L.orc_list_raw.argtypes = [V, _ip, V, C.c_long]
        L.orc_eam_energy.argtypes = [V, V, _up, C.c_int, C.POINTER(C.c_double)]
        L.orc_eam_gradient.argtypes = [V, V, _up, _bp, C.c_int, _dp]
        L.orc_eam_hessian.argtypes = [V, V, _up, _bp, C.c_int, _dp]
        L.orc_spline_build.restype = C.c_long
        L.orc_spline_build.argtypes = [_dp, C.c_long, C.c_double, V, C.c_long]
        L.orc_spline_points.argtypes = [_dp, C.c_long, C.c_double, _dp, C.c_long, _dp]
        L.orc_eam_fprime.argtypes = [V, V, _up, _bp, _dp]
        L.orc_brute_neighbours.restype = C.c_long
        L.orc_brute_neighbours.argtypes = [_dp, _ip, _dp, C.c_long, C.c_double, _ip, V, V, C.c_long]
        L.orc_lbfgs_minimise.argtypes = [V, C.POINTER(LBFGSOptions), _dp, _ip, C.c_long, _dp, _up, _bp, _dp,
                                         C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.orc_dimer_find_sp.argtypes = [V, C.POINTER(DimerOptions), _dp, _ip, C.c_long, _dp, _dp, _up, _bp, _dp, V,
                                        C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_long), C.POINTER(C.c_double)]
        L.orc_dimer_batch.argtypes = [V, C.POINTER(DimerOptions), C.c_int, _lp, _dp, _ip, _dp, _dp, _up, _bp, _ip,
                                      C.c_int, _ip, _ip]
        L.orc_xoshiro.argtypes = [_u64p, _u64p, C.c_long]
        L.orc_normal_draws.argtypes = [_u64p, C.c_double, C.c_double, C.c_long, _dp]
        L.orc_perturb.argtypes = [C.c_void_p, C.c_long, _dp, _u8p, C.c_long, C.c_double, C.c_double, _u64p, _dp,
                                  _dp, C.POINTER(C.c_double)]
        L.orc_max_threads.restype = C.c_int
        L.orc_adjacent.argtypes = [_ip, C.c_int, _ip]
        L.orc_cell_idx.argtypes = [_dp, C.c_double, _dp]
        _lib = L
    return _lib


def _check(st: int, what: str) -> None:
    if st != OK:
        raise OracleError(st, what)


def normal_draws(state, mean: float, stddev: float, count: int):
    """count draws of std::normal_distribution<double>(mean, stddev) (libstdc++) from the xoshiro256**
    stream in state; returns (draws, state after)."""
    st = np.array(state, dtype=np.uint64)
    out = np.zeros(count, dtype=np.float64)
    lib().orc_normal_draws(st, mean, stddev, count, out)
    return out, st


def perturb(nl: "List", centre: int, in_pos, frozen, stddev: float, r_pert: float, state):
    """Master::perturb (find.cpp:1147-1214) with nl built with cut-off r_pert on in_pos; returns
    (positions (n,3), axis (n,3), stddev drawn, state after)."""
    x = np.ascontiguousarray(in_pos, dtype=np.float64).reshape(-1)
    n = x.size // 3
    out, ax = np.zeros(3 * n), np.zeros(3 * n)
    st = np.array(state, dtype=np.uint64)
    sd = C.c_double()
    _check(lib().orc_perturb(nl.h, centre, x, np.ascontiguousarray(frozen, dtype=np.uint8), n, stddev, r_pert, st,
                             out, ax, C.byref(sd)), "perturb")
    return out.reshape(-1, 3), ax.reshape(-1, 3), sd.value, st


def find_batch(data: EAMData, dimer_opt: DimerOptions, lbfgs_opt: LBFGSOptions, tot: int, extents, periodic,
               in_pos, types, frozen, centre: int, nl_pert: "List", cache: list, batch_size: int, state, geo,
               masses, zero_modes: int, stddev: float = 0.6, r_pert: float = 4.0, max_retries: int = 3):
    """Master::find_batch (saddle/find.cpp:684-755) run on one thread: per search, perturb (:707) and
    centroid_align when nothing is frozen (:709-711), Dimer::find_sp with the cache as history and the
    collision angle of :692 (find_sp, :983-1009), retried with a new perturbation on Spline::OutOfBounds
    up to max_retries times before raising (:712-721); saddle_2_mech on a success (:725-729); after the
    batch, a success without a mechanism is cached (:734-745). Returns (per-search dicts, state after)."""
    theta_tol = ((30 - 2.5) * np.exp(-0.02 * tot) + 2.5) / 360.0 * 2.0 * np.pi
    x0 = np.asarray(in_pos, np.float64).reshape(-1, 3)
    fz = np.asarray(frozen, np.uint8)
    nothing_frozen = int(fz.sum()) == 0
    hist = [np.asarray(h, np.float64).reshape(-1, 3) for h in cache]
    out = []
    for _ in range(batch_size):
        retry = 0
        while True:
            p, a, _, state = perturb(nl_pert, centre, x0, fz, stddev, r_pert, state)
            if nothing_frozen:
                p = p + (np.cumsum(x0, axis=0)[-1] / x0.shape[0] - np.cumsum(p, axis=0)[-1] / p.shape[0])
            try:
                r = dimer_find_sp(data, dimer_opt, extents, periodic, p, a, types, fz, in_min=x0, hist=hist or None,
                                  theta_tol=theta_tol)
                break
            except OracleError as e:
                if e.status != SPLINE_OOB:
                    raise
                retry += 1
                if retry > max_retries:
                    raise RuntimeError(f"Consecutive spline-out-of-bounds @{centre}")
        mech = None
        if r["exit"] == 0:
            mech = mechanism(data, dimer_opt, lbfgs_opt, extents, periodic, types, fz, x0, r["x"], r["axis"], geo,
                             masses, zero_modes)
        out.append(dict(exit=r["exit"], steps=r["steps"], x=r["x"], axis=r["axis"], start=(p, a), retries=retry,
                        mech=mech))
    for o in out:
        if o["mech"] is None and o["exit"] == 0:
            cache.append(o["x"].copy())
    return out, state


def xoshiro(seed, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.uint64)
    lib().orc_xoshiro(np.asarray(seed, dtype=np.uint64), out, n)
    return out


class EAMData:
    """DataEAM (data.cpp:67-153) parsed by the oracle."""

    def __init__(self, path: str):
        self.h = lib().orc_eam_load(path.encode())
        if not self.h:
            raise OracleError(INVALID, f"load {path}")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_eam_free(self.h)
            self.h = None

    @property
    def r_cut(self) -> float:
        return lib().orc_eam_rcut(self.h)

    @property
    def n_types(self) -> int:
        return lib().orc_eam_ntypes(self.h)

    def mass(self, t: int) -> float:
        return lib().orc_eam_mass(self.h, t)

    def spline(self, kind: int, a: int, b: int, deriv: int, x: float) -> float:
        out = C.c_double()
        _check(lib().orc_spline_eval(self.h, kind, a, b, deriv, x, C.byref(out)), "spline")
        return out.value

    def table(self, kind: int, a: int, b: int = 0) -> np.ndarray:
        n = lib().orc_spline_table(self.h, kind, a, b, None, 0)
        out = np.zeros((n, 4), dtype=np.float64)
        lib().orc_spline_table(self.h, kind, a, b, out.ctypes.data, out.size)
        return out


class List:
    """neigh::List (list.hpp:71-211) restated."""

    def __init__(self, extents, periodic, r_cut: float):
        self.ext = np.ascontiguousarray(extents, dtype=np.float64)
        self.per = np.ascontiguousarray(periodic, dtype=np.int32)
        self.h = lib().orc_list_new(self.ext, self.per, float(r_cut))
        if not self.h:
            raise OracleError(INVALID, "List()")
        self.n = 0

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_list_free(self.h)
            self.h = None

    def rebuild(self, pos: np.ndarray, threads: int = 1) -> None:
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        self.n = pos.size // 3
        _check(lib().orc_list_rebuild(self.h, pos, self.n, threads), "rebuild")

    def update(self, delta: np.ndarray) -> None:
        _check(lib().orc_list_update(self.h, np.ascontiguousarray(delta, dtype=np.float64).reshape(-1)), "update")

    @property
    def num_ghosts(self) -> int:
        return lib().orc_list_num_ghosts(self.h)

    def shape(self) -> np.ndarray:
        s = np.zeros(3, dtype=np.int32)
        lib().orc_list_shape(self.h, s)
        return s

    def slots(self):
        tot = lib().orc_list_slots(self.h, None, None, 0)
        pos = np.zeros((tot, 3), dtype=np.float64)
        img = np.zeros(tot, dtype=np.int64)
        lib().orc_list_slots(self.h, pos.ctypes.data, img.ctypes.data, tot)
        return pos, img

    def neighbours(self, r_cut: float):
        """(counts, real indices, dr) in for_neighbours order, CSR."""
        counts = np.zeros(self.n, dtype=np.int32)
        tot = lib().orc_list_neighbours(self.h, r_cut, counts, None, None, 0)
        if tot < 0:
            raise OracleError(INVALID, "neighbours")
        idx = np.zeros(tot, dtype=np.int32)
        dr = np.zeros((tot, 3), dtype=np.float64)
        lib().orc_list_neighbours(self.h, r_cut, counts, idx.ctypes.data, dr.ctypes.data, tot)
        return counts, idx, dr

    def raw(self):
        counts = np.zeros(self.n, dtype=np.int32)
        tot = lib().orc_list_raw(self.h, counts, None, 0)
        slots = np.zeros(tot, dtype=np.int32)
        lib().orc_list_raw(self.h, counts, slots.ctypes.data, tot)
        return counts, slots


def eam_energy(data: EAMData, nl: List, types: np.ndarray, threads: int = 1) -> float:
    e = C.c_double()
    _check(lib().orc_eam_energy(data.h, nl.h, np.ascontiguousarray(types, dtype=np.uint32), threads, C.byref(e)),
           "energy")
    return e.value


def eam_gradient(data: EAMData, nl: List, types: np.ndarray, frozen: np.ndarray, threads: int = 1) -> np.ndarray:
    g = np.zeros(3 * nl.n, dtype=np.float64)
    _check(lib().orc_eam_gradient(data.h, nl.h, np.ascontiguousarray(types, dtype=np.uint32),
                                  np.ascontiguousarray(frozen, dtype=np.uint8), threads, g), "gradient")
    return g.reshape(-1, 3)


def eam_hessian(data: EAMData, nl: List, types: np.ndarray, frozen: np.ndarray, threads: int = 1) -> np.ndarray:
    """EAM::hessian (eam.cpp:122-233): the dense (3n, 3n) matrix with only its lower 3x3 blocks filled."""
    h = np.zeros(9 * nl.n * nl.n, dtype=np.float64)
    _check(lib().orc_eam_hessian(data.h, nl.h, np.ascontiguousarray(types, dtype=np.uint32),
                                 np.ascontiguousarray(frozen, dtype=np.uint8), threads, h), "hessian")
    return h.reshape(3 * nl.n, 3 * nl.n)


def spline_build(y, dx: float) -> np.ndarray:
    """Spline::Spline (spline.cpp:27-103): the (n + 4, 4) coefficients {a, b, c, d} of a sample table."""
    y = np.ascontiguousarray(y, dtype=np.float64)
    n = lib().orc_spline_build(y, y.size, dx, None, 0)
    out = np.zeros((n, 4), dtype=np.float64)
    lib().orc_spline_build(y, y.size, dx, out.ctypes.data, out.size)
    return out


def spline_points(y, dx: float, x) -> np.ndarray:
    """Spline::f / fp / fpp (spline.hpp:100-123) of the spline of a sample table: (m, 3)."""
    y = np.ascontiguousarray(y, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.zeros((x.size, 3), dtype=np.float64)
    _check(lib().orc_spline_points(y, y.size, dx, x, x.size, out), "spline")
    return out


def mass_weight(h: np.ndarray, masses: np.ndarray) -> np.ndarray:
    """Hessian::mass_weight (system/hessian.hpp:136-143): every 3x3 block (j, i) times 1/sqrt(m_i m_j);
    masses per atom."""
    m = np.repeat(np.asarray(masses, np.float64), 3)
    return h * (1.0 / np.sqrt(np.outer(m, m)))


def hessian_eigenvalues(lower: np.ndarray, masses: np.ndarray | None = None) -> np.ndarray:
    """Hessian::mass_weight (when masses are given) then Hessian::eigenvalues (system/hessian.hpp:86-93):
    the ascending eigenvalues of the symmetric matrix the lower triangle defines (SelfAdjointEigenSolver
    reads the lower triangle only)."""
    w = lower if masses is None else mass_weight(lower, masses)
    return np.linalg.eigvalsh(w, UPLO="L")


def eam_fprime(data: EAMData, nl: List, types: np.ndarray, frozen: np.ndarray) -> np.ndarray:
    fp = np.zeros(nl.n, dtype=np.float64)
    _check(lib().orc_eam_fprime(data.h, nl.h, np.ascontiguousarray(types, dtype=np.uint32),
                                np.ascontiguousarray(frozen, dtype=np.uint8), fp), "fprime")
    return fp


def brute_neighbours(extents, periodic, pos: np.ndarray, r_cut: float):
    ext = np.ascontiguousarray(extents, dtype=np.float64)
    per = np.ascontiguousarray(periodic, dtype=np.int32)
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
    n = pos.size // 3
    counts = np.zeros(n, dtype=np.int32)
    tot = lib().orc_brute_neighbours(ext, per, pos, n, r_cut, counts, None, None, 0)
    idx = np.zeros(tot, dtype=np.int32)
    dr = np.zeros((tot, 3), dtype=np.float64)
    lib().orc_brute_neighbours(ext, per, pos, n, r_cut, counts, idx.ctypes.data, dr.ctypes.data, tot)
    return counts, idx, dr


def lbfgs_minimise(data: EAMData, opt: LBFGSOptions, extents, periodic, pos, types, frozen):
    """Returns (failed, iters, positions, gradient)."""
    x = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1).copy()
    g = np.zeros_like(x)
    failed, iters = C.c_int(), C.c_int()
    _check(lib().orc_lbfgs_minimise(data.h, C.byref(opt), np.ascontiguousarray(extents, dtype=np.float64),
                                    np.ascontiguousarray(periodic, dtype=np.int32), x.size // 3, x,
                                    np.ascontiguousarray(types, dtype=np.uint32),
                                    np.ascontiguousarray(frozen, dtype=np.uint8), g, C.byref(failed),
                                    C.byref(iters)), "lbfgs")
    return bool(failed.value), iters.value, x.reshape(-1, 3), g.reshape(-1, 3)


def local_environment(counts, idx, dr, types, frozen, i: int):
    """Catalogue::rebuild_env up to the hash for atom i, from the list's (counts, idx, dr) in visiting
    order: rebuild_geo_from_nl (env/geometry.hpp:391-407) and Fingerprint::rebuild (env/heuristics.hpp:
    93-110), binary64 in the reference's operation order (sequential centroid sum, (x^2 + y^2) + z^2).
    Returns (positions (K,3), colours, indices, sorted r_0j, sorted r_ij)."""
    o = int(np.sum(counts[:i]))
    c = int(counts[i])
    p = [np.zeros(3)] + [np.asarray(dr[o + k], np.float64) for k in range(c)]
    col = [2 * int(types[i]) + int(frozen[i])] + [2 * int(types[q]) + int(frozen[q]) for q in idx[o:o + c]]
    ind = [i] + [int(q) for q in idx[o:o + c]]
    s = np.zeros(3)
    for v in p:  # Vec::Zero() += each position, in order
        s = s + v
    cen = s / float(len(p))
    q = [v - cen for v in p]

    def norm(d):
        return np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])

    r0 = sorted(norm(q[j] - q[0]) for j in range(1, len(q)))
    rij = sorted(norm(q[a] - q[b]) for a in range(1, len(q)) for b in range(1, a))
    return np.array(q), np.array(col), np.array(ind), np.array(r0), np.array(rij)


def furthest_atom(pos, extents, periodic, i: int) -> int:
    """Master's separation list entry for atom i (saddle/find.cpp:224-243): the first atom at the largest
    minimum-image distance from i."""
    d = np.asarray(pos, np.float64) - np.asarray(pos, np.float64)[i]
    for k in range(3):
        if periodic[k]:
            d[:, k] -= extents[k] * np.rint(d[:, k] / extents[k])
    r = np.linalg.norm(d, axis=1)
    k_best, best = 0, 0.0
    for j in range(r.size):  # strict > keeps the first maximum, as the reference's loop
        if r[j] > best:
            k_best, best = j, r[j]
    return k_best


def adj_min(data: EAMData, opt: LBFGSOptions, extents, periodic, types, frozen, dimer_pos, dimer_axis, in_pos,
            centre: int | None, nudge_frac: float = 0.01):
    """Master::do_adj_min (saddle/find.cpp:1014-1090): relax from the saddle nudged by +/- nudge_frac of its
    distance from the initial minimum along the axis (freezing the atom furthest from the centre when
    nothing is frozen, :1026-1034), call the relaxed state nearer the initial minimum 'rev' (:1054-1058),
    remove the centre-of-mass drift of rev from all three states (:1062-1075), and require the atom that
    moves most between rev and fwd to be the centre (min_max, :148-173 and :1082-1087). Returns None
    where the reference returns no pathway, else dict(rev, sp, fwd)."""
    x0 = np.asarray(in_pos, np.float64).reshape(-1, 3)
    x = np.asarray(dimer_pos, np.float64).reshape(-1, 3)
    ax = np.asarray(dimer_axis, np.float64).reshape(-1, 3)
    fz = np.asarray(frozen, np.uint8).copy()
    disp = np.linalg.norm(x - x0)
    if int(fz.sum()) == 0 and centre is not None:
        fz[furthest_atom(x0, extents, periodic, centre)] = 1
    got = []
    for sign in (1.0, -1.0):
        failed, _, xm, _ = lbfgs_minimise(data, opt, extents, periodic, x + sign * ax * disp * nudge_frac, types, fz)
        if failed:
            return None
        got.append(xm)
    fwd, rev = got
    if np.linalg.norm(rev - x0) > np.linalg.norm(fwd - x0):
        fwd, rev = rev, fwd
    drift = rev.mean(axis=0) - x0.mean(axis=0)
    rev, sp, fwd = rev - drift, x - drift, fwd - drift
    if centre is not None:
        r = ((rev - fwd) ** 2).sum(axis=1)
        k_max, best = 0, 0.0
        for j in range(r.size):
            if r[j] > best:
                k_max, best = j, r[j]
        if k_max != centre:
            return None
    return dict(rev=rev, sp=sp, fwd=fwd)


def dimer_find_sp(data: EAMData, opt: DimerOptions, extents, periodic, pos, axis, types, frozen, in_min=None,
                  hist=None, theta_tol: float = 0.0, count_frozen: int | None = None):
    """Dimer::find_sp. Returns dict(exit, steps, grad_calls, curv, x, axis)."""
    x = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1).copy()
    ax = np.ascontiguousarray(axis, dtype=np.float64).reshape(-1).copy()
    fz = np.ascontiguousarray(frozen, dtype=np.uint8)
    if count_frozen is None:
        count_frozen = int(fz.sum())
    im = x.copy() if in_min is None else np.ascontiguousarray(in_min, dtype=np.float64).reshape(-1)
    n_hist = 0
    hp = None
    if hist is not None and len(hist):
        h = np.ascontiguousarray(np.stack([np.asarray(s, dtype=np.float64).reshape(-1) for s in hist]))
        n_hist, hp = h.shape[0], h
    ex, st, gc, cv = C.c_int(), C.c_int(), C.c_long(), C.c_double()
    _check(lib().orc_dimer_find_sp(data.h, C.byref(opt), np.ascontiguousarray(extents, dtype=np.float64),
                                   np.ascontiguousarray(periodic, dtype=np.int32), x.size // 3, x, ax,
                                   np.ascontiguousarray(types, dtype=np.uint32), fz, im,
                                   None if hp is None else hp.ctypes.data, n_hist, theta_tol, count_frozen,
                                   C.byref(ex), C.byref(st), C.byref(gc), C.byref(cv)), "dimer")
    return dict(exit=ex.value, steps=st.value, grad_calls=gc.value, curv=cv.value, x=x.reshape(-1, 3),
                axis=ax.reshape(-1, 3))


def dimer_batch(data: EAMData, opt: DimerOptions, offsets, extents, periodic, pos, axis, types, frozen,
                count_frozen, threads: int):
    """Independent searches spread over threads (Master::find_batch's fan-out). In-place on copies."""
    x = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1).copy()
    ax = np.ascontiguousarray(axis, dtype=np.float64).reshape(-1).copy()
    ns = len(offsets) - 1
    ex = np.zeros(ns, dtype=np.int32)
    st = np.zeros(ns, dtype=np.int32)
    _check(lib().orc_dimer_batch(data.h, C.byref(opt), ns, np.ascontiguousarray(offsets, dtype=np.int64),
                                 np.ascontiguousarray(extents, dtype=np.float64).reshape(-1),
                                 np.ascontiguousarray(periodic, dtype=np.int32).reshape(-1), x, ax,
                                 np.ascontiguousarray(types, dtype=np.uint32),
                                 np.ascontiguousarray(frozen, dtype=np.uint8),
                                 np.ascontiguousarray(count_frozen, dtype=np.int32), threads, ex, st), "dimer_batch")
    return ex, st, x.reshape(-1, 3), ax.reshape(-1, 3)


def max_threads() -> int:
    return lib().orc_max_threads()


def adjacent(shape, cell: int) -> list[int]:
    """AdjacentCells (neigh/adjacent.hpp:40-70) of one cell."""
    out = np.zeros(26, dtype=np.int32)
    n = lib().orc_adjacent(np.ascontiguousarray(shape, dtype=np.int32), cell, out)
    return out[:n].tolist()


def cell_idx(extents, r_cut: float, x) -> int:
    """HyperGrid(extents, r_cut).cell_idx(x) (system/boxes/hypergrid.hpp:43-99)."""
    return lib().orc_cell_idx(np.ascontiguousarray(extents, dtype=np.float64), r_cut,
                              np.ascontiguousarray(x, dtype=np.float64))


def _energy_at(data: EAMData, extents, periodic, pos, types) -> float:
    nl = List(extents, periodic, data.r_cut)
    nl.rebuild(np.asarray(pos, np.float64), 1)
    return eam_energy(data, nl, types)


def _frequencies(data: EAMData, extents, periodic, pos, types, frozen, masses) -> np.ndarray:
    nl = List(extents, periodic, data.r_cut)
    nl.rebuild(np.asarray(pos, np.float64), 1)
    return hessian_eigenvalues(eam_hessian(data, nl, types, frozen), masses)


def minimum_modes(data: EAMData, extents, periodic, pos, types, frozen, masses, tol: float = 1e-6) -> dict:
    """Master::calc_minima_hess (saddle/find.cpp:1094-1144): log product of the non-zero eigenvalues and the
    zero-mode count; raises on a negative mode or a count other than 3 per frozen atom (3 when none)."""
    freq = _frequencies(data, extents, periodic, pos, types, frozen, masses)
    logp, zeros = 0.0, 0
    for i in range(freq.size):
        if not freq[i] > -tol:
            raise RuntimeError(f"Mode {i} has eigenvalue = {freq[i]}")
        if freq[i] > tol:
            logp += float(np.log(freq[i]))
        else:
            zeros += 1
    n_frozen = int(np.asarray(frozen).sum())
    expect = 3 * n_frozen if n_frozen > 0 else 3
    if zeros != expect:
        raise RuntimeError(f"Expecting {expect} zero modes but found {zeros}")
    return dict(log_prod_eigen=logp, zero_modes=zeros)


def mechanism(data: EAMData, dimer_opt: DimerOptions, lbfgs_opt: LBFGSOptions, extents, periodic, types, frozen,
              in_pos, sp_pos, sp_axis, geo, masses, zero_modes: int, basin_tol: float = 0.05,
              stationary_tol: float = 0.025, capture_r_tol: float = 0.05, capture_e_tol: float = 0.01,
              zero_tol: float = 1e-6, nudge_frac: float = 0.01):
    """Master::saddle_2_mech (saddle/find.cpp:757-981) with recon_relax (:77-125) for one saddle: the
    pathway (adj_min) and its checks (:771-797), the three energies on rebuilt lists (:801-810), the
    mechanism on the geometry's atoms (:812-836), the prefactor (:838-871) and the reconstruction onto
    rev with its poison tests (:874-956). Returns None where the reference returns no mechanism; raises
    where it throws."""
    geo = np.asarray(geo, np.int64)
    path = adj_min(data, lbfgs_opt, extents, periodic, types, frozen, sp_pos, sp_axis, in_pos, int(geo[0]),
                   nudge_frac)
    if path is None:
        return None
    x0 = np.asarray(in_pos, np.float64).reshape(-1, 3)
    rev, sp, fwd = path["rev"], path["sp"], path["fwd"]
    if np.linalg.norm(rev - x0) > basin_tol or np.linalg.norm(fwd - rev) < basin_tol:
        return None
    if np.linalg.norm(rev - sp) < stationary_tol or np.linalg.norm(fwd - sp) < stationary_tol:
        return None
    e0 = _energy_at(data, extents, periodic, rev, types)
    esp = _energy_at(data, extents, periodic, sp, types)
    ef = _energy_at(data, extents, periodic, fwd, types)
    if not esp > e0:
        raise RuntimeError(f"Bad internal state Esp={esp} but E0={e0}!")
    ax = np.asarray(sp_axis, np.float64).reshape(-1, 3)[geo]
    s = 0.0
    for a in ax:
        s += float(a @ a)
    m = dict(barrier=esp - e0, delta=ef - e0, delta_sp=sp[geo] - rev[geo], delta_fwd=fwd[geo] - rev[geo],
             axis=ax / np.sqrt(s), rev=rev, sp=sp, fwd=fwd)
    freq = _frequencies(data, extents, periodic, sp, types, frozen, masses)
    if not freq[0] < -zero_tol:
        raise RuntimeError(f"Saddle-point with minimum mode={freq[0]}")
    pre, zeros = 0.0, 0
    for i in range(1, freq.size):
        if freq[i] < -zero_tol:
            return None
        if freq[i] > zero_tol:
            pre += float(np.log(freq[i]))
        else:
            zeros += 1
    if zeros != zero_modes:
        raise RuntimeError(f"Expecting {zero_modes} zero modes but hessian has {zeros}")
    m["kinetic_pre"] = pre
    # recon_relax onto rev
    re_min, re_sp = rev.copy(), rev.copy()
    re_min[geo] += m["delta_fwd"]
    re_sp[geo] += m["delta_sp"]
    n_frozen = int(np.asarray(frozen).sum())
    if n_frozen == 0:
        re_sp = re_sp + (rev.mean(axis=0) - re_sp.mean(axis=0))
    axis = np.zeros_like(rev)
    axis[geo] = m["axis"]
    failed, _, rel_min, _ = lbfgs_minimise(data, lbfgs_opt, extents, periodic, re_min, types, frozen)
    d = dimer_find_sp(data, dimer_opt, extents, periodic, re_sp, axis, types, frozen, in_min=rev,
                      count_frozen=n_frozen)
    for which, ok, x, base, ref_x, e_ref in (("fwd", not failed, rel_min, re_min, fwd, ef),
                                             ("sp", d["exit"] == 0, d["x"], re_sp, sp, esp)):
        if not ok:
            m["poison_" + which], m["err_" + which] = True, None
            continue
        x = np.asarray(x, np.float64).reshape(-1, 3)
        m["err_" + which] = float(np.linalg.norm(x - base))
        x = x + (ref_x.mean(axis=0) - x.mean(axis=0))
        e = _energy_at(data, extents, periodic, x, types)
        m["poison_" + which] = bool(np.linalg.norm(x - ref_x) > capture_r_tol or abs(e - e_ref) > capture_e_tol)
    if m["poison_fwd"] and m["barrier"] < 0.5:
        raise RuntimeError(f"Mechanism @{int(geo[0])} with energy barrier = {m['barrier']}eV is poisoned!")
    return m
