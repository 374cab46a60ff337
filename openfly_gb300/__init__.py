"""openfly_gb300 -- the GB300 (sm_103a) saddle-search inner loop of openFLY behind a C ABI.

Python mirror of the reference's interfaces for this path, calling libflygpu through ctypes:
  List          fly::neigh::List            (include/libfly/neigh/list.hpp:71-211)
  EAM           fly::potential::EAM         (include/libfly/potential/EAM/eam.hpp:42-120)
plus the search entry points added in openfly_gb300.search. There is no CPU fallback: importing a
compute entry point without the built library raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB as _LIB_PATH

FP64, MIXED = 0, 1

OK, INVALID_ARG, SPLINE_OOB, GHOST_OVERFLOW, NLIST_OVERFLOW, OOM, TIMEOUT, CUDA_ERROR = range(8)


class FlyGPUError(RuntimeError):
    """A non-zero status from libflygpu (fly::RuntimeError in the reference)."""

    def __init__(self, status: int, what: str, detail: str = ""):
        super().__init__(f"{what}: {status_string(status)} (status {status}){': ' + detail if detail else ''}")
        self.status = status


class SplineOutOfBounds(FlyGPUError):
    """Spline::OutOfBounds (utility/spline.hpp:46-51): an argument left the tabulated region."""


_lib: C.CDLL | None = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def lib() -> C.CDLL:
    """Load libflygpu.so (built in-tree by openfly_gb300.build). Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise ImportError(f"libflygpu is not built ({_LIB_PATH} missing): run openfly_gb300.build.build()")
    L = C.CDLL(_LIB_PATH)
    V, I64 = C.c_void_p, C.c_int64
    L.flygpu_status_string.restype = C.c_char_p
    L.flygpu_status_string.argtypes = [C.c_int]
    L.flygpu_last_error.restype = C.c_char_p
    L.flygpu_eam_load.argtypes = [C.c_char_p, C.POINTER(V)]
    L.flygpu_eam_destroy.argtypes = [V]
    L.flygpu_eam_r_cut.restype = C.c_double
    L.flygpu_eam_r_cut.argtypes = [V]
    L.flygpu_eam_n_types.argtypes = [V]
    L.flygpu_eam_table.restype = I64
    L.flygpu_eam_table.argtypes = [V, C.c_int, C.c_int, C.c_int, V, I64]
    L.flygpu_list_create.argtypes = [_dp, _ip, C.c_double, V, C.POINTER(V)]
    L.flygpu_list_destroy.argtypes = [V]
    L.flygpu_list_rebuild.argtypes = [V, V, I64]
    L.flygpu_list_rebuild_device.argtypes = [V, V, I64]
    L.flygpu_list_update.argtypes = [V, V]
    L.flygpu_list_update_device.argtypes = [V, V]
    L.flygpu_list_size.restype = I64
    L.flygpu_list_size.argtypes = [V]
    L.flygpu_list_num_ghosts.restype = I64
    L.flygpu_list_num_ghosts.argtypes = [V]
    L.flygpu_list_neighbours.argtypes = [V, C.c_double, V, V, V, I64, C.POINTER(I64)]
    L.flygpu_list_sync.argtypes = [V]
    L.flygpu_list_set_timing.argtypes = [V, C.c_int]
    L.flygpu_list_kernel_times.argtypes = [V, V, V]
    L.flygpu_launch_count.restype = I64
    for name in ("flygpu_eam_energy",):
        getattr(L, name).argtypes = [V, V, V, V, C.c_int, V]
    L.flygpu_eam_gradient.argtypes = [V, V, V, V, C.c_int, V]
    L.flygpu_eam_energy_gradient.argtypes = [V, V, V, V, C.c_int, V, V]
    L.flygpu_eam_energy_gradient_device.argtypes = [V, V, V, V, C.c_int, V, V]
    L.flygpu_eam_hessian.argtypes = [V, V, V, V, V]
    L.flygpu_spline_build.restype = I64
    L.flygpu_spline_build.argtypes = [V, I64, C.c_double, V, I64]
    L.flygpu_hessian_eigenvalues.argtypes = [V, V, V, V, V, V, V]
    L.flygpu_hessian_eigenvalues_batch.argtypes = [V, V, C.c_int, V, C.c_int, V]
    _lib = L
    return L


def spline_build(y, dx: float) -> np.ndarray:
    """Spline::Spline (spline.cpp:27-103) as every EAM table is built: (n + 4, 4) binary64 {a,b,c,d}."""
    y = np.ascontiguousarray(y, dtype=np.float64)
    n = lib().flygpu_spline_build(y.ctypes.data, y.size, dx, None, 0)
    if n < 0:
        raise FlyGPUError(1, "Spline", lib().flygpu_last_error().decode())
    out = np.zeros((n, 4), dtype=np.float64)
    lib().flygpu_spline_build(y.ctypes.data, y.size, dx, out.ctypes.data, out.size)
    return out


def launch_count() -> int:
    """Kernels libflygpu has launched since it was loaded."""
    return lib().flygpu_launch_count()


def status_string(status: int) -> str:
    return lib().flygpu_status_string(status).decode()


def check(status: int, what: str) -> None:
    if status != OK:
        detail = lib().flygpu_last_error().decode()
        cls = SplineOutOfBounds if status == SPLINE_OOB else FlyGPUError
        raise cls(status, what, detail)


def _ptr(a) -> int | None:
    """Address of a numpy array or a torch tensor (host or device), None for None."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def _host(a, dtype) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=dtype).reshape(-1)


class EAM:
    """fly::potential::EAM over device spline tables built from a LAMMPS eam/fs file
    (DataEAM, potential/EAM/data.hpp:54)."""

    def __init__(self, path: str):
        h = C.c_void_p()
        check(lib().flygpu_eam_load(path.encode(), C.byref(h)), f"EAM({path})")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.flygpu_eam_destroy(self.h)
            self.h = None

    def r_cut(self) -> float:
        """EAM::r_cut (eam.hpp:71)."""
        return lib().flygpu_eam_r_cut(self.h)

    @property
    def n_types(self) -> int:
        return lib().flygpu_eam_n_types(self.h)

    def table(self, kind: int, a: int, b: int = 0) -> np.ndarray:
        """binary64 spline coefficients {a,b,c,d} per interval of F(a) (kind 0), phi(a,b) (1), v(a,b) (2)."""
        n = lib().flygpu_eam_table(self.h, kind, a, b, None, 0)
        if n < 0:
            raise FlyGPUError(INVALID_ARG, "table")
        out = np.zeros((n, 4), dtype=np.float64)
        lib().flygpu_eam_table(self.h, kind, a, b, out.ctypes.data, out.size)
        return out

    def energy(self, types, frozen, nl: "List", precision: int = FP64) -> float:
        """EAM::energy (eam.hpp:83)."""
        e = C.c_double()
        t, f = _host(types, np.uint32), _host(frozen, np.uint8)
        check(lib().flygpu_eam_energy(self.h, nl.h, t.ctypes.data, f.ctypes.data, precision, C.addressof(e)),
              "EAM::energy")
        return e.value

    def gradient(self, types, frozen, nl: "List", precision: int = FP64) -> np.ndarray:
        """EAM::gradient (eam.hpp:95); returns (n, 3)."""
        g = np.zeros(3 * nl.size(), dtype=np.float64)
        t, f = _host(types, np.uint32), _host(frozen, np.uint8)
        check(lib().flygpu_eam_gradient(self.h, nl.h, t.ctypes.data, f.ctypes.data, precision, g.ctypes.data),
              "EAM::gradient")
        return g.reshape(-1, 3)

    def energy_gradient(self, types, frozen, nl: "List", precision: int = FP64, out: np.ndarray | None = None):
        """Both in one density pass and one force pass; returns (energy, gradient (n, 3))."""
        g = np.zeros(3 * nl.size(), dtype=np.float64) if out is None else out
        e = C.c_double()
        t = None if types is None else _host(types, np.uint32)
        f = None if frozen is None else _host(frozen, np.uint8)
        check(lib().flygpu_eam_energy_gradient(self.h, nl.h, _ptr(t), _ptr(f), precision, C.addressof(e), _ptr(g)),
              "EAM::energy+gradient")
        return e.value, g.reshape(-1, 3)

    def hessian(self, types, frozen, nl: "List") -> np.ndarray:
        """EAM::hessian (eam.hpp:110): the dense (3n, 3n) binary64 matrix, lower 3x3 blocks filled."""
        n = nl.size()
        h = np.zeros((3 * n, 3 * n), dtype=np.float64)
        t, f = _host(types, np.uint32), _host(frozen, np.uint8)
        check(lib().flygpu_eam_hessian(self.h, nl.h, t.ctypes.data, f.ctypes.data, h.ctypes.data), "EAM::hessian")
        return h

    def hessian_eigenvalues(self, types, frozen, nl: "List", masses=None, weighted: bool = False):
        """Hessian::mass_weight + Hessian::eigenvalues (system/hessian.hpp:86-93,136-143) of EAM::hessian:
        ascending eigenvalues (3n,); masses per type (None: the potential file's). With weighted=True
        also returns the mass-weighted matrix."""
        n = nl.size()
        eig = np.zeros(3 * n, dtype=np.float64)
        w = np.zeros((3 * n, 3 * n), dtype=np.float64) if weighted else None
        t, f = _host(types, np.uint32), _host(frozen, np.uint8)
        m = None if masses is None else _host(masses, np.float64)
        check(lib().flygpu_hessian_eigenvalues(self.h, nl.h, t.ctypes.data, f.ctypes.data, _ptr(m), eig.ctypes.data,
                                               _ptr(w)), "Hessian::eigenvalues")
        return (eig, w) if weighted else eig

    def energy_gradient_device(self, nl: "List", d_energy, d_grad, d_types=None, d_frozen=None,
                               precision: int = MIXED) -> None:
        """Device-pointer form (torch CUDA tensors); does not synchronise."""
        check(lib().flygpu_eam_energy_gradient_device(self.h, nl.h, _ptr(d_types), _ptr(d_frozen), precision,
                                                      _ptr(d_energy), _ptr(d_grad)), "EAM::energy+gradient")


class List:
    """fly::neigh::List for an orthorhombic box (list.hpp:86-90): extents (3,), periodic (3,) flags."""

    def __init__(self, extents, periodic, r_cut: float, stream: int | None = None):
        h = C.c_void_p()
        self.extents = np.ascontiguousarray(extents, dtype=np.float64)
        self.periodic = np.ascontiguousarray(periodic, dtype=np.int32)
        check(lib().flygpu_list_create(self.extents, self.periodic, float(r_cut), stream, C.byref(h)), "List()")
        self.h = h
        self.r_cut = float(r_cut)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.flygpu_list_destroy(self.h)
            self.h = None

    def rebuild(self, positions) -> None:
        """List::rebuild (list.hpp:98). positions: (n, 3) host array."""
        p = _host(positions, np.float64)
        check(lib().flygpu_list_rebuild(self.h, p.ctypes.data, p.size // 3), "List::rebuild")

    def rebuild_device(self, d_pos, n: int) -> None:
        check(lib().flygpu_list_rebuild_device(self.h, _ptr(d_pos), n), "List::rebuild")

    def update(self, delta) -> None:
        """List::update (list.hpp:118): r <- r - delta."""
        d = _host(delta, np.float64)
        check(lib().flygpu_list_update(self.h, d.ctypes.data), "List::update")

    def update_device(self, d_delta) -> None:
        check(lib().flygpu_list_update_device(self.h, _ptr(d_delta)), "List::update")

    def size(self) -> int:
        return lib().flygpu_list_size(self.h)

    @property
    def num_ghosts(self) -> int:
        return lib().flygpu_list_num_ghosts(self.h)

    def sync(self) -> None:
        check(lib().flygpu_list_sync(self.h), "List sync")

    KERNELS = ("density", "force", "update", "rebuild")

    def set_timing(self, enable: bool) -> None:
        """Record CUDA events around the density, force, update and rebuild kernels."""
        check(lib().flygpu_list_set_timing(self.h, int(enable)), "set_timing")

    def kernel_times(self) -> dict:
        """{kernel: (total ms, launches)} since the last call; synchronises the list's stream."""
        ms = np.zeros(4, dtype=np.float64)
        cnt = np.zeros(4, dtype=np.int64)
        check(lib().flygpu_list_kernel_times(self.h, ms.ctypes.data, cnt.ctypes.data), "kernel_times")
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.KERNELS)}

    def neighbours(self, r_cut: float):
        """(counts, real indices, dr) of every pair List::for_neighbours visits, in visiting order."""
        n = self.size()
        counts = np.zeros(n, dtype=np.int32)
        tot = C.c_int64()
        check(lib().flygpu_list_neighbours(self.h, r_cut, counts.ctypes.data, None, None, 0, C.byref(tot)),
              "neighbours")
        idx = np.zeros(tot.value, dtype=np.int32)
        dr = np.zeros((tot.value, 3), dtype=np.float64)
        check(lib().flygpu_list_neighbours(self.h, r_cut, counts.ctypes.data, idx.ctypes.data, dr.ctypes.data,
                                           tot.value, C.byref(tot)), "neighbours")
        return counts, idx, dr
