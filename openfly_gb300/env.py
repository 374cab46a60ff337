"""Catalogue local environments on the GPU (flygpu_env_*): geometry and fingerprint of every atom.

Mirrors Catalogue::rebuild_env (env/catalogue.cpp:66-78) up to the graph hash: rebuild_geo_from_nl
(env/geometry.hpp:391-407) and Fingerprint::rebuild (env/heuristics.hpp:93-110).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import List, check, lib

_ready = False


def _setup() -> None:
    global _ready
    if _ready:
        return
    L = lib()
    V = C.c_void_p
    L.flygpu_env_build.argtypes = [V, C.c_double, V, V, C.POINTER(V)]
    L.flygpu_env_sizes.argtypes = [V, V, V, V, V]
    L.flygpu_env_get.argtypes = [V, V, V, V, V, V, V, V]
    L.flygpu_env_destroy.argtypes = [V]
    L.flygpu_env_destroy.restype = None
    _ready = True


@dataclass
class Environments:
    """geo_offsets (n+1); geo_pos (G,3), geo_colour (G,), geo_index (G,) for all atoms' geometries;
    r0j (G-n,) with atom i's values at geo_offsets[i]-i .. geo_offsets[i+1]-i-1; rij_offsets (n+1), rij."""

    geo_offsets: np.ndarray
    geo_pos: np.ndarray
    geo_colour: np.ndarray
    geo_index: np.ndarray
    r0j: np.ndarray
    rij_offsets: np.ndarray
    rij: np.ndarray

    def geometry(self, i: int):
        a, b = self.geo_offsets[i], self.geo_offsets[i + 1]
        return self.geo_pos[a:b], self.geo_colour[a:b], self.geo_index[a:b]

    def fingerprint(self, i: int):
        a, b = self.geo_offsets[i], self.geo_offsets[i + 1]
        return self.r0j[a - i:b - i - 1], self.rij[self.rij_offsets[i]:self.rij_offsets[i + 1]]


def local_environments(nl: List, r_env: float, types: np.ndarray, frozen: np.ndarray, copy: bool = True):
    """Every atom's local environment from the GPU neighbour list ``nl`` (built on the current positions).
    copy=False builds them on the device and returns only the sizes (atoms, geometry entries, r_0j and
    r_ij values) without copying them to the host."""
    _setup()
    L = lib()
    ty = np.ascontiguousarray(types, dtype=np.uint32)
    fz = np.ascontiguousarray(frozen, dtype=np.uint8)
    h = C.c_void_p()
    check(L.flygpu_env_build(nl.h, float(r_env), ty.ctypes.data, fz.ctypes.data, C.byref(h)), "local_environments")
    try:
        n, g, r0, rij = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(L.flygpu_env_sizes(h, C.byref(n), C.byref(g), C.byref(r0), C.byref(rij)), "local_environments")
        if not copy:
            return dict(atoms=n.value, geometry_entries=g.value, r0j_values=r0.value, rij_values=rij.value)
        out = Environments(np.zeros(n.value + 1, np.int64), np.zeros((g.value, 3)), np.zeros(g.value, np.int32),
                           np.zeros(g.value, np.int32), np.zeros(r0.value), np.zeros(n.value + 1, np.int64),
                           np.zeros(rij.value))
        check(L.flygpu_env_get(h, out.geo_offsets.ctypes.data, out.geo_pos.ctypes.data, out.geo_colour.ctypes.data,
                               out.geo_index.ctypes.data, out.rij_offsets.ctypes.data, out.r0j.ctypes.data,
                               out.rij.ctypes.data), "local_environments")
    finally:
        L.flygpu_env_destroy(h)
    return out
