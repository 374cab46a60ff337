"""Pinned host buffers through the host C ABI: a pinned gradient buffer receives the force pass's stores
directly over the host link, a pinned update delta is copied asynchronously. Both must give the same bits
as pageable buffers, which take the copy path."""
import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _pinned(a: np.ndarray) -> np.ndarray:
    t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    return t.numpy()


@pytest.mark.parametrize("precision", ["FP64", "MIXED"])
def test_pinned_update_and_gradient_equal_pageable(gpu, geam, precision):
    prec = getattr(gpu, precision)
    s = W.fe_h_crystal(n_cells=8)
    rng = np.random.default_rng(3)
    deltas = [rng.normal(0, 0.01, s.pos.shape) for _ in range(3)]
    rc = geam.r_cut() + 0.3
    a = gpu.List(s.extents, s.periodic, rc)
    b = gpu.List(s.extents, s.periodic, rc)
    a.rebuild(s.pos)
    b.rebuild(s.pos)
    g_page = np.empty(3 * s.n)
    g_pin = _pinned(np.zeros(3 * s.n))
    ea, _ = geam.energy_gradient(s.types, s.frozen, a, prec, out=g_page)
    eb, _ = geam.energy_gradient(s.types, s.frozen, b, prec, out=g_pin)
    assert ea == eb and np.array_equal(g_page, g_pin)
    for d in deltas:
        a.update(d.reshape(-1))
        b.update(_pinned(d.reshape(-1)))
        ea, _ = geam.energy_gradient(None, None, a, prec, out=g_page)
        eb, _ = geam.energy_gradient(None, None, b, prec, out=g_pin)
        assert ea == eb
        assert np.array_equal(g_page, g_pin)
    # a pageable update on the pinned-gradient list, and the reverse, keep agreeing
    a.update(_pinned(deltas[0].reshape(-1)))
    b.update(deltas[0].reshape(-1))
    ea, _ = geam.energy_gradient(None, None, a, prec, out=g_pin)
    eb, _ = geam.energy_gradient(None, None, b, prec, out=g_page)
    assert ea == eb and np.array_equal(g_page, g_pin)
