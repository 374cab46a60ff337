"""Spline construction (spline.cpp:27-103) and evaluation (spline.hpp:81-154): the reference's spline
cases (tests/utility/spline.cpp:27-82) on the oracle, and the library's host builder, which every
EAM table of the device goes through, bit-exact against the oracle. CPU only."""
import numpy as np
import pytest

from test_hessian import near


def test_constant_spline(oracle):
    # tests/utility/spline.cpp:27-36
    f, fp, fpp = oracle.spline_points([1.0, 1.0, 1.0, 1.0], 1.0, [0.0])[0]
    assert near(f, 1.0) and near(fp, 0.0) and near(fpp, 0.0)


def _cubic_tables(seed: int, count: int):
    rng = np.random.default_rng(seed)
    for _ in range(count):
        c = rng.uniform(-1.0, 1.0, 4)
        yield c, rng


def test_random_cubics(oracle):
    # tests/utility/spline.cpp:38-82: 100 random cubics tabulated at 100 points on [0, 1), checked at
    # 1000 points in [0.1, 0.9] with near(..., 1e-5, 0.01) on f, f' and f''
    dx = 1.0 / 100
    for c, rng in _cubic_tables(1334, 100):
        x0, x1, x2, x3 = c
        tab = [x0 * x ** 3 + x1 * x ** 2 + x2 * x + x3 for x in np.arange(100) * dx]
        xs = rng.uniform(0.1, 0.9, 1000)
        got = oracle.spline_points(tab, dx, xs)
        f = x0 * xs ** 3 + x1 * xs ** 2 + x2 * xs + x3
        fp = 3 * x0 * xs ** 2 + 2 * x1 * xs + x2
        fpp = 6 * x0 * xs + 2 * x1
        for k in range(xs.size):
            assert near(got[k, 0], f[k], 1e-5, 0.01)
            assert near(got[k, 1], fp[k], 1e-5, 0.01)
            assert near(got[k, 2], fpp[k], 1e-5, 0.01)


@pytest.mark.parametrize("n,dx", [(2, 1.0), (4, 1.0), (100, 0.01), (10001, 5.3e-4), (5000, 2e-3)])
def test_library_builder_bit_exact(fly, oracle, n, dx):
    rng = np.random.default_rng(n)
    y = np.cumsum(rng.normal(size=n)) * rng.uniform(0.1, 10.0)
    lib = fly.spline_build(y, dx)
    ref = oracle.spline_build(y, dx)
    assert lib.shape == (n + 4, 4)
    assert np.array_equal(lib, ref)


def test_library_builder_rejects_bad_input(fly):
    with pytest.raises(fly.FlyGPUError):
        fly.spline_build([1.0], 1.0)
    with pytest.raises(fly.FlyGPUError):
        fly.spline_build([1.0, 2.0], 0.0)
