"""Master's random stream and find_batch's host logic, on the CPU (no GPU calls).

* xoshiro256** (utility/random.hpp:42-162): the library's stream equals the oracle's and the values the
  published definition gives for seed {1, 2, 3, 4};
* std::normal_distribution as libstdc++ draws it (Marsaglia's polar method with a cached second value):
  the library's restatement equals the oracle's calls into libstdc++ itself, bit for bit;
* Master::find_batch (find.cpp:684-755) over stand-ins for the device calls: a retry's perturbation is
  drawn right after the failed one and the searches after it are perturbed again from there, as on one
  reference thread; more than three consecutive out-of-bounds attempts raise; only successes without a
  mechanism are cached.
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def S(fly):
    from openfly_gb300 import search

    return search


def test_xoshiro_known_values_and_oracle(S, oracle):
    g = S.Xoshiro([1, 2, 3, 4])
    # first outputs from the definition: rotl(2 * 5, 7) * 9 = 11520, then rotl(0 * 5, 7) * 9 = 0
    assert g.next() == 11520
    assert g.next() == 0
    for seed in ([1, 2, 3, 4], [1, 3, 3, 4], [0x9E3779B97F4A7C15, 7, 0, 1 << 63]):
        g = S.Xoshiro(seed)
        ours = np.array([g.next() for _ in range(2000)], dtype=np.uint64)
        assert np.array_equal(ours, oracle.xoshiro(seed, 2000))


def test_xoshiro_rejects_zero_seed(S, fly):
    with pytest.raises(fly.FlyGPUError):
        S.Xoshiro([0, 0, 0, 0])


def test_long_jump_is_a_fixed_linear_map(S):
    # long_jump is linear over GF(2) in the state: jump(a ^ b) = jump(a) ^ jump(b)
    a, b = S.Xoshiro([1, 2, 3, 4]), S.Xoshiro([5, 6, 7, 8])
    c = S.Xoshiro([1 ^ 5, 2 ^ 6, 3 ^ 7, 4 ^ 8])
    for g in (a, b, c):
        g.long_jump()
    assert all(x ^ y == z for x, y, z in zip(a.state, b.state, c.state))
    assert a.state != (1, 2, 3, 4)


@pytest.mark.parametrize("mean,stddev", [(0.0, 1.0), (0.6, 0.2), (0.0, 0.37), (-2.5, 3.0)])
def test_normal_draws_equal_libstdcxx(S, oracle, mean, stddev):
    for seed in ([1, 3, 3, 4], [11, 0, 5, 99]):
        g = S.Xoshiro(seed)
        ours = g.normal(mean, stddev, 5001)  # odd count: the object ends with a cached value unused
        ref, st = oracle.normal_draws(seed, mean, stddev, 5001)
        assert np.array_equal(ours, ref)
        assert g.state == tuple(int(x) for x in st)


# ------------------------------------------------------------------ find_batch host logic


class _FakeBatch:
    """Stands in for search.Batch: a search 'fails' out of bounds when its start's first coordinate is in
    `oob`; otherwise it succeeds and returns its start as the saddle."""

    oob: set = set()
    runs: list = []

    def __init__(self, eam, searches, **kw):
        self.searches = searches
        _FakeBatch.runs.append(len(searches))

    def run(self, tuning=None):
        pass

    def results(self, positions=True):
        from openfly_gb300 import SPLINE_OOB

        res = []
        for s in self.searches:
            bad = float(np.asarray(s.pos)[0, 0]) in _FakeBatch.oob
            res.append(dict(status=SPLINE_OOB if bad else 0, exit_code=-4 if bad else 0, steps=1, grad_calls=1,
                            curvature=0.0, energy=0.0))
        return res, [np.asarray(s.pos) for s in self.searches], [np.asarray(s.axis) for s in self.searches]


def _fake_perturb(draws):
    """perturb stand-in: the start's first coordinate is the stream's next output (so a start names the
    draw it came from); records every draw."""

    def f(nl, centre, x0, frozen, g, stddev, r_pert):
        v = float(g.next() % 1000003)
        draws.append(v)
        p = np.array(x0, dtype=np.float64).reshape(-1, 3).copy()
        p[0, 0] = v
        return p, np.ones_like(p), stddev

    return f


def _setup_fakes(S, monkeypatch, mech_for=lambda k: None):
    draws: list = []
    monkeypatch.setattr(S, "perturb", _fake_perturb(draws))
    monkeypatch.setattr(S, "Batch", _FakeBatch)
    monkeypatch.setattr(S, "mechanisms", lambda eam, sads, mins, geos, **kw: [mech_for(s) for s in sads])
    _FakeBatch.runs = []
    return draws


def _minimum(S, n=4, frozen=1):
    fz = np.zeros(n, np.uint8)
    fz[-frozen:] = 1 if frozen else 0
    return S.Search(np.arange(3 * n, dtype=np.float64).reshape(-1, 3) + 100.0, np.zeros(n, np.uint32), fz,
                    np.full(3, 50.0), np.zeros(3, np.int32))


def test_find_batch_replays_the_stream_after_a_retry(S, monkeypatch):
    draws = _setup_fakes(S, monkeypatch)
    g = S.Xoshiro([1, 3, 3, 4])
    seq = [float(g.next() % 1000003) for _ in range(8)]
    _FakeBatch.oob = {seq[1]}  # search 1's first attempt fails: its retry takes draw 2, search 2 draw 3, ...
    prng = S.Xoshiro([1, 3, 3, 4])
    cache: list = []
    out = S.find_batch(None, 0, _minimum(S), 0, None, cache, 4, prng, geo=[0, 1])
    assert [o["retries"] for o in out] == [0, 1, 0, 0]
    assert [o["start"][0][0, 0] for o in out] == [seq[0], seq[2], seq[3], seq[4]]
    # the stream ends where a single reference thread's would: after five perturbations
    g = S.Xoshiro([1, 3, 3, 4])
    for _ in range(5):
        g.next()
    assert prng.state == g.state
    # speculative draws are discarded: searches 2 and 3 were perturbed twice, the batch ran twice
    assert draws == [seq[0], seq[1], seq[2], seq[3], seq[2], seq[3], seq[4]]
    assert _FakeBatch.runs == [4, 3]
    # every success without a mechanism is cached
    assert len(cache) == 4


def test_find_batch_raises_after_three_retries(S, monkeypatch):
    _setup_fakes(S, monkeypatch)
    g = S.Xoshiro([2, 3, 3, 4])
    seq = [float(g.next() % 1000003) for _ in range(8)]
    _FakeBatch.oob = set(seq[1:5])  # search 1: first attempt and three retries fail
    with pytest.raises(RuntimeError, match="Consecutive spline-out-of-bounds"):
        S.find_batch(None, 0, _minimum(S), 0, None, [], 3, S.Xoshiro([2, 3, 3, 4]), geo=[0])
    _FakeBatch.oob = set(seq[1:4])  # three failures, the third retry succeeds
    out = S.find_batch(None, 0, _minimum(S), 0, None, [], 3, S.Xoshiro([2, 3, 3, 4]), geo=[0])
    assert [o["retries"] for o in out] == [0, 3, 0]


def test_find_batch_caches_only_successes_without_mechanism(S, monkeypatch):
    _setup_fakes(S, monkeypatch, mech_for=lambda s: {"barrier": 1.0} if s.pos[0, 0] % 2 == 0 else None)
    _FakeBatch.oob = set()
    cache = [np.zeros((4, 3))]
    out = S.find_batch(None, 7, _minimum(S), 0, None, cache, 6, S.Xoshiro([5, 3, 3, 4]), geo=[0])
    no_mech = [o for o in out if o["mech"] is None]
    assert len(cache) == 1 + len(no_mech)
    for c, o in zip(cache[1:], no_mech):
        assert np.array_equal(c, o["pos"])


def test_find_batch_aligns_centroids_when_nothing_is_frozen(S, monkeypatch):
    _setup_fakes(S, monkeypatch)
    _FakeBatch.oob = set()
    m = _minimum(S, frozen=0)
    out = S.find_batch(None, 0, m, 0, None, [], 2, S.Xoshiro([1, 3, 3, 4]), geo=[0])
    for o in out:
        assert np.allclose(S.centroid(o["start"][0]), S.centroid(m.pos), atol=1e-12)
    out = S.find_batch(None, 0, _minimum(S, frozen=1), 0, None, [], 2, S.Xoshiro([1, 3, 3, 4]), geo=[0])
    assert not np.allclose(S.centroid(out[0]["start"][0]), S.centroid(m.pos))


def test_theta_tol_is_the_reference_schedule(S):
    assert S.theta_tol(0) == pytest.approx(np.pi / 6)
    assert S.theta_tol(10 ** 6) == pytest.approx(2.5 / 360 * 2 * np.pi)
