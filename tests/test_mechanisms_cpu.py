"""The host logic of search.mechanisms (Master::saddle_2_mech, find.cpp:757-981, with recon_relax,
:77-125) and search.pathways (do_adj_min, :1014-1090) without a GPU: the device calls it makes (pathways, the batched Hessian eigenvalues and the
batched relaxations) are replaced by stand-ins returning chosen values, so each of the reference's
branches is reached on purpose."""
import numpy as np
import pytest

from openfly_gb300 import search as S

N = 4  # atoms; atom 0 moves, the others are fixed


def _state(shift):
    x = np.zeros((N, 3))
    x[:, 0] = np.arange(N) * 3.0
    x[0, 1] = shift
    return x


class FakeBatch:
    """Stands in for search.Batch: every minimisation ends at `fwd`, every dimer at `sp`."""

    plan: dict = {}

    def __init__(self, eam, reqs, **kw):
        self.reqs = reqs

    def run(self, tuning=None):
        pass

    def results(self, positions=True):
        res, pos = [], []
        for r in self.reqs:
            key = "min" if r.mode == S.MINIMISE else "sp"
            x, e, code = self.plan[key]
            res.append(dict(status=0, exit_code=code, energy=e, steps=1, grad_calls=1, curvature=0.0))
            pos.append(x.copy())
        return res, pos, [np.zeros((N, 3)) for _ in self.reqs]


def _setup(monkeypatch, path, freq, min_freq=None, plan=None):
    monkeypatch.setattr(S, "pathways", lambda *a, **k: [path])
    monkeypatch.setattr(S, "hessian_eigenvalues_batch",
                        lambda eam, systems, masses=None, workers=8:
                        [np.asarray(min_freq if s.pos is MINIMUM else freq, float) for s in systems])
    FakeBatch.plan = plan or {}
    monkeypatch.setattr(S, "Batch", FakeBatch)


MINIMUM = _state(0.0)
REV, SP, FWD = _state(0.0), _state(0.6), _state(1.2)
FROZEN = np.array([0, 1, 1, 1], np.uint8)  # 3 frozen atoms: 9 zero modes at the minimum


def _saddle():
    ax = np.zeros((N, 3))
    ax[0, 1] = 2.0
    return S.Search(SP, np.zeros(N, np.uint32), FROZEN, np.full(3, 20.0), np.zeros(3, np.int32), axis=ax)


def _path(**kw):
    p = dict(rev=REV, sp=SP, fwd=FWD, E_rev=-10.0, E_sp=-9.5, E_fwd=-9.9)
    p.update(kw)
    return p


GOOD_SP = np.array([-1.0] + [0.0] * 9 + [2.0, 3.0])  # one negative mode, 9 zeros, two positive
GOOD_MIN = np.array([0.0] * 9 + [1.0, 2.0, 4.0])


def _run(**kw):
    return S.mechanisms(None, [_saddle()], [MINIMUM], [np.array([0, 1])], **kw)[0]


def test_mechanism_built_with_prefactor(monkeypatch):
    _setup(monkeypatch, _path(), GOOD_SP, GOOD_MIN, {"min": (FWD, -9.9, 0), "sp": (SP, -9.5, 0)})
    m = _run()
    assert m["barrier"] == pytest.approx(0.5) and m["delta"] == pytest.approx(0.1)
    assert np.allclose(m["delta_sp"], (SP - REV)[[0, 1]]) and np.allclose(m["delta_fwd"], (FWD - REV)[[0, 1]])
    assert np.allclose(m["axis"], [[0, 1, 0], [0, 0, 0]])  # normalised on the geometry's atoms
    assert m["kinetic_pre"] == pytest.approx(np.log(2.0) + np.log(3.0))
    hz = np.sqrt(np.exp(np.log(8.0) - m["kinetic_pre"]) / (2 * np.pi * S.AMU_KG))  # find.cpp:286-292
    assert m["prefactor_hz"] == pytest.approx(hz)
    assert not m["poison_sp"] and not m["poison_fwd"]


@pytest.mark.parametrize("change", [dict(rev=_state(0.2)),       # rev > basin_tol from the minimum
                                    dict(fwd=_state(0.01)),      # fwd within basin_tol of rev
                                    dict(sp=_state(0.01))])      # saddle within stationary_tol of rev
def test_pathway_checks_reject(monkeypatch, change):
    _setup(monkeypatch, _path(**change), GOOD_SP, GOOD_MIN)
    assert _run() is None


def test_second_order_saddle_is_dropped(monkeypatch):
    freq = GOOD_SP.copy()
    freq[1] = -0.5
    _setup(monkeypatch, _path(), np.sort(freq), GOOD_MIN)
    assert _run() is None


def test_reference_errors(monkeypatch):
    _setup(monkeypatch, _path(E_sp=-10.5), GOOD_SP, GOOD_MIN)
    with pytest.raises(RuntimeError, match="Bad internal state"):
        _run()
    _setup(monkeypatch, _path(), np.abs(GOOD_SP), GOOD_MIN)
    with pytest.raises(RuntimeError, match="minimum mode"):
        _run()
    freq = GOOD_SP.copy()
    freq[2] = 0.5  # one zero mode too few
    _setup(monkeypatch, _path(), np.sort(freq), GOOD_MIN)
    with pytest.raises(RuntimeError, match="zero modes"):
        _run()


def test_poison_verdicts(monkeypatch):
    # the relaxed final state lands elsewhere (and its barrier is >= 0.5 eV, so no error is raised)
    far = _state(1.2)
    far[0, 1] += 0.2
    _setup(monkeypatch, _path(), GOOD_SP, GOOD_MIN, {"min": (far, -9.9, 0), "sp": (SP, -9.5 + 0.02, 0)})
    m = _run()
    assert m["poison_fwd"] and m["poison_sp"]  # 0.2 A > capture_r_tol; 0.02 eV > capture_E_tol
    # a failed relaxation poisons too
    _setup(monkeypatch, _path(), GOOD_SP, GOOD_MIN, {"min": (FWD, -9.9, 1), "sp": (SP, -9.5, 0)})
    m = _run()
    assert m["poison_fwd"] and m["err_fwd"] is None and not m["poison_sp"]


def test_poisoned_low_barrier_raises(monkeypatch):
    far = _state(1.2)
    far[0, 1] += 0.2
    _setup(monkeypatch, _path(E_sp=-9.8), GOOD_SP, GOOD_MIN, {"min": (far, -9.9, 0), "sp": (SP, -9.8, 0)})
    with pytest.raises(RuntimeError, match="poisoned"):
        _run()


class FakeRelax:
    """Stands in for search.Batch inside pathways: the + nudged relaxation ends at `plus`, the - nudged
    one at `minus` (plus a uniform drift), and the zero-step energy batch reports e["sp"]."""

    plus = minus = None
    drift = np.zeros(3)
    e = dict(plus=-9.9, minus=-10.0, sp=-9.5)
    code = 0

    def __init__(self, eam, reqs, lbfgs=None, **kw):
        self.reqs, self.energy_only = reqs, lbfgs is not None and lbfgs.iter_max == 0

    def run(self, tuning=None):
        pass

    def results(self, positions=True):
        if self.energy_only:
            return [dict(status=0, exit_code=0, energy=self.e["sp"])] * len(self.reqs), None, None
        res, pos = [], []
        for k in range(len(self.reqs)):
            which = "plus" if k % 2 == 0 else "minus"
            res.append(dict(status=0, exit_code=self.code, energy=self.e[which]))
            pos.append(getattr(self, which) + self.drift)
        return res, pos, [None] * len(self.reqs)


def _paths(monkeypatch, plus, minus, drift=(0.0, 0.0, 0.0), centre=0, code=0):
    FakeRelax.plus, FakeRelax.minus, FakeRelax.drift, FakeRelax.code = plus, minus, np.asarray(drift), code
    monkeypatch.setattr(S, "Batch", FakeRelax)
    return S.pathways(None, [_saddle()], [MINIMUM], [centre])[0]


def test_pathways_assigns_rev_and_removes_drift(monkeypatch):
    # find.cpp:1054-1075: the relaxed state nearer the initial minimum is rev; rev's centroid drift from the
    # minimum is removed from all three states
    p = _paths(monkeypatch, plus=FWD, minus=REV, drift=(0.05, -0.02, 0.01))
    assert np.allclose(p["rev"], REV) and np.allclose(p["fwd"], FWD)
    assert np.allclose(p["sp"], SP - np.array([0.05, -0.02, 0.01]))
    assert (p["E_rev"], p["E_fwd"], p["E_sp"]) == (-10.0, -9.9, -9.5) and p["barrier"] == pytest.approx(0.5)
    q = _paths(monkeypatch, plus=REV, minus=FWD)  # the other way round: still rev = the nearer one
    assert np.allclose(q["rev"], REV) and q["E_rev"] == -9.9


def test_pathways_centre_and_failure(monkeypatch):
    # find.cpp:1082-1087: the atom moving most between rev and fwd must be the centre (atom 0 here)
    assert _paths(monkeypatch, plus=FWD, minus=REV, centre=1) is None
    assert _paths(monkeypatch, plus=FWD, minus=REV, centre=0) is not None
    # a relaxation that does not converge gives no pathway (find.cpp:1038-1050)
    assert _paths(monkeypatch, plus=FWD, minus=REV, code=1) is None
