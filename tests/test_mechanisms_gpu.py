"""Master::saddle_2_mech on the device (search.mechanisms: do_adj_min, the pathway checks, energies, the
mechanism, the Hessian prefactor and recon_relax, all relaxations batched) against the oracle's
restatement (oracle.mechanism) on saddles of binary64 cluster searches."""
import numpy as np
import pytest

from openfly_gb300 import search as S
from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu

BARRIER_EV = 1e-5     # barrier and delta of the same pathway
DELTA_A = 1e-3        # displacements of the geometry's atoms
PRE_ABS = 1e-3        # kinetic_pre, a sum of ~100-300 log eigenvalues
SHAPE = S.Tuning(4, 128, 2, 0)  # a fixed launch shape: results must not depend on the autotuner's timing


@pytest.fixture(scope="module")
def saddles(gpu, geam):
    # As Master does: relax each cluster to its minimum, perturb around the centre (Master::perturb) and
    # climb from there (binary64 throughout, so the device and the oracle follow the same pathways).
    clusters = W.search_clusters(n=24, seed=11)
    lb = S.LBFGSOptions.defaults(f2norm=1e-6)
    relax = S.Batch(geam, [S.from_cluster(c, mode=S.MINIMISE) for c in clusters], precision=gpu.FP64, lbfgs=lb)
    relax.run(SHAPE)
    _, minima, _ = relax.results()
    rng = np.random.default_rng(5)
    starts = []
    for c, x in zip(clusters, minima):
        s = c.sys
        sysm = W.System(x, s.types, s.frozen, s.extents, s.periodic)
        p, a = W.perturb(sysm, c.centre, rng)
        starts.append(S.Search(p, s.types, s.frozen, s.extents, s.periodic, axis=a, in_min=x))
    opt = S.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-5, max_steps=1000)
    b = S.Batch(geam, starts, precision=gpu.FP64, dimer=opt)
    b.run(SHAPE)
    res, pos, ax = b.results()
    found = [(c, x, S.Search(xs, c.sys.types, c.sys.frozen, c.sys.extents, c.sys.periodic, axis=a))
             for c, x, r, xs, a in zip(clusters, minima, res, pos, ax) if r["status"] == 0 and r["exit_code"] == 0]
    # Master keeps a mechanism only in the environment of the atom that moves most (find.cpp:1082-1087): each
    # saddle's geometry is centred on that atom of its pathway (the atom and its neighbours within 4 A)
    paths = S.pathways(geam, [s for *_, s in found], [x for _, x, _ in found], None, precision=gpu.FP64, lbfgs=lb,
                       tuning=SHAPE)
    out = []
    for (c, x, s), p in zip(found, paths):
        if p is None:
            continue
        mm = int(np.argmax(((p["rev"] - p["fwd"]) ** 2).sum(axis=1)))
        d = np.linalg.norm(x - x[mm], axis=1)
        geo = np.concatenate([[mm], np.flatnonzero((d < 4.0) & (np.arange(c.sys.n) != mm))])
        out.append((c, x, s, geo))
    assert len(out) >= 4
    return out, opt, lb


def test_mechanisms_match_oracle(gpu, oracle, geam, odata, saddles):
    found, opt, lb = saddles
    mechs = S.mechanisms(geam, [s for _, _, s, _ in found], [x for _, x, _, _ in found], [g for *_, g in found],
                         precision=gpu.FP64, dimer=opt, lbfgs=lb, tuning=SHAPE)
    odim = oracle.DimerOptions.defaults(n=6, rot_n=6, f2norm=1e-5, max_steps=1000)
    olb = oracle.LBFGSOptions.defaults(f2norm=1e-6)
    built = 0
    for (c, x, s, geo), m in zip(found, mechs):
        sy = c.sys
        masses = np.array([odata.mass(int(t)) for t in sy.types])
        zm = oracle.minimum_modes(odata, sy.extents, sy.periodic, x, sy.types, sy.frozen, masses)["zero_modes"]
        ref = oracle.mechanism(odata, odim, olb, sy.extents, sy.periodic, sy.types, sy.frozen, x, s.pos, s.axis,
                               geo, masses, zm)
        assert (m is None) == (ref is None)
        if m is None:
            continue
        built += 1
        assert abs(m["barrier"] - ref["barrier"]) < BARRIER_EV
        assert abs(m["delta"] - ref["delta"]) < BARRIER_EV
        assert np.abs(m["delta_sp"] - ref["delta_sp"]).max() < DELTA_A
        assert np.abs(m["delta_fwd"] - ref["delta_fwd"]).max() < DELTA_A
        assert np.abs(m["axis"] - ref["axis"]).max() < 1e-12
        assert abs(m["kinetic_pre"] - ref["kinetic_pre"]) < PRE_ABS
        # the prefactor in Hz (find.cpp:286-292) from the minimum's and the saddle's log products
        lp = oracle.minimum_modes(odata, sy.extents, sy.periodic, x, sy.types, sy.frozen, masses)["log_prod_eigen"]
        hz = np.sqrt(np.exp(lp - ref["kinetic_pre"]) / (2 * np.pi * 1.6605390666050e-27))
        assert abs(m["prefactor_hz"] / hz - 1) < 2 * PRE_ABS
        assert m["poison_sp"] == ref["poison_sp"] and m["poison_fwd"] == ref["poison_fwd"]
    assert built >= 2


def test_minimum_modes(gpu, oracle, geam, odata):
    # Master::calc_minima_hess on a relaxed cluster: 3 zero modes per frozen atom, the same log product
    c = W.search_clusters(n=1, seed=3)[0]
    s = c.sys
    _, x = S.minimise_system(geam, S.Search(s.pos, s.types, s.frozen, s.extents, s.periodic, mode=S.MINIMISE),
                             gpu.FP64, lbfgs=S.LBFGSOptions.defaults(f2norm=1e-8))
    got = S.minimum_modes(geam, [S.Search(x, s.types, s.frozen, s.extents, s.periodic)])[0]
    assert got["zero_modes"] == 3 * int(s.frozen.sum())
    masses = np.array([odata.mass(int(t)) for t in s.types])
    ref = oracle.minimum_modes(odata, s.extents, s.periodic, x, s.types, s.frozen, masses)
    assert ref["zero_modes"] == got["zero_modes"]
    assert abs(got["log_prod_eigen"] - ref["log_prod_eigen"]) < 1e-8 * max(1.0, abs(ref["log_prod_eigen"]))
