"""Whole-system LBFGS::minimise with every vector on the device (flygpu_minimise) vs the oracle's
LBFGS::minimise (src/minimise/LBFGS/lbfgs.cpp:29-115)."""
import numpy as np
import pytest

from openfly_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S(gpu):
    from openfly_gb300 import search

    return search


def _energy(O, odata, s, x):
    nl = O.List(s.extents, s.periodic, odata.r_cut)
    nl.rebuild(x, 1)
    return O.eam_energy(odata, nl, s.types)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_minimise_system_matches_oracle(gpu, oracle, odata, geam, S, precision):
    # the 431-atom vacancy cell (periodic, sigma 0.02 A) relaxed to |F| < 1e-4 eV/A
    O = oracle
    s = W.fe_vacancy_cell()
    prec = gpu.FP64 if precision == "fp64" else gpu.MIXED
    lopt = S.LBFGSOptions.defaults(f2norm=1e-4)
    olopt = O.LBFGSOptions.defaults(f2norm=1e-4)
    req = S.Search(s.pos, s.types, s.frozen, s.extents, s.periodic, mode=S.MINIMISE)
    r, x = S.minimise_system(geam, req, prec, lbfgs=lopt)
    failed, iters, xo, go = O.lbfgs_minimise(odata, olopt, s.extents, s.periodic, s.pos, s.types, s.frozen)
    assert r["status"] == 0 and r["exit_code"] == int(failed) == 0
    e_ref = _energy(O, odata, s, xo)
    assert abs(_energy(O, odata, s, x) - e_ref) < 1e-5  # the same minimum
    assert abs(r["energy"] - e_ref) < (1e-5 if precision == "fp64" else 1e-3)
    if precision == "fp64":
        assert abs(r["steps"] - iters) <= max(3, iters // 10)  # reduction order only


def test_minimise_system_with_frozen_atoms_and_hydrogen(gpu, oracle, odata, geam, S):
    # a cluster with a frozen shell and H: frozen atoms stay put, the rest relaxes to the oracle's minimum
    O = oracle
    cl = W.cluster(np.random.default_rng(12), 10.0, n_h=2, n_vac=1)
    s = cl.sys
    lopt = S.LBFGSOptions.defaults(f2norm=1e-4)
    olopt = O.LBFGSOptions.defaults(f2norm=1e-4)
    r, x = S.minimise_system(geam, S.Search(s.pos, s.types, s.frozen, s.extents, s.periodic, mode=S.MINIMISE),
                             gpu.FP64, lbfgs=lopt)
    failed, iters, xo, go = O.lbfgs_minimise(odata, olopt, s.extents, s.periodic, s.pos, s.types, s.frozen)
    assert r["exit_code"] == int(failed) == 0
    fz = s.frozen.astype(bool)
    assert np.array_equal(x[fz], s.pos[fz])
    assert np.abs(x - xo).max() < 1e-3
    assert abs(r["energy"] - _energy(O, odata, s, xo)) < 1e-5
