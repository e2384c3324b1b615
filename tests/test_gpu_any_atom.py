"""GPU parity in any-atom charge-group mode (topology switch-atom flag 0:
nbpplis2(_lrf), nbpwlis2(_lrf), nbqplis2, src/nonbondene.f90:950-1086,
1369-1516, 2137-2242, 2493-2618, 3408-3519) against the CPU oracle.

Tolerances are those of the switch-atom parity tests: lists identical as sets,
FP64 energies within 1e-6 kcal/mol and gradients within 1e-6 relative, LRF
records within 1e-10 (FP64) / 1e-3 (mixed) relative; mixed energies within
1e-3 relative."""
import dataclasses

import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.qnb import (LIST_PP, LIST_PP14, LIST_PW, LIST_QP, LIST_QW, LIST_WW, PREC_FP64,
                          PREC_MIXED, NonbondedEngine)
from q6_gb300.system import default_solvent_params, make_system

pytestmark = pytest.mark.gpu

CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
CUT_SHORT = dict(Rcq=8.0, RcLRF=11.0, Rcpp=6.0, Rcpw=6.0, Rcww=6.0)
KINDS = {LIST_PP: "pp", LIST_PW: "pw", LIST_WW: "ww", LIST_QP: "qp", LIST_QW: "qw", LIST_PP14: "pp14"}
UNORDERED = {LIST_PP, LIST_PP14, LIST_WW}


def any_atom(s):
    return dataclasses.replace(s, iuse_switch_atom=0)


SYS = {
    "droplet": any_atom(make_system(R=15.0, n_solute=60, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2,
                                    seed=101)),
    "excl": any_atom(make_system(R=14.0, n_solute=70, group_sizes=(3, 6), ntypes=6, nq=6, nstates=2,
                                 seed=606, excl_radius=12.5)),
    "big_groups": any_atom(make_system(R=18.0, n_solute=400, group_sizes=(5, 8), ntypes=8, nq=8,
                                       nstates=2, seed=707)),
}


def pairset(i, j, kind):
    if kind in UNORDERED:
        i, j = np.minimum(i, j), np.maximum(i, j)
    return set(zip(i.tolist(), j.tolist()))


def grad_ok(d, d0, rel):
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    return np.all(np.abs(d - d0) <= rel * scale + 1e-9)


@pytest.mark.parametrize("name", list(SYS))
@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
@pytest.mark.parametrize("cut", [CUT, CUT_SHORT], ids=["rc10", "rc6_lrf11"])
def test_any_atom_lists_match_as_sets(name, prec, cut):
    s = SYS[name]
    o = Oracle(s)
    o.make_pair_lists(s.x, **cut)
    with NonbondedEngine(s, precision=prec) as eng:
        eng.make_pair_lists(s.x, **cut)
        for kind, label in KINDS.items():
            assert eng.list_size(kind) == o.list_size(kind), (label, eng.list_size(kind), o.list_size(kind))
            assert pairset(*eng.export_pairs(kind), kind) == pairset(*o.export_pairs(kind), kind), label


@pytest.mark.parametrize("name", list(SYS))
@pytest.mark.parametrize("cut", [CUT, CUT_SHORT], ids=["rc10", "rc6_lrf11"])
def test_any_atom_lrf_records(name, cut):
    s = SYS[name]
    o = Oracle(s)
    o.make_pair_lists(s.x, **cut)
    L0 = o.lrf()
    for prec, rel in ((PREC_FP64, 1e-10), (PREC_MIXED, 1e-3)):
        with NonbondedEngine(s, precision=prec) as eng:
            eng.make_pair_lists(s.x, **cut)
            L = eng.lrf()
        scale = np.abs(L0).max(0) + 1e-12
        assert np.all(np.abs(L - L0) <= rel * scale), prec


@pytest.mark.parametrize("name", list(SYS))
@pytest.mark.parametrize("use_lrf", [True, False])
def test_any_atom_fp64_energies_and_gradients(name, use_lrf):
    s = SYS[name]
    lam = [0.5, 0.5]
    sp = default_solvent_params(s)
    o = Oracle(s, use_lrf=use_lrf)
    o.set_solvent_params(sp)
    d0, E0, EQ0, R0 = o.evaluate(s.x, lam, cut=CUT_SHORT, solvent=sp)
    with NonbondedEngine(s, precision=PREC_FP64, use_lrf=use_lrf) as eng:
        eng.set_solvent_params(sp)
        d, E, EQ, R = eng.evaluate(s.x, lam, cut=CUT_SHORT, solvent=sp)
    for k in E0:
        assert abs(E[k] - E0[k]) <= 1e-6, (k, E[k], E0[k])
    assert np.all(np.abs(EQ - EQ0) <= 1e-6)
    assert grad_ok(d, d0, 1e-6)


@pytest.mark.parametrize("name", list(SYS))
def test_any_atom_mixed_energies_and_gradients(name):
    s = SYS[name]
    lam = [0.5, 0.5]
    sp = default_solvent_params(s)
    o = Oracle(s)
    o.set_solvent_params(sp)
    d0, E0, EQ0, _ = o.evaluate(s.x, lam, cut=CUT, solvent=sp)
    with NonbondedEngine(s, precision=PREC_MIXED) as eng:
        eng.set_solvent_params(sp)
        d, E, EQ, _ = eng.evaluate(s.x, lam, cut=CUT, solvent=sp)
    for k in E0:
        assert abs(E[k] - E0[k]) <= 1e-3 * max(1.0, abs(E0[k])), (k, E[k], E0[k])
    assert np.allclose(EQ, EQ0, rtol=1e-3, atol=1e-3)
    assert grad_ok(d, d0, 2e-3)
