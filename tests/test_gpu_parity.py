"""GPU parity: the CUDA engine against the CPU FP64 oracle on the same inputs.

Plain FP64 form: pair lists identical as sets, every energy term within
1e-6 kcal/mol, gradients within 1e-6 relative (|dd_i| <= 1e-6 max(|d_i|,
median |d|)).  Mixed form: same lists; energies within 1e-3 relative and
gradients within 2e-3 of the same norm (FP32 pair arithmetic); results are
bit-identical between runs (fixed-point accumulation).
"""
import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.qnb import (LIST_PP, LIST_PP14, LIST_PW, LIST_QP, LIST_QW, LIST_WW, PREC_FP64,
                          PREC_MIXED, NonbondedEngine)
from q6_gb300.system import default_solvent_params, make_system

pytestmark = pytest.mark.gpu

CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
KINDS = {LIST_PP: "pp", LIST_PW: "pw", LIST_WW: "ww", LIST_QP: "qp", LIST_QW: "qw", LIST_PP14: "pp14"}
UNORDERED = {LIST_PP, LIST_PP14, LIST_WW}


def systems():
    return {
        "droplet": make_system(R=15.0, n_solute=60, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2,
                               seed=101),
        "excl_soft": make_system(R=13.0, n_solute=80, group_sizes=(3, 6), ntypes=8, nq=8, nstates=3,
                                 seed=202, excl_radius=11.0, soft_pairs=[(0, 5), (2, 7)],
                                 el_scale=[((1, 6), (0.5, 0.7, 0.9))]),
        "tiny": make_system(R=6.0, n_solute=9, nq=2, nstates=1, seed=303),
    }


SYS = systems()


def pairset(i, j, kind):
    if kind in UNORDERED:
        a, b = np.minimum(i, j), np.maximum(i, j)
    else:
        a, b = i, j
    return set(zip(a.tolist(), b.tolist()))


def grad_ok(d, d0, rel):
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    return np.all(np.abs(d - d0) <= rel * scale + 1e-9)


@pytest.mark.parametrize("name", list(SYS))
@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_pair_lists_match_as_sets(name, prec):
    s = SYS[name]
    o = Oracle(s)
    o.make_pair_lists(s.x, **CUT)
    with NonbondedEngine(s, precision=prec) as eng:
        eng.make_pair_lists(s.x, **CUT)
        for kind, label in KINDS.items():
            n0 = o.list_size(kind)
            assert eng.list_size(kind) == n0, (label, eng.list_size(kind), n0)
            gi, gj = eng.export_pairs(kind)
            ri, rj = o.export_pairs(kind)
            assert pairset(gi, gj, kind) == pairset(ri, rj, kind), label


@pytest.mark.parametrize("name", list(SYS))
def test_fp64_energies_and_gradients(name):
    s = SYS[name]
    lam = [1.0 / s.nstates] * s.nstates
    sp = default_solvent_params(s)
    o = Oracle(s)
    o.set_solvent_params(sp)
    d0, E0, EQ0, R0 = o.evaluate(s.x, lam, cut=CUT, solvent=sp, Tfree=300.0)
    with NonbondedEngine(s, precision=PREC_FP64) as eng:
        eng.set_solvent_params(sp)
        d, E, EQ, R = eng.evaluate(s.x, lam, cut=CUT, solvent=sp, Tfree=300.0)
    for k in E0:
        assert abs(E[k] - E0[k]) <= 1e-6, (k, E[k], E0[k])
    assert np.all(np.abs(EQ - EQ0) <= 1e-6), (EQ, EQ0)
    assert abs(R[0] - R0[0]) <= 1e-6 and abs(R[1] - R0[1]) <= 1e-6, (R, R0)
    assert grad_ok(d, d0, 1e-6)


@pytest.mark.parametrize("name", list(SYS))
def test_lrf_records_match(name):
    s = SYS[name]
    o = Oracle(s)
    o.make_pair_lists(s.x, **CUT)
    L0 = o.lrf()
    # mixed form: FP32 terms, sums folded into double-float accumulators
    # every few source groups (measured within 7e-6 of each coefficient's scale)
    for prec, rel in ((PREC_FP64, 1e-10), (PREC_MIXED, 2e-5)):
        with NonbondedEngine(s, precision=prec) as eng:
            eng.make_pair_lists(s.x, **CUT)
            L = eng.lrf()
        scale = np.abs(L0).max(0) + 1e-12
        assert np.all(np.abs(L - L0) <= rel * scale), prec


@pytest.mark.parametrize("name", list(SYS))
def test_mixed_energies_and_gradients(name):
    s = SYS[name]
    lam = [1.0 / s.nstates] * s.nstates
    sp = default_solvent_params(s)
    o = Oracle(s)
    o.set_solvent_params(sp)
    d0, E0, EQ0, R0 = o.evaluate(s.x, lam, cut=CUT, solvent=sp)
    with NonbondedEngine(s, precision=PREC_MIXED) as eng:
        eng.set_solvent_params(sp)
        d, E, EQ, R = eng.evaluate(s.x, lam, cut=CUT, solvent=sp)
    for k in E0:
        assert abs(E[k] - E0[k]) <= 1e-3 * max(1.0, abs(E0[k])), (k, E[k], E0[k])
    assert np.allclose(EQ, EQ0, rtol=1e-3, atol=1e-3)
    assert grad_ok(d, d0, 2e-3)


def test_mixed_is_bit_deterministic():
    s = SYS["droplet"]
    outs = []
    for _ in range(2):
        with NonbondedEngine(s, precision=PREC_MIXED) as eng:
            d, E, EQ, _ = eng.evaluate(s.x, [0.5, 0.5], cut=CUT)
            outs.append((d.copy(), np.array(list(E.values())), EQ.copy()))
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
    assert np.array_equal(outs[0][2], outs[1][2])


def test_qp_qw_lists_kept_after_first_build():
    """nbqplist/nbqwlist return early once built when Rcq^2 > rexcl_o^2."""
    s = SYS["droplet"]
    with NonbondedEngine(s, precision=PREC_FP64) as eng:
        eng.make_pair_lists(s.x, **CUT)
        n = eng.list_size(LIST_QW)
        x2 = s.x * 1.5   # push waters out; the Q lists must not change
        eng.make_pair_lists(x2, **CUT)
        assert eng.list_size(LIST_QW) == n


def test_md_false_runs_only_q_terms():
    s = SYS["droplet"]
    o = Oracle(s)
    o.set_lambda([0.5, 0.5])
    o.make_pair_lists(s.x, **CUT)
    d0, E0, EQ0 = o.pot_energy_nonbonds(s.x, md=False)
    with NonbondedEngine(s, precision=PREC_FP64) as eng:
        eng.set_lambda([0.5, 0.5])
        eng.make_pair_lists(s.x, **CUT)
        d, E, EQ = eng.pot_energy_nonbonds(s.x, md=False)
    assert all(v == 0.0 for v in E.values())
    assert np.all(np.abs(EQ - EQ0) <= 1e-6)
    assert grad_ok(d, d0, 1e-6)


def test_watpol_running_average_state():
    s = SYS["droplet"]
    sp = default_solvent_params(s, itdis=2.0)
    o = Oracle(s)
    o.set_solvent_params(sp)
    with NonbondedEngine(s, precision=PREC_FP64) as eng:
        eng.set_solvent_params(sp)
        for istep in range(5):
            x = s.x + 0.01 * istep
            d0 = np.zeros_like(x)
            d = np.zeros_like(x)
            e0 = o.watpol(x, d0, istep)
            e = eng.watpol(x, d, istep)
            assert abs(e - e0) <= 1e-6
            assert grad_ok(d, d0, 1e-6)
        a0 = o.watpol_state()
        a = eng.watpol_state()
    for u, v in zip(a, a0):
        assert np.allclose(u, v, rtol=1e-9, atol=1e-12)
