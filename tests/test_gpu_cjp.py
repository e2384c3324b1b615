"""GPU against the CPU oracle on a real topology: the reference's 2cjp FEP
inputs (tests/exclude_tests/inputs: a protein and its ligand in a 20 A
sphere, 5,622 atoms, 1,167 charge groups, 1,875 excluded atoms, 40 Q atoms in
2 states with FEP atom types and two soft pairs; the 20-atom ligand group is
all Q atoms, larger than the rows' 15-atom groups).  At the topology
coordinates, cut-offs 10 A / LRF on, the FP64 form within 1e-6 kcal/mol per
term (1e-9 relative above 1,000) and 1e-6 relative per gradient component,
the mixed form within 1e-3 relative and 2e-3 on the gradient; every pair
list equal to the oracle's as a set; three lambda windows batched equal to
single contexts bit for bit."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from tests.golden.cjp import load_cjp
from tests.test_gpu_configs import assert_lists_equal_as_sets, batched_vs_single, fp64_bar, grad_ok

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.fixture(scope="module")
def cjp():
    s = load_cjp()
    o = Oracle(s, use_lrf=True)
    ref = o.evaluate(s.x, [0.3, 0.7], cut=CUT)
    o.make_pair_lists(s.x, **CUT)
    return s, o, ref


@pytest.mark.parametrize("prec,tol,gtol", [(PREC_FP64, 1e-6, 1e-6), (PREC_MIXED, 1e-3, 2e-3)])
def test_cjp_matches_oracle(cjp, prec, tol, gtol):
    s, o, (d0, E0, EQ0, _) = cjp
    with NonbondedEngine(s, precision=prec, use_lrf=True) as eng:
        d, E, EQ, _ = eng.evaluate(s.x, [0.3, 0.7], cut=CUT)
        assert_lists_equal_as_sets(eng, o, s.natom, ("2cjp", prec))
    for k in E0:
        bar = fp64_bar(E0[k]) if prec == PREC_FP64 else tol * max(1.0, abs(E0[k]))
        assert abs(E[k] - E0[k]) <= bar, (prec, k, E[k], E0[k])
    qbar = np.maximum(fp64_bar(1.0), 1e-9 * np.abs(EQ0)) if prec == PREC_FP64 else tol * np.maximum(1.0, np.abs(EQ0))
    assert np.all(np.abs(EQ - EQ0) <= qbar), (prec, EQ, EQ0)
    assert grad_ok(d, d0, gtol), prec


def test_cjp_lambda_windows_batched_equal_single():
    s = load_cjp()
    batched_vs_single(s, CUT, [[1.0, 0.0], [0.5, 0.5], [0.0, 1.0]], check_windows=(0, 2))
