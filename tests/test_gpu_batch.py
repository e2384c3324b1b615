"""Batched windows: one context with several lambda windows gives, per
window, the results of a single-window context on the same inputs (FP64 within
1e-9 kcal/mol; mixed bit-identical, since its sums are exact fixed point)."""
import numpy as np
import pytest

from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.system import default_solvent_params, make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_batch_matches_single_windows(prec):
    s = make_system(R=14.0, n_solute=70, group_sizes=(3, 6), ntypes=8, nq=7, nstates=2, seed=909)
    sp = default_solvent_params(s)
    W = 3
    rng = np.random.default_rng(5)
    xs = np.stack([s.x + rng.normal(0, 0.02, s.x.shape) for _ in range(W)])
    lams = [[1.0, 0.0], [0.3, 0.7], [0.0, 1.0]]
    with NonbondedEngine(s, precision=prec, windows=W) as b:
        b.set_solvent_params(sp)
        for w in range(W):
            b.set_lambda(lams[w], window=w)
        b.set_coordinates_dev(xs)
        b.make_pair_lists_dev(**CUT)
        E, EQ, R = b.compute_dev(Tfree=300.0, istep=0, sync=True)
        D = b.gradient_dev()
    for w in range(W):
        with NonbondedEngine(s, precision=prec) as e:
            e.set_solvent_params(sp)
            e.set_lambda(lams[w])
            e.set_coordinates_dev(xs[w][None])
            e.make_pair_lists_dev(**CUT)
            E1, EQ1, R1 = e.compute_dev(Tfree=300.0, istep=0, sync=True)
            D1 = e.gradient_dev()
        tol = 1e-9 if prec == PREC_FP64 else 0.0
        for k in E1[0]:
            assert abs(E[w][k] - E1[0][k]) <= tol * max(1, abs(E1[0][k])), (w, k)
        assert np.all(np.abs(EQ[w] - EQ1[0]) <= tol * np.maximum(1, np.abs(EQ1[0])))
        assert np.all(np.abs(R[w] - R1[0]) <= tol * np.maximum(1, np.abs(R1[0])))
        scale = max(1.0, float(np.abs(D1).max()))
        assert np.abs(D[w] - D1[0]).max() <= tol * scale
