"""The launch-geometry autotuner: the mixed form's results are bit-identical
before and after tuning (they do not depend on the geometry), the watpol
running averages survive it, and the chosen values are among the candidates."""
import numpy as np
import pytest

from q6_gb300.qnb import PREC_FP64, PREC_MIXED, TUNE_NAMES, NonbondedEngine
from q6_gb300.system import default_solvent_params, lambdas_for_window, make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.mark.parametrize("prec", [PREC_MIXED, PREC_FP64])
def test_autotune_keeps_results(prec):
    s = make_system(R=16.0, n_solute=120, group_sizes=(3, 6), ntypes=8, nq=8, nstates=2, seed=6161)
    W = 4
    with NonbondedEngine(s, precision=prec, windows=W) as e:
        e.set_solvent_params(default_solvent_params(s, itdis=3.0))
        for w in range(W):
            e.set_lambda(lambdas_for_window(w / (W - 1), s.nstates), window=w)
        e.set_coordinates_dev(np.stack([s.x] * W))
        e.make_pair_lists_dev(**CUT)
        E0, EQ0, R0 = e.compute_dev(istep=1, sync=True)
        D0 = e.gradient_dev()
        ws0 = e.watpol_state()
        default = e.tuning()
        chosen = e.autotune(reps=2)
        assert set(chosen) == set(TUNE_NAMES)
        assert all(1 <= v <= 64 for v in chosen.values())
        assert e.tuning() == chosen
        ws1 = e.watpol_state()
        for a, b in zip(ws0, ws1):
            assert np.array_equal(a, b)
        assert np.all(e.gradient_dev() == 0.0)   # cleared by the tuner
        e.make_pair_lists_dev(**CUT)
        E1, EQ1, R1 = e.compute_dev(istep=1, sync=True)
        D1 = e.gradient_dev()
        e.set_tuning(default)
        assert e.tuning() == default
    if prec == PREC_MIXED:
        for w in range(W):
            assert E0[w] == E1[w]
        assert np.array_equal(EQ0, EQ1) and np.array_equal(D0, D1)
    else:
        for w in range(W):
            for k in E0[w]:
                assert abs(E0[w][k] - E1[w][k]) <= 1e-9 * max(1.0, abs(E0[w][k]))
        assert np.allclose(D0, D1, rtol=1e-12, atol=1e-9)
