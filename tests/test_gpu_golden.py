"""The reference's own step-0 golden energies reproduced by the CUDA engine."""
import numpy as np
import pytest

from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from tests.golden.lig_w import load_lig_w
from tests.test_golden import _step0_coordinates

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_lig_w_step0_on_gpu(prec):
    s, g = load_lig_w()
    x = _step0_coordinates(s, g)
    with NonbondedEngine(s, precision=prec) as eng:
        d, E, EQ, _ = eng.evaluate(x, [1.0], cut=dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0))
    el = E["pp_el"] + E["ww_el"] + E["pw_el"]
    vdw = E["pp_vdw"] + E["ww_vdw"] + E["pw_vdw"]
    # the Q-atom line (the quantity free energies are built from) must print
    # the reference's strings in both forms
    assert f"{EQ[0, 2] + EQ[0, 4]:10.2f}" == f"{g['golden_qsurr_el']:10.2f}"
    assert f"{EQ[0, 3] + EQ[0, 5]:10.2f}" == f"{g['golden_qsurr_vdw']:10.2f}"
    if prec == PREC_FP64:
        assert f"{el:.2f}" == f"{g['golden_el']:.2f}"
        assert f"{vdw:.2f}" == f"{g['golden_vdw']:.2f}"
    else:
        # EL is a sum of ~7e5 cancelling water Coulomb terms: FP32 pair
        # arithmetic is allowed 0.05 kcal/mol on it (0.005 plus rounding on vdW)
        assert abs(el - g["golden_el"]) <= 0.05, el
        assert abs(vdw - g["golden_vdw"]) <= 0.01, vdw
