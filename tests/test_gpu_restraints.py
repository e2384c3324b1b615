"""p_restrain on the GPU (qnb_set_restraints) against the oracle: sequence
restraints in all three modes, position, distance, angle and wall
restraints, state-dependent and not, energies within 1e-9 (both forms:
FP64 terms, the mixed form sums them in fixed point) and the gradient
within the suite's bars."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.md import MdSetup
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.restraints import Restraints
from q6_gb300.system import make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_restraints_on_gpu(prec):
    s = make_system(R=11.0, n_solute=30, group_sizes=(3, 5), ntypes=6, nq=4, nstates=2, seed=404)
    n, w0 = s.nat_solute, s.nat_solute
    r = Restraints(
        seq=[(0, 9, 2.0, 0, 0), (10, 19, 1.5, 1, 1), (20, 29, 1.0, 1, 2)],
        pos=[(3, -1, s.x[3] + 0.2, (5.0, 4.0, 3.0)), (7, 1, s.x[7] - 0.1, (2.0, 2.0, 2.0))],
        dist=[(0, n - 1, 3.0, 4.0, 10.0, 0), (2, 12, 1.0, 1.5, 7.0, -1)],
        ang=[(0, 1, 2, 100.0, 30.0, 1), (4, 5, 6, 120.0, 20.0, -1)],
        wall=[(w0, w0 + 60, 6.0, 15.0, 0.6, 0.5, 1)])
    lam = [0.3, 0.7]
    x = s.x + np.random.default_rng(8).normal(0, 0.1, s.x.shape)
    with NonbondedEngine(s, precision=prec) as e:
        e.set_lambda(lam)
        e.md_init(MdSetup())          # the masses the centre modes use
        e.set_restraints(r)
        e.set_coordinates_dev(x[None])
        e.make_pair_lists_dev(**CUT)
        e.compute_dev(sync=True)
        Er = e.restraint_energies()
        D = e.gradient_dev()
    o = Oracle(s)
    d0, _, _, _ = o.evaluate(x, lam, cut=CUT)
    d0, ep, eq = o.p_restrain(x, r, lam, d=d0)
    assert ep != 0.0 and np.all(eq != 0.0)
    assert Er[0, 4] == pytest.approx(ep, rel=1e-9, abs=1e-9)
    assert np.allclose(Er[0, 5:], eq, rtol=1e-9, atol=1e-9)
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    gtol = 1e-6 if prec == PREC_FP64 else 2e-3
    assert np.all(np.abs(D[0] - d0) <= gtol * scale + 1e-9)
