"""nonbond_solvent_internal on the GPU (src/nonbondene.f90:6082-6154)
against the oracle: a synthetic intra-molecular list on the SPC droplet
(the list comes from q6_gb300.solvent for solvents with torsions; SPC has
none, so the pairs here are set directly), both forms, host and device
paths."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.system import config_small, default_solvent_params

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
PAIRS = np.array([[0, 1], [1, 0], [1, 2], [2, 0]], dtype=np.int32)
A = np.array([300.0, 0.0, 55.0, 12.0])
B = np.array([20.0, 0.0, 3.0, 1.5])
EL = np.array([0.4, -0.2, 0.15, 0.05])


def grad_ok(d, d0, rel):
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    return bool(np.all(np.abs(d - d0) <= rel * scale + 1e-9))


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_solvent_internal_vs_oracle(prec):
    s = config_small()
    sp = default_solvent_params(s)
    o = Oracle(s)
    o.set_solvent_params(sp)
    o.set_solvent_internal(PAIRS, A, B, EL)
    d0, E0, EQ0, _ = o.evaluate(s.x, [0.5, 0.5], cut=CUT, solvent=sp)
    tol, gtol = (1e-6, 1e-6) if prec == PREC_FP64 else (1e-3, 2e-3)
    with NonbondedEngine(s, precision=prec) as e:
        e.set_solvent_params(sp)
        e.set_solvent_internal(PAIRS, A, B, EL)
        d, E, EQ, _ = e.evaluate(s.x, [0.5, 0.5], cut=CUT, solvent=sp)
    for k in ("ww_el", "ww_vdw"):
        bar = tol if prec == PREC_FP64 else tol * max(1.0, abs(E0[k]))
        assert abs(E[k] - E0[k]) <= bar, (k, E[k], E0[k])
    assert grad_ok(d, d0, gtol)


def test_solvent_internal_device_path_and_removal():
    s = config_small()
    sp = default_solvent_params(s)
    with NonbondedEngine(s, precision=PREC_MIXED, windows=2) as e:
        e.set_solvent_params(sp)
        e.set_lambda([0.5, 0.5], window=0)
        e.set_lambda([0.5, 0.5], window=1)
        e.set_coordinates_dev(np.stack([s.x, s.x]))
        e.make_pair_lists_dev(**CUT)
        E_off, _, _ = e.compute_dev(sync=True)
        e.gradient_dev()
        e.set_solvent_internal(PAIRS, A, B, EL)     # recaptures the step graph
        E_on, _, _ = e.compute_dev(sync=True)
        e.gradient_dev()
        e.set_solvent_internal([], [], [], [])
        E_off2, _, _ = e.compute_dev(sync=True)
    o = Oracle(s)
    o.make_pair_lists(s.x, **CUT)
    _, Ea, _ = o.pot_energy_nonbonds(s.x)
    o.set_solvent_internal(PAIRS, A, B, EL)
    _, Eb, _ = o.pot_energy_nonbonds(s.x)
    for w in range(2):
        assert E_off[w] == E_off2[w]
        for k in ("ww_el", "ww_vdw"):
            want = Eb[k] - Ea[k]
            assert abs((E_on[w][k] - E_off[w][k]) - want) <= 1e-3 * max(1.0, abs(want)), (w, k)
