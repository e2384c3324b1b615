"""Adjoint of the Q-atom energies: dE_s/d(qcrg, qA, qB) from the GPU kernel
against central finite differences of the FP64 oracle's energies (h = 1e-5
relative), and the mixed-form adjoint against the FP64-form adjoint."""
import copy

import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.system import make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


def oracle_state_energy(s, st):
    o = Oracle(s)
    o.set_lambda([1.0] * s.nstates)
    o.make_pair_lists(s.x, **CUT)
    d, E, EQ = o.pot_energy_nonbonds(s.x)
    d, EQ = o.nonbond_qq(s.x, d, EQ)
    o.close()
    return float(EQ[st].sum())


def gpu_adjoint(s, prec):
    with NonbondedEngine(s, precision=prec) as eng:
        eng.set_coordinates_dev(s.x[None])
        eng.make_pair_lists_dev(**CUT)
        dq, dA, dB = eng.q_adjoint_dev()
    return dq[0], dA[0], dB[0]


@pytest.fixture(scope="module")
def evb4():
    # 4-state EVB-like system: many Q atoms, log-normal Q LJ factors per state
    return make_system(R=11.0, n_solute=40, group_sizes=(3, 5), ntypes=12, nq=16, nstates=4, q_sigma=0.4,
                       lognormal_q=True, seed=4242, soft_pairs=[(1, 9)], el_scale=[((2, 11), (0.5, 0.6, 0.7, 0.8))])


def test_adjoint_matches_finite_differences(evb4):
    s = evb4
    dq, dA, dB = gpu_adjoint(s, PREC_FP64)
    rng = np.random.default_rng(1)
    picks = [(int(rng.integers(s.nqat)), int(rng.integers(s.nstates))) for _ in range(6)]
    for iq, st in picks:
        # charge (scaled)
        h = 1e-5 * max(1.0, abs(s.qcrg[iq, st]))
        sp, sm = copy.deepcopy(s), copy.deepcopy(s)
        sp.qcrg = s.qcrg.copy(); sp.qcrg[iq, st] += h
        sm.qcrg = s.qcrg.copy(); sm.qcrg[iq, st] -= h
        fd = (oracle_state_energy(sp, st) - oracle_state_energy(sm, st)) / (2 * h)
        assert abs(fd - dq[iq, st]) <= 1e-4 * max(1.0, abs(fd)), ("q", iq, st, fd, dq[iq, st])
        # code-1 LJ factors of the Q type used by (iq, st)
        t = int(s.qiac[iq, st])
        for arr, g, name in ((s.qavdw, dA, "A"), (s.qbvdw, dB, "B")):
            h = 1e-5 * max(1.0, abs(arr[t, 0]))
            sp, sm = copy.deepcopy(s), copy.deepcopy(s)
            pa, ma = arr.copy(), arr.copy()
            pa[t, 0] += h
            ma[t, 0] -= h
            if name == "A":
                sp.qavdw, sm.qavdw = pa, ma
            else:
                sp.qbvdw, sm.qbvdw = pa, ma
            fd = (oracle_state_energy(sp, st) - oracle_state_energy(sm, st)) / (2 * h)
            assert abs(fd - g[iq, st]) <= 1e-4 * max(1e-3, abs(fd)), (name, iq, st, fd, g[iq, st])


def test_mixed_adjoint_matches_fp64_adjoint(evb4):
    a64 = gpu_adjoint(evb4, PREC_FP64)
    a32 = gpu_adjoint(evb4, PREC_MIXED)
    for g64, g32 in zip(a64, a32):
        scale = np.abs(g64).max()
        assert np.all(np.abs(g32 - g64) <= 1e-3 * scale)
