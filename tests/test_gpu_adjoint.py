"""Adjoint of the Q-atom energies: dE_s/d(qcrg, qA, qB) from the GPU kernel.

Config 4 as specified: 30 Q atoms in 4 states, every one of the 120 charges
and 240 code-1 LJ factors, 200 seeded snapshots (one batched window each),
against the FP64 reference gradient (oracle/adjoint.py, pinned to the C
oracle's energies and central differences) and against central differences
(h = 1e-5 relative) of the reference energies, within 1e-4 relative; the gap
gradient d(E2 - E1) as its own assertion; the arithmetic combination rule.
Also a system with soft pairs and electrostatic scaling against the C
oracle's central differences, and the mixed form against the FP64 form."""
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


def gpu_adjoint_snapshots(s, prec, xs):
    """Adjoint of every snapshot, one batched window each: [n][nq][S] x 3."""
    with NonbondedEngine(s, precision=prec, windows=len(xs)) as eng:
        eng.set_coordinates_dev(np.stack(xs))
        eng.make_pair_lists_dev(**CUT)
        return eng.q_adjoint_dev()


def close(g, ref, rel):
    scale = np.abs(ref).max()
    return bool(np.all(np.abs(g - ref) <= rel * np.maximum(np.abs(ref), 1e-3 * scale)))


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_config4_adjoint_200_snapshots(prec):
    from oracle.adjoint import QEnergyReference
    from q6_gb300.system import config_adjoint
    s = config_adjoint()
    rng = np.random.default_rng(4000)
    xs = [s.x + rng.normal(0.0, 0.05, s.x.shape) for _ in range(200)]
    dq, dA, dB = gpu_adjoint_snapshots(s, prec, xs)
    ref = QEnergyReference(s)
    assert dq.shape == (200, 30, 4) and dA.shape == (200, 30, 4)
    for n, x in enumerate(xs):
        _, gq, ga, gb = ref.evaluate(x)
        fq, fa, fb = ref.finite_differences(x, h=1e-5)
        for name, g, r, f in (("q", dq[n], gq, fq), ("A", dA[n], ga, fa), ("B", dB[n], gb, fb)):
            assert close(g, r, 1e-9), (prec, n, name)          # the FP64 reference gradient
            assert close(g, f, 1e-4), (prec, n, name)          # central differences
            # the gap E2 - E1: +dE2/dp for state-2 parameters, -dE1/dp for state 1
            gap = np.zeros_like(g)
            gap[:, 1], gap[:, 0] = g[:, 1], -g[:, 0]
            gap_fd = np.zeros_like(f)
            gap_fd[:, 1], gap_fd[:, 0] = f[:, 1], -f[:, 0]
            assert close(gap, gap_fd, 1e-4), (prec, n, name, "gap")


def test_arithmetic_rule_adjoint():
    from oracle.adjoint import QEnergyReference
    from q6_gb300.system import config_adjoint
    from tests.test_oracle_adjoint import arithmetic_variant
    s = arithmetic_variant(config_adjoint())
    rng = np.random.default_rng(4100)
    xs = [s.x + rng.normal(0.0, 0.05, s.x.shape) for _ in range(20)]
    ref = QEnergyReference(s)
    for prec in (PREC_FP64, PREC_MIXED):
        dq, dA, dB = gpu_adjoint_snapshots(s, prec, xs)
        for n, x in enumerate(xs):
            _, gq, ga, gb = ref.evaluate(x)
            fq, fa, fb = ref.finite_differences(x, h=1e-5)
            for name, g, r, f in (("q", dq[n], gq, fq), ("A", dA[n], ga, fa), ("B", dB[n], gb, fb)):
                assert close(g, r, 1e-9), (prec, n, name)
                assert close(g, f, 1e-4), (prec, n, name)


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
    """Both forms recompute the pair terms in FP64: equal to rounding."""
    a64 = gpu_adjoint(evb4, PREC_FP64)
    a32 = gpu_adjoint(evb4, PREC_MIXED)
    for g64, g32 in zip(a64, a32):
        assert close(g32, g64, 1e-10)
