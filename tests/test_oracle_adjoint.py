"""The FP64 reference of the Q-atom parameter gradients (oracle/adjoint.py).

Its per-state energies equal the C oracle's on seeded snapshots of the
config-4 system (30 Q atoms, 4 states, log-normal Q LJ factors) and on an
arithmetic-rule variant of it; its analytic gradients equal central
differences (h = 1e-5 relative) of the C oracle's energies for every one of
the 120 charges and 240 LJ factors, and those of the gap E2 - E1."""
import copy

import numpy as np
import pytest

from oracle.adjoint import QEnergyReference
from oracle.oracle import Oracle
from q6_gb300.system import config_adjoint

CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


def arithmetic_variant(s):
    """The same system under the arithmetic combination rule: each type's
    geometric factors a = sqrt(A_ii), b = sqrt(B_ii) become R* and sqrt(eps)
    with the same like-pair A and B (A = (2R)^12 e^2, B = 2 (2R)^6 e^2)."""
    def conv(a, b):
        a, b = np.asarray(a, float), np.asarray(b, float)
        ok = (a > 0) & (b > 0)
        R = np.where(ok, 0.5 * (2.0 * a * a / np.where(ok, b * b, 1.0)) ** (1.0 / 6.0), 0.0)
        e = np.where(ok, b * b / (2.0 * np.where(ok, a, 1.0)), 0.0)
        return R, e
    t = copy.deepcopy(s)
    t.avdw, t.bvdw = conv(s.avdw, s.bvdw)
    t.qavdw, t.qbvdw = conv(s.qavdw, s.qbvdw)
    t.ivdw_rule = 2
    return t


def oracle_q_energies(s, x):
    o = Oracle(s)
    o.set_lambda([1.0] * s.nstates)
    o.make_pair_lists(x, **CUT)
    d, E, EQ = o.pot_energy_nonbonds(x)
    d, EQ = o.nonbond_qq(x, d, EQ)
    o.close()
    return EQ.sum(1)


def snapshots(s, n, seed):
    rng = np.random.default_rng(seed)
    return [s.x + rng.normal(0.0, 0.05, s.x.shape) for _ in range(n)]


@pytest.fixture(scope="module")
def cfg4():
    return config_adjoint()


@pytest.mark.parametrize("rule", ["geometric", "arithmetic"])
def test_reference_energies_equal_the_oracle(cfg4, rule):
    s = cfg4 if rule == "geometric" else arithmetic_variant(cfg4)
    ref = QEnergyReference(s)
    for x in snapshots(s, 4, 7):
        E0 = oracle_q_energies(s, x)
        assert np.allclose(ref.energies(x), E0, rtol=1e-12, atol=1e-9), (rule, ref.energies(x), E0)


def test_reference_gradient_against_oracle_central_differences(cfg4):
    """All 30 x 4 charges and 30 x 4 x 2 code-1 LJ factors, h = 1e-5
    relative, one snapshot; the gap gradient d(E2 - E1)/dp is checked from
    the same differences (parameters of states 3 and 4 leave it unchanged)."""
    s = cfg4
    x = snapshots(s, 1, 11)[0]
    _, gq, ga, gb = QEnergyReference(s).evaluate(x)
    fds = {k: np.zeros((s.nqat, s.nstates, s.nstates)) for k in "qab"}   # [iq, param state, energy state]
    for iq in range(s.nqat):
        for st in range(s.nstates):
            for kind in "qab":
                t = int(s.qiac[iq, st])
                val = s.qcrg[iq, st] if kind == "q" else (s.qavdw[t, 0] if kind == "a" else s.qbvdw[t, 0])
                h = 1e-5 * max(1.0, abs(val))
                E = []
                for sign in (1.0, -1.0):
                    sp = copy.deepcopy(s)
                    if kind == "q":
                        sp.qcrg = s.qcrg.copy()
                        sp.qcrg[iq, st] += sign * h
                    elif kind == "a":
                        sp.qavdw = s.qavdw.copy()
                        sp.qavdw[t, 0] += sign * h
                    else:
                        sp.qbvdw = s.qbvdw.copy()
                        sp.qbvdw[t, 0] += sign * h
                    E.append(oracle_q_energies(sp, x))
                fds[kind][iq, st] = (E[0] - E[1]) / (2.0 * h)
    for kind, g in (("q", gq), ("a", ga), ("b", gb)):
        fd = fds[kind]
        own = fd[:, np.arange(s.nstates), np.arange(s.nstates)]           # dE_s / dp(., s)
        scale = np.abs(g).max()
        assert np.all(np.abs(own - g) <= 1e-4 * np.maximum(np.abs(g), 1e-3 * scale)), kind
        # other states' energies do not depend on a state's parameters
        off = fd.copy()
        off[:, np.arange(s.nstates), np.arange(s.nstates)] = 0.0
        assert np.abs(off).max() <= 1e-6 * scale, kind
        # the gap E2 - E1: +dE2/dp(.,2), -dE1/dp(.,1), 0 for the others
        gap_fd = fd[:, :, 1] - fd[:, :, 0]
        gap = np.zeros_like(g)
        gap[:, 1], gap[:, 0] = g[:, 1], -g[:, 0]
        assert np.all(np.abs(gap_fd - gap) <= 1e-4 * np.maximum(np.abs(gap), 1e-3 * scale)), kind


def test_arithmetic_rule_gradient_against_central_differences(cfg4):
    s = arithmetic_variant(cfg4)
    ref = QEnergyReference(s)
    for x in snapshots(s, 3, 13):
        _, gq, ga, gb = ref.evaluate(x)
        fq, fa, fb = ref.finite_differences(x, h=1e-5)
        for g, f in ((gq, fq), (ga, fa), (gb, fb)):
            scale = np.abs(g).max()
            assert np.all(np.abs(g - f) <= 1e-4 * np.maximum(np.abs(g), 1e-3 * scale))
    # and a sample of the same against the C oracle's differences
    x = snapshots(s, 1, 17)[0]
    _, gq, ga, gb = ref.evaluate(x)
    rng = np.random.default_rng(3)
    for _ in range(8):
        iq, st = int(rng.integers(s.nqat)), int(rng.integers(s.nstates))
        t = int(s.qiac[iq, st])
        for arr_name, g in (("qavdw", ga), ("qbvdw", gb)):
            arr = getattr(s, arr_name)
            h = 1e-5 * max(1.0, abs(arr[t, 0]))
            E = []
            for sign in (1.0, -1.0):
                sp = copy.deepcopy(s)
                a2 = arr.copy()
                a2[t, 0] += sign * h
                setattr(sp, arr_name, a2)
                E.append(oracle_q_energies(sp, x)[st])
            fd = (E[0] - E[1]) / (2.0 * h)
            assert abs(fd - g[iq, st]) <= 1e-4 * max(abs(g[iq, st]), 1e-3 * np.abs(g).max()), (arr_name, iq, st)
