"""Bonded terms on the GPU (qnb_set_bonded) against the oracle's restatement.

lig_w: the reference's step-0 bonded columns (solute bond, angle, torsion,
improper; Q-atom bond, angle, torsion, improper) reproduced on the device in
both forms, and every energy and the gradient within 1e-9 (FP64 form) /
2e-5 relative (mixed form: FP32 arithmetic per term, as the reference's
single-precision build, summed in 2^-32 fixed point) of the oracle.  A generated system with Q bonded terms in two states (Morse and
harmonic Q bonds): batched windows bit-equal to single contexts (mixed), and
the FP64 form against the oracle with both improper forms."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.bonded import synthetic_bonded
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.system import lambdas_for_window, make_system
from tests.golden.lig_w import lig_w_bonded, load_lig_w
from tests.test_golden import _step0_coordinates

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


def device_eval(s, bt, x, lams, prec):
    W = len(lams)
    with NonbondedEngine(s, precision=prec, windows=W) as e:
        for w in range(W):
            e.set_lambda(lams[w], window=w)
        e.set_bonded(bt)
        e.set_coordinates_dev(np.stack([x] * W) if x.ndim == 2 else x)
        e.make_pair_lists_dev(**CUT)
        E, EQ, _ = e.compute_dev(sync=True)
        Eb, EQb = e.bonded_energies()
        D = e.gradient_dev()
    return E, EQ, Eb, EQb, D


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_lig_w_bonded_on_gpu(prec):
    s, g = load_lig_w()
    x = _step0_coordinates(s, g)
    bt = lig_w_bonded(s)
    E, EQ, Eb, EQb, D = device_eval(s, bt, x, [[1.0]], prec)
    got = [Eb[0, 0], Eb[0, 1], Eb[0, 2], Eb[0, 3], EQb[0, 0, 0], EQb[0, 0, 1], EQb[0, 0, 2], EQb[0, 0, 3]]
    want = [g[k] for k in ("golden_bnd", "golden_ang", "golden_tor", "golden_imp",
                           "golden_qbnd", "golden_qang", "golden_qtor", "golden_qimp")]
    for a, b in zip(got, want):
        assert f"{a:.2f}" == f"{b:.2f}", (a, b)
    o = Oracle(s)
    d0, _, _, _ = o.evaluate(x, [1.0], cut=CUT)
    d0, Eb0, EQb0 = o.bonded(x, bt, [1.0], d0)
    # mixed form: FP32 arithmetic per term (the reference's single-precision build)
    rtol, atol = (1e-9, 1e-9) if prec == PREC_FP64 else (2e-5, 2e-4)
    assert np.allclose(Eb[0], Eb0, rtol=rtol, atol=atol)
    assert np.allclose(EQb[0], EQb0, rtol=rtol, atol=atol)
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    gtol = 1e-6 if prec == PREC_FP64 else 2e-3   # the nonbonded part dominates the mixed-form bar
    assert np.all(np.abs(D[0] - d0) <= gtol * scale + 1e-9)


@pytest.fixture(scope="module")
def sys_q():
    return make_system(R=13.0, n_solute=60, group_sizes=(3, 5), ntypes=6, nq=10, nstates=2, seed=818)


@pytest.mark.parametrize("imp_type", [1, 2])
def test_generated_bonded_fp64_matches_oracle(sys_q, imp_type):
    s = sys_q
    bt = synthetic_bonded(s, seed=9)
    bt.imp_type = imp_type
    x = s.x + np.random.default_rng(1).normal(0, 0.03, s.x.shape)
    lam = [0.35, 0.65]
    E, EQ, Eb, EQb, D = device_eval(s, bt, x, [lam], PREC_FP64)
    o = Oracle(s)
    d0, _, _, _ = o.evaluate(x, lam, cut=CUT)
    d0, Eb0, EQb0 = o.bonded(x, bt, lam, d0)
    assert np.allclose(Eb[0], Eb0, rtol=1e-9, atol=1e-9)
    assert np.allclose(EQb[0], EQb0, rtol=1e-9, atol=1e-9)
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    assert np.all(np.abs(D[0] - d0) <= 1e-6 * scale + 1e-9)


def test_generated_bonded_batched_equals_single(sys_q):
    s = sys_q
    bt = synthetic_bonded(s, seed=10)
    rng = np.random.default_rng(5)
    xs = np.stack([s.x + rng.normal(0, 0.03, s.x.shape) for _ in range(3)])
    lams = [lambdas_for_window(l, 2) for l in (0.0, 0.4, 1.0)]
    Eb3, EQb3, D3 = device_eval(s, bt, xs, lams, PREC_MIXED)[2:]
    for w in (0, 2):
        Eb1, EQb1, D1 = device_eval(s, bt, xs[w], [lams[w]], PREC_MIXED)[2:]
        assert np.array_equal(Eb3[w], Eb1[0]) and np.array_equal(EQb3[w], EQb1[0])
        assert np.array_equal(D3[w], D1[0])


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_fix_shell_on_gpu(prec):
    """fix_shell inside qnb_compute_dev against the oracle: excluded atoms
    (fk_fix 200) and shell atoms beyond 3 A of the solute centre (fk_pshell
    10) restrained to the generated coordinates, evaluated at displaced ones."""
    from q6_gb300.md import make_shell
    s = make_system(R=12.0, n_solute=40, group_sizes=(3, 5), ntypes=6, nq=4, nstates=2, seed=13,
                    excl_radius=10.0)
    sh = make_shell(s, 3.0)
    x = s.x + np.random.default_rng(2).normal(0, 0.05, s.x.shape)
    with NonbondedEngine(s, precision=prec) as e:
        e.set_lambda([0.5, 0.5])
        e.set_shell_restraint(s.x, sh, 200.0, 10.0)
        e.set_coordinates_dev(x[None])
        e.make_pair_lists_dev(**CUT)
        e.compute_dev(sync=True)
        Er = e.restraint_energies()
        D = e.gradient_dev()
    o = Oracle(s)
    d0, _, _, _ = o.evaluate(x, [0.5, 0.5], cut=CUT)
    d0, E0 = o.fix_shell(x, s.x, sh, 200.0, 10.0, d0)
    assert E0[0] > 0 and E0[1] > 0
    assert np.allclose(Er[0, :2], E0, rtol=1e-9, atol=1e-9)
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    gtol = 1e-6 if prec == PREC_FP64 else 2e-3
    assert np.all(np.abs(D[0] - d0) <= gtol * scale + 1e-9)


@pytest.mark.parametrize("breaking", [0, 1])
def test_morse_couplings_match_oracle(sys_q, breaking):
    from tests.test_oracle_bonded import coupled_terms
    s = sys_q
    bt = coupled_terms(s, seed=9, breaking=breaking)
    x = s.x + np.random.default_rng(2).normal(0, 0.03, s.x.shape)
    lam = [0.35, 0.65]
    o = Oracle(s)
    d0, _, _, _ = o.evaluate(x, lam, cut=CUT)
    d0, Eb0, EQb0 = o.bonded(x, bt, lam, d0)
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    for prec, tol in ((PREC_FP64, 1e-9), (PREC_MIXED, 1e-4)):
        E, EQ, Eb, EQb, D = device_eval(s, bt, x, [lam], prec)
        assert np.allclose(EQb[0], EQb0, rtol=tol, atol=tol), prec
        assert np.all(np.abs(D[0] - d0) <= (1e-6 if prec == PREC_FP64 else 1e-3) * scale + 1e-9), prec
