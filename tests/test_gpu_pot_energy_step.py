"""qnb_pot_energy_step: the nonbonded side of pot_energy of a single-window
context in one host-buffer call equals the four separate entry points
(qnb_pot_energy_nonbonds, qnb_nonbond_qq, qnb_restrain_solvent, qnb_watpol)
made back to back on the same coordinates, over steps that cross a list
rebuild and a watpol update (itdis 2), in both forms: energies within 1e-10
relative and the gradient within 1e-10 of its scale (the separate calls add
their parts on the host, the fused call on the device); and it refuses a
batched context."""
import numpy as np
import pytest

from q6_gb300.qnb import E_FIELDS, PREC_FP64, PREC_MIXED, NonbondedEngine, QnbError
from q6_gb300.system import config_small, default_solvent_params

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_fused_step_equals_separate_calls(prec):
    s = config_small()
    sp = default_solvent_params(s, itdis=2.0)
    rng = np.random.default_rng(5)
    xs = [s.x + rng.normal(0.0, 0.01, s.x.shape) for _ in range(4)]
    out = {}
    for mode in ("fused", "separate"):
        rec = []
        with NonbondedEngine(s, precision=prec) as e:
            e.set_solvent_params(sp)
            e.set_lambda([0.3, 0.7])
            for k, x in enumerate(xs):
                if k % 3 == 0:
                    e.make_pair_lists(x, **CUT)
                d = np.zeros_like(x)
                if mode == "fused":
                    d, E, EQ, R = e.pot_energy_step(x, d, Tfree=300.0, istep=k)
                else:
                    d, E, EQ = e.pot_energy_nonbonds(x, d)
                    d, EQ = e.nonbond_qq(x, d, EQ)
                    R = np.array([e.restrain_solvent(x, d, 300.0), e.watpol(x, d, k)])
                rec.append((d.copy(), E, EQ.copy(), np.asarray(R, float).copy()))
        out[mode] = rec
    for (d1, E1, EQ1, R1), (d0, E0, EQ0, R0) in zip(out["fused"], out["separate"]):
        for k in E0:
            assert E1[k] == pytest.approx(E0[k], rel=1e-10, abs=1e-10), k
        np.testing.assert_allclose(EQ1, EQ0, rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(R1, R0, rtol=1e-10, atol=1e-10)
        assert np.abs(d1 - d0).max() <= 1e-10 * np.abs(d0).max()
    assert any(r[3][1] != 0.0 for r in out["fused"])   # watpol contributed


def test_fused_step_refuses_batches():
    s = config_small()
    with NonbondedEngine(s, precision=PREC_MIXED, windows=2) as e:
        e.set_lambda([0.5, 0.5])
        e.set_coordinates_dev(np.stack([s.x, s.x]))
        e.make_pair_lists_dev(**CUT)
        with pytest.raises(QnbError):
            e.pot_energy_step(s.x)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_step_host_equals_upload_build_compute_download(prec):
    """qnb_step_host (one host synchronisation) against the separate batched
    calls on three windows over steps that cross two list rebuilds and a
    watpol update: the same device work, so the gradient and energies agree
    bit for bit in the mixed form (fixed-point sums) and within 1e-10 in the
    FP64 form (FP64 atomics sum in arrival order); a context without lists is
    refused."""
    s = config_small()
    sp = default_solvent_params(s, itdis=2.0)
    W = 3
    rng = np.random.default_rng(9)
    xs = [np.stack([s.x + rng.normal(0.0, 0.01, s.x.shape) for _ in range(W)]) for _ in range(5)]
    out = {}
    for mode in ("fused", "separate"):
        rec = []
        with NonbondedEngine(s, precision=prec, windows=W) as e:
            e.set_solvent_params(sp)
            for w in range(W):
                e.set_lambda([0.2 + 0.3 * w, 0.8 - 0.3 * w], window=w)
            if mode == "fused":
                with pytest.raises(QnbError):
                    e.step_host(xs[0])
            e.set_coordinates_dev(xs[0])
            e.make_pair_lists_dev(**CUT)
            for k, x in enumerate(xs):
                rebuild = k % 3 == 0
                if mode == "fused":
                    d, E, EQ, R = e.step_host(x, Tfree=300.0, istep=k, rebuild_lists=rebuild)
                else:
                    e.set_coordinates_dev(x)
                    if rebuild:
                        e.make_pair_lists_dev(**CUT)
                    E, EQ, R = e.compute_dev(Tfree=300.0, istep=k, sync=True)
                    E = np.array([[w[f] for f in E_FIELDS] for w in E])
                    d = e.gradient_dev()
                rec.append((d.copy(), E, EQ.copy(), R.copy()))
        out[mode] = rec
    for (d1, E1, EQ1, R1), (d0, E0, EQ0, R0) in zip(out["fused"], out["separate"]):
        if prec == PREC_MIXED:
            assert np.array_equal(E1, E0)
            assert np.array_equal(EQ1, EQ0) and np.array_equal(R1, R0)
            assert np.array_equal(d1, d0)
            continue
        np.testing.assert_allclose(E1, E0, rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(EQ1, EQ0, rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(R1, R0, rtol=1e-10, atol=1e-10)
        assert np.abs(d1 - d0).max() <= 1e-10 * np.abs(d0).max()
    assert np.abs(out["fused"][-1][0]).max() > 0.0
