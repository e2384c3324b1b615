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


def _device_step0(s, prec, seeds):
    """qdyn's start and step 0 for every seed as one batched context (one
    window per seed) through the device-resident MD path: Maxwell velocities,
    qnb_md_prepare (initial_constraint, stop_cm_translation, temperature)
    and one qnb_md_run step.  Returns per-window (POT, KIN)."""
    from q6_gb300.md import maxwell_velocities
    from tests.golden.lig_w import lig_w_eq1_inputs
    setup, sp, top, bt = lig_w_eq1_inputs(s)
    W = len(seeds)
    with NonbondedEngine(s, precision=prec, windows=W) as e:
        e.set_solvent_params(sp)
        for w in range(W):
            e.set_lambda([1.0], window=w)
        e.set_coordinates_dev(np.stack([s.x] * W))
        e.set_bonded(bt)
        e.md_init(setup, bonded=top)
        e.md_set_velocities(np.stack([maxwell_velocities(s, setup.temp0, sd) for sd in seeds]))
        e.md_prepare(stop_cm=True)
        rec, EQ, Eb = e.md_run(1)
    out = []
    for w in range(W):
        r = rec[0, w]
        pot = (r["E"].sum() + EQ[0, w].sum() + r["solvent_radial"] + r["water_pol"] + r["fix"] + r["shell"]
               + r["protein"] + Eb[0, w][:6].sum() + Eb[0, w][8:12].sum())
        out.append((pot, r["ekin"]))
    return np.array(out)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_lig_w_step0_dynamics_on_gpu(prec):
    """The reference's step-0 POT, KIN and TOT bands (row 1 of
    SPH_leap-frog_berendsen_benchmark.en, 20 seeds) from the device MD path,
    20 seeds as 20 batched windows; the first two windows also equal the
    oracle's step for the same velocities (FP64 within 1e-8 relative; the
    mixed form's FP32 pair arithmetic within 0.05 kcal/mol on POT, mostly
    the ~7e5 cancelling water Coulomb terms, and 0.05 on KIN)."""
    from tests.golden.lig_w import lig_w_eq1_inputs
    from tests.test_golden import _step0_energies
    s, g = load_lig_w()
    seeds = [1000 + k for k in range(20)]
    res = _device_step0(s, prec, seeds)
    setup, sp, top, bt = lig_w_eq1_inputs(s)
    for w in range(2):
        pot, kin, _ = _step0_energies(s, seeds[w], setup, sp, top, bt)
        if prec == PREC_FP64:
            assert abs(res[w, 0] - pot) <= 1e-8 * abs(pot), (w, res[w, 0], pot)
            assert abs(res[w, 1] - kin) <= 1e-8 * abs(kin), (w, res[w, 1], kin)
        else:
            assert abs(res[w, 0] - pot) <= 0.05, (w, res[w, 0], pot)
            assert abs(res[w, 1] - kin) <= 0.05, (w, res[w, 1], kin)
    slack = 0.005 if prec == PREC_FP64 else 0.05
    for ours, band in ((res[:, 0], g["golden_pot_band"]), (res[:, 1], g["golden_kin_band"]),
                       (res[:, 0] + res[:, 1], g["golden_tot_band"])):
        ref_mean, ref_sd = 0.5 * (band[0] + band[1]), 0.5 * (band[1] - band[0])
        se = np.sqrt((ours.std(ddof=1) ** 2 + ref_sd ** 2) / 20.0)
        assert abs(ours.mean() - ref_mean) <= 3.0 * se + slack, (prec, ours.mean(), ref_mean, se)
