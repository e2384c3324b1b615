"""Pins the CPU oracle to Q6's own regression test.

tests/basic_tests/eval_test.sh:99 of Q6 requires the step-0 Q-atom line
"Q-surr. 1 1.0000      3.12    139.43" for the spherical lig_w system, and row 1
of SPH_leap-frog_berendsen_benchmark.en (zero-width band) gives EL -7.30 and
VdW -413.17 (solute + solvent + solute-solvent rows).  qdyn computes these
after its start-up SHAKE of the solvent (initial_constraint,
src/bondene.f90:1025-1048) at the topology coordinates.
"""
import numpy as np

from oracle.oracle import Oracle, shake
from tests.golden.lig_w import lig_w_bonded, load_lig_w


def _step0_coordinates(s, g):
    mols = {}
    for (i, j), b0 in zip(g["wbond_ij"], g["wbond_b0"]):
        mols.setdefault((int(i) - s.nat_solute) // s.solv_atom, []).append((int(i), int(j), float(b0)))
    winv = 1.0 / s.mass[s.iac]
    return shake(s.x, [mols[k] for k in sorted(mols)], winv)


def test_lig_w_step0_energies_match_reference_strings():
    s, g = load_lig_w()
    x = _step0_coordinates(s, g)
    o = Oracle(s, use_lrf=True)
    d, E, EQ, _ = o.evaluate(x, [1.0], cut=dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0))
    qsurr_el = EQ[0, 2] + EQ[0, 4]
    qsurr_vdw = EQ[0, 3] + EQ[0, 5]
    el = E["pp_el"] + E["ww_el"] + E["pw_el"]
    vdw = E["pp_vdw"] + E["ww_vdw"] + E["pw_vdw"]
    # the reference prints f10.2: compare the printed strings
    assert f"{qsurr_el:10.2f}" == f"{g['golden_qsurr_el']:10.2f}"
    assert f"{qsurr_vdw:10.2f}" == f"{g['golden_qsurr_vdw']:10.2f}"
    assert f"{el:.2f}" == f"{g['golden_el']:.2f}"
    assert f"{vdw:.2f}" == f"{g['golden_vdw']:.2f}"
    # all solute atoms are Q atoms: no pp / pw pairs
    assert o.list_size(0) == 0 and o.list_size(1) == 0
    assert o.list_size(2) % 9 == 0


def test_lig_w_without_shake_misses_golden():
    """The start-up SHAKE matters: topology coordinates alone print 3.03."""
    s, g = load_lig_w()
    o = Oracle(s, use_lrf=True)
    d, E, EQ, _ = o.evaluate(s.x, [1.0])
    assert f"{EQ[0, 2] + EQ[0, 4]:.2f}" != f"{g['golden_qsurr_el']:.2f}"


def test_lig_w_step0_bonded_energies_match_reference_strings():
    """Row 1 of SPH_leap-frog_berendsen_benchmark.en: the solute row's bond,
    angle, torsion, improper (31.61 30.69 6.28 0.05) and the Q-atom row's
    (-122.04 0.68 2.17 0.00), with the FEP-redefined terms and the SHAKE-
    constrained solvent bonds removed from the topology lists as qdyn does."""
    s, g = load_lig_w()
    x = _step0_coordinates(s, g)
    o = Oracle(s, use_lrf=True)
    _, Eb, EQb = o.bonded(x, lig_w_bonded(s), [1.0])
    got = [Eb[0], Eb[1], Eb[2], Eb[3], EQb[0, 0], EQb[0, 1], EQb[0, 2], EQb[0, 3]]
    want = [g[k] for k in ("golden_bnd", "golden_ang", "golden_tor", "golden_imp",
                           "golden_qbnd", "golden_qang", "golden_qtor", "golden_qimp")]
    for a, b in zip(got, want):
        assert f"{a:.2f}" == f"{b:.2f}", (a, b)


def _step0_energies(s, seed, setup, sp, top, bt):
    """qdyn's first MD step on the oracle: Maxwell velocities at the input's
    0.1 K (numpy's generator in place of qdyn's random stream),
    initial_constraint, stop_cm_translation and temperature(), then step 0
    (pair lists, pot_energy, leap-frog with Berendsen, SHAKE, temperature).
    Returns (POT, KIN, Tfree of the start)."""
    from oracle.oracle import OracleMD
    from q6_gb300.md import build_constraints, maxwell_velocities, md_params
    cons = build_constraints(s, setup, top)
    p = md_params(s, setup, cons)
    o = Oracle(s, use_lrf=True)
    o.set_solvent_params(sp)
    omd = OracleMD(o, p, cons, sp=sp, lam=np.array([1.0]), bonded=bt)
    x, v = omd.prepare(s.x, maxwell_velocities(s, setup.temp0, seed))
    tfree0 = omd.tfree
    r = omd.step(x, v, 0, setup.cut)
    pot = (sum(r["E"].values()) + r["EQ"].sum() + r["erst"][0] + r["erst"][1] + r["Eb"][:6].sum()
           + r["EQb"].sum())
    o.close()
    return pot, r["ekin"], tfree0


def test_lig_w_step0_potential_and_kinetic_energy_match_reference_bands():
    """Row 1 of SPH_leap-frog_berendsen_benchmark.en holds the reference's
    step-0 POT, KIN and TOT as mean -/+ one standard deviation over the 20
    random seeds of its benchmark.  POT covers every term of the path the
    printed strings leave out (LRF, Q-Q, solvent radial restraint, water
    polarisation) and KIN covers SHAKE and the Berendsen step.  Three qdyn
    behaviours matter and are reproduced: the rigid-water angles are cleared
    by init_constraints; the Born term is on with wat_shells' mu_w; and the
    Tfree of restrain_solvent's shift comes from initial_constraint's SHAKE
    of the start (about 35 K, not the 0.1 K of the Maxwell draw), since the
    topology waters meet the constraints only to SHAKE's tolerance.  Over
    20 seeds of our own the means must agree within three standard errors
    plus the print rounding, and the spreads within a factor of two."""
    from tests.golden.lig_w import lig_w_eq1_inputs
    s, g = load_lig_w()
    setup, sp, top, bt = lig_w_eq1_inputs(s)
    res = np.array([_step0_energies(s, 1000 + k, setup, sp, top, bt) for k in range(20)])
    pot, kin = res[:, 0], res[:, 1]
    assert np.all(res[:, 2] > 20.0)            # the start's Tfree is set by SHAKE, not by 0.1 K
    for ours, band in ((pot, g["golden_pot_band"]), (kin, g["golden_kin_band"]), (pot + kin, g["golden_tot_band"])):
        ref_mean, ref_sd = 0.5 * (band[0] + band[1]), 0.5 * (band[1] - band[0])
        sd = ours.std(ddof=1)
        se = np.sqrt((sd ** 2 + ref_sd ** 2) / 20.0)
        assert abs(ours.mean() - ref_mean) <= 3.0 * se + 0.005, (ours.mean(), ref_mean, se)
        assert 0.5 <= sd / ref_sd <= 2.0, (sd, ref_sd)


def test_lig_w_shaken_water_angles_are_cleared():
    """init_constraints clears the first angle whose end atoms are a
    constrained pair: each rigid water's H-O-H angle (6.33 kcal/mol at step
    0 if it were kept)."""
    from tests.golden.lig_w import lig_w_bonded, lig_w_topology_terms
    s, g = load_lig_w()
    top, bt = lig_w_topology_terms(s), lig_w_bonded(s)
    water = np.arange(len(bt.angles)) >= bt.nangles_solute
    assert np.all(bt.angles[water, 3] == -1) and np.all(top.angles[water, 3] >= 0)
    assert np.all(bt.angles[~water, 3] == top.angles[~water, 3])
    x = _step0_coordinates(s, g)
    o = Oracle(s, use_lrf=True)
    _, Eb, _ = o.bonded(x, bt, [1.0])
    _, Eb_top, _ = o.bonded(x, top, [1.0])
    assert Eb[5] == 0.0 and abs(Eb_top[5] - 6.33) < 0.01
