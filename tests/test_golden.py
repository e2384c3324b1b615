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
