"""Pins the periodic-box restatement (oracle/box.py) to Q6's own regression
test for the box.

Row 1 of tests/basic_tests/PBC_leap-frog_berendsen_benchmark.en (zero-width
bands) is the step-0 energy of the prep_PBC system (the lig_w solute, all 46
atoms Q atoms, in a 49.633 A box of 4,072 SPC waters) run with q_atom 24 and
lrf 24: Q-surr. el -31.30 and vdW 228.64 (eval_test.sh:101), EL 380.33 and
VdW -1990.55, and the potential energy POT -1512.62.  POT holds every term
of the step: the box lists' water-water and Q-water energies, the box LRF
(lrf_update with its lattice shift, lrf_taylor over all non-Q atoms), the
static Q-Q pairs and the bonded terms; its LRF part is -67.06 kcal/mol, so
the box LRF is pinned to the reference by it."""
import numpy as np
import pytest

from oracle.box import box_energies, box_lists, box_lrf, box_lrf_taylor
from oracle.oracle import Oracle
from tests.golden.lig_w import PBC_CUT, lig_w_bonded, lig_w_pbc_step0_coordinates, load_lig_w


@pytest.fixture(scope="module")
def step0():
    s, g = load_lig_w("pbc")
    x = lig_w_pbc_step0_coordinates(s, g)
    L, qs = g["boxlength"], g["qswitch"]
    lists = box_lists(s, x, L, qs, PBC_CUT)
    _, E, EQ = box_energies(s, x, [1.0], L, qs, PBC_CUT, lists)
    rec = box_lrf(s, x, L, PBC_CUT)
    elrf, _ = box_lrf_taylor(s, x, rec)
    o = Oracle(s, use_lrf=False)
    o.set_lambda([1.0])
    o.make_pair_lists(x, **dict(PBC_CUT, Rcq=99.0))
    _, EQs = o.nonbond_qq(x)
    _, Eb, EQb = o.bonded(x, lig_w_bonded(s), np.array([1.0]))
    o.close()
    return dict(s=s, g=g, lists=lists, E=E, EQ=EQ, elrf=elrf, EQs=EQs, Eb=Eb, EQb=EQb)


def test_pbc_step0_printed_strings(step0):
    E, EQ, g = step0["E"], step0["EQ"], step0["g"]
    assert not step0["lists"]["pp"] and not step0["lists"]["pw"] and not step0["lists"]["qp"]
    assert f"{EQ[0, 2] + EQ[0, 4]:10.2f}" == f"{g['golden_qsurr_el']:10.2f}"    # Q-surr. el
    assert f"{EQ[0, 3] + EQ[0, 5]:10.2f}" == f"{g['golden_qsurr_vdw']:10.2f}"   # Q-surr. vdW
    assert f"{E['ww_el']:.2f}" == f"{g['golden_el']:.2f}"
    assert f"{E['ww_vdw']:.2f}" == f"{g['golden_vdw']:.2f}"


def test_pbc_step0_potential_energy_with_box_lrf(step0):
    d = step0
    rest = sum(d["E"].values()) + d["EQ"].sum() + d["EQs"].sum() + d["Eb"][:6].sum() + d["EQb"].sum()
    pot = rest + d["elrf"]
    lo, hi = d["g"]["golden_pot_band"]
    assert lo == hi
    assert f"{pot:.2f}" == f"{lo:.2f}", pot
    assert abs(d["elrf"]) > 50.0 and f"{rest:.2f}" != f"{lo:.2f}"   # the LRF term is needed
