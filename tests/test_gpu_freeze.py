"""excluded_freeze on the GPU (qnb_set_freeze; src/potene.f90:401-405,
src/bondene.f90:791-855): every evaluation puts the excluded atoms back to
their topology positions with zero fix_shell energy and force, so an MD run
leaves them within one step's move of xtop while the free atoms move; the
ih = 1 sequence restraint drops the excluded light atoms, its energy equal to
that of the same restraint over the remaining atoms."""
import dataclasses

import numpy as np
import pytest

from q6_gb300.md import MdSetup, make_shell, maxwell_velocities
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.restraints import Restraints
from q6_gb300.system import make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.fixture(scope="module")
def sysf():
    # waters beyond 10 A excluded, plus the four outermost non-Q solute atoms,
    # two of them marked light (the generated solute has no hydrogens)
    s = make_system(R=12.0, n_solute=40, group_sizes=(3, 5), ntypes=6, nq=4, nstates=2, seed=606,
                    excl_radius=10.0)
    excl = np.asarray(s.excl).copy()
    heavy = np.asarray(s.heavy).copy()
    r = np.linalg.norm(s.x[:s.nat_solute], axis=1)
    r[np.asarray(s.iqseq)] = -1.0
    out = np.argsort(r)[-4:]
    excl[out] = 1
    heavy[out[:2]] = 0
    return dataclasses.replace(s, excl=excl, heavy=heavy)


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED])
def test_frozen_atoms_stay(sysf, prec):
    s = sysf
    excl = np.asarray(s.excl).astype(bool)
    assert excl.sum() > 0
    xtop = s.x.copy()
    with NonbondedEngine(s, precision=prec, windows=1) as e:
        e.set_lambda([0.5, 0.5])
        e.set_shell_restraint(xtop, make_shell(s, 0.85), fk_fix=200.0, fk_pshell=10.0)
        e.set_freeze(True)
        e.set_coordinates_dev(s.x[None])
        e.md_init(MdSetup(stepsize=1.0, nbcycle=5, cut=CUT))
        e.md_set_velocities(maxwell_velocities(s, 300.0, 5)[None])
        e.md_prepare(stop_cm=True)
        rec, _, _ = e.md_run(30)
        x, v = e.md_state(0)
        Er = e.restraint_energies()
    assert np.all(rec["fix"] == 0.0) and Er[0, 0] == 0.0
    move = np.linalg.norm(x - xtop, axis=1)
    # one step's move under the force of the last evaluation, at most
    assert move[excl].max() < 0.02
    assert move[~excl].max() > 5 * move[excl].max()


def test_freeze_drops_excluded_light_atoms_from_ih_selection(sysf):
    # geometric-centre sequence restraint with ih = 1 over the whole solute:
    # the frozen (excluded) atoms sit at xtop, and the excluded light atoms
    # leave the centre; E = 0.5 fk |centre(x) - centre(xtop)|^2
    s = sysf
    excl = np.asarray(s.excl).astype(bool)
    heavy = np.asarray(s.heavy).astype(bool)
    ns = s.nat_solute
    assert (excl[:ns] & ~heavy[:ns]).any()
    x = s.x + np.random.default_rng(3).normal(0, 0.2, s.x.shape)
    fk = 2.0
    with NonbondedEngine(s, precision=PREC_FP64, windows=1) as e:
        e.set_lambda([0.5, 0.5])
        e.set_shell_restraint(s.x, np.zeros(s.natom, np.uint8), fk_fix=0.0, fk_pshell=0.0)
        e.set_freeze(True)
        e.md_init(MdSetup(cut=CUT))   # the centre modes need the masses
        e.set_restraints(Restraints(seq=[(0, ns - 1, fk, 1, 1)]), xtop=s.x)
        e.set_coordinates_dev(x[None])
        e.make_pair_lists_dev(**CUT)
        e.compute_dev(sync=True)
        E = e.restraint_energies()[0, 4]
    xf = x.copy()
    xf[excl] = s.x[excl]
    pick = heavy[:ns] | ~excl[:ns]
    dr = xf[:ns][pick].mean(0) - s.x[:ns][pick].mean(0)
    assert E == pytest.approx(0.5 * fk * float(dr @ dr), rel=1e-10)
    dr_all = xf[:ns].mean(0) - s.x[:ns].mean(0)
    assert abs(0.5 * fk * float(dr_all @ dr_all) - E) > 1e-6 * E
