"""The oracle's bonded terms (bond_calc/angle_calc/torsion_calc,
src/bonded.f90:53-320; bond, angle, torsion, improper(2) and the Q bonded
terms, src/bondene.f90:41-762): gradients against central finite
differences of the energy (lambda-weighted for the Q terms), and the
removal rules of redefined and constrained terms."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.bonded import BondedTerms, remove_redefined, remove_shaken, synthetic_bonded
from q6_gb300.system import make_system


@pytest.fixture(scope="module")
def sys_b():
    return make_system(R=9.0, n_solute=24, group_sizes=(3, 5), ntypes=4, nq=8, nstates=2, seed=31)


def energy(o, x, bt, lam):
    _, Eb, EQb = o.bonded(x, bt, lam)
    return Eb.sum() + float(np.dot(lam, EQb.sum(1)))


@pytest.mark.parametrize("imp_type", [1, 2])
def test_bonded_gradient_matches_finite_differences(sys_b, imp_type):
    s = sys_b
    bt = synthetic_bonded(s, seed=3)
    bt.imp_type = imp_type
    lam = np.array([0.3, 0.7])
    rng = np.random.default_rng(0)
    x = s.x + rng.normal(0, 0.05, s.x.shape)   # away from the equilibrium values
    o = Oracle(s)
    d, Eb, EQb = o.bonded(x, bt, lam)
    assert np.count_nonzero(Eb) >= 5 and np.count_nonzero(EQb) >= 4
    atoms = sorted(set(rng.choice(s.nat_solute, 10, replace=False).tolist()) | {int(s.iqseq[0])} |
                   {s.nat_solute, s.nat_solute + 1})
    h = 1e-5
    for a in atoms:
        for c in range(3):
            xp, xm = x.copy(), x.copy()
            xp[a, c] += h
            xm[a, c] -= h
            fd = (energy(o, xp, bt, lam) - energy(o, xm, bt, lam)) / (2 * h)
            assert abs(fd - d[a, c]) <= 1e-5 * max(1.0, abs(fd)), (a, c, fd, d[a, c])


def test_q_urey_bradley_gradient(sys_b):
    s = sys_b
    bt = synthetic_bonded(s, seed=4)
    bt.urey_bradley = 1
    bt.qanglib = bt.qanglib.copy()
    bt.qanglib[:, 2] = 25.0
    bt.qanglib[:, 3] = 2.4
    lam = np.array([0.6, 0.4])
    x = s.x + np.random.default_rng(2).normal(0, 0.04, s.x.shape)
    o = Oracle(s)
    d, _, _ = o.bonded(x, bt, lam)
    a = int(bt.qangles[0, 0])
    h = 1e-5
    for c in range(3):
        xp, xm = x.copy(), x.copy()
        xp[a, c] += h
        xm[a, c] -= h
        fd = (energy(o, xp, bt, lam) - energy(o, xm, bt, lam)) / (2 * h)
        assert abs(fd - d[a, c]) <= 1e-5 * max(1.0, abs(fd))


def test_removal_rules():
    bt = BondedTerms(bonds=np.array([[0, 1, 0], [2, 1, 0], [3, 4, 0], [5, 6, 0]], np.int32), nbonds_solute=3,
                     bondlib=np.array([[100.0, 1.0]]),
                     angles=np.array([[0, 1, 2, 0], [2, 1, 0, 0], [0, 1, 3, 0]], np.int32),
                     torsions=np.array([[0, 1, 2, 3, 0], [3, 2, 1, 0, 0], [0, 1, 2, 4, 0]], np.int32),
                     impropers=np.array([[2, 1, 0, 3, 0], [3, 1, 2, 0, 0], [0, 1, 3, 2, 0]], np.int32),
                     qbonds=np.array([[1, 2]], np.int32), qangles=np.array([[0, 1, 2]], np.int32),
                     qtorsions=np.array([[0, 1, 2, 3]], np.int32), qimpropers=np.array([[0, 1, 2, 3]], np.int32))
    r = remove_redefined(bt)
    assert r.bonds[:, 2].tolist() == [0, -1, 0, 0]
    assert r.angles[:, 3].tolist() == [-1, -1, 0]
    assert r.torsions[:, 4].tolist() == [-1, -1, 0]
    # (k,j,i,l) and (l,j,k,i) orders match, (i,j,l,k) does not
    assert r.impropers[:, 4].tolist() == [-1, -1, 0]
    heavy = np.array([1, 1, 1, 1, 1, 0, 1], bool)
    sh = remove_shaken(r, heavy, nat_solute=5)
    assert sh.bonds[:, 2].tolist() == [0, -1, 0, -1]   # solvent bond with a hydrogen constrained
