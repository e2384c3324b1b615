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


def coupled_terms(s, seed, breaking=0):
    """Generated bonded terms with Morse couplings ([angle_couplings] etc.):
    the first Q angle, torsion and improper coupled to Q bonds whose r0 is
    shortened so the bonds are stretched (EMorseD < 1)."""
    bt = synthetic_bonded(s, seed=seed)
    bt.qbondlib = np.array(bt.qbondlib, dtype=np.float64)
    bt.qbondlib[:, 2] -= 0.15
    nb = len(bt.qbonds)
    assert nb >= 2 and len(bt.qangles) >= 2
    bt.ang_coupl = np.array([[0, 0, breaking], [1, nb - 1, 0]], np.int32)
    if len(bt.qtorsions):
        bt.tor_coupl = np.array([[0, 1, breaking]], np.int32)
    if len(bt.qimpropers):
        bt.imp_coupl = np.array([[0, 0, 0]], np.int32)
    return bt


def test_morse_coupled_gradient_matches_finite_differences(sys_b):
    s = sys_b
    bt = coupled_terms(s, seed=3)
    lam = np.array([0.3, 0.7])
    x = s.x + np.random.default_rng(5).normal(0, 0.03, s.x.shape)
    o = Oracle(s)
    d, _, EQb = o.bonded(x, bt, lam)
    _, _, EQu = o.bonded(x, _uncoupled(bt), lam)
    assert not np.allclose(EQb[:, 1], EQu[:, 1])   # the coupling changes the angle energy
    atoms = sorted({int(a) for a in np.concatenate([bt.qangles[:2].ravel(), bt.qbonds[[0, -1]].ravel()])})
    h = 1e-5
    for a in atoms:
        for c in range(3):
            xp, xm = x.copy(), x.copy()
            xp[a, c] += h
            xm[a, c] -= h
            fd = (energy(o, xp, bt, lam) - energy(o, xm, bt, lam)) / (2 * h)
            assert abs(fd - d[a, c]) <= 1e-5 * max(1.0, abs(fd)), (a, c, fd, d[a, c])


def _uncoupled(bt):
    import dataclasses
    return dataclasses.replace(bt, ang_coupl=np.zeros((0, 3), np.int32), tor_coupl=np.zeros((0, 3), np.int32),
                               imp_coupl=np.zeros((0, 3), np.int32))
