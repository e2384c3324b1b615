"""The oracle's p_restrain (src/bondene.f90:764-1020): gradients against
central finite differences of E%restraint%protein + sum_s lambda_s
EQ(s)%restraint for every kind with a gradient force, and the two centre
modes of sequence restraints, whose forces are not the energy's gradient
in the reference: dr fk m_i / 12.010 on each atom (geometric centre) and
dr fk (mass centre)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from q6_gb300.restraints import Restraints
from q6_gb300.system import make_system


@pytest.fixture(scope="module")
def sys_r():
    return make_system(R=11.0, n_solute=30, group_sizes=(3, 5), ntypes=6, nq=4, nstates=2, seed=404)


def restraints(s):
    n = s.nat_solute
    w0 = s.nat_solute
    return Restraints(
        seq=[(0, 9, 2.0, 0, 0), (10, 19, 1.5, 1, 0)],
        pos=[(3, -1, s.x[3] + 0.2, (5.0, 4.0, 3.0)), (7, 1, s.x[7] - 0.1, (2.0, 2.0, 2.0))],
        dist=[(0, n - 1, 3.0, 4.0, 10.0, 0), (2, 12, 1.0, 1.5, 7.0, -1)],
        ang=[(0, 1, 2, 100.0, 30.0, 1), (4, 5, 6, 120.0, 20.0, -1)],
        wall=[(w0, w0 + 30, 6.0, 15.0, 0.6, 0.5, 1)])


def total(o, x, r, lam):
    _, ep, eq = o.p_restrain(x, r, lam)
    return ep + float(np.dot(lam, eq))


def test_restraint_gradients(sys_r):
    s = sys_r
    r = restraints(s)
    lam = np.array([0.25, 0.75])
    rng = np.random.default_rng(3)
    x = s.x + rng.normal(0, 0.15, s.x.shape)
    o = Oracle(s)
    d, ep, eq = o.p_restrain(x, r, lam)
    assert ep != 0.0 and np.all(eq != 0.0)
    atoms = [0, 1, 2, 3, 5, 7, 12, 15, s.nat_solute - 1, s.nat_solute + 1, s.nat_solute + 9]
    h = 1e-6
    for a in atoms:
        for c in range(3):
            xp, xm = x.copy(), x.copy()
            xp[a, c] += h
            xm[a, c] -= h
            fd = (total(o, xp, r, lam) - total(o, xm, r, lam)) / (2 * h)
            assert abs(fd - d[a, c]) <= 1e-5 * max(1.0, abs(fd)), (a, c, fd, d[a, c])


def test_geometric_centre_force_quirk(sys_r):
    s = sys_r
    o = Oracle(s)
    x = s.x.copy()
    x[:10] += np.array([0.3, -0.2, 0.1])
    d, ep, _ = o.p_restrain(x, Restraints(seq=[(0, 9, 4.0, 1, 1)]), [0.5, 0.5])
    dr = np.array([0.3, -0.2, 0.1])
    assert ep == pytest.approx(0.5 * 4.0 * dr @ dr)
    m = s.mass[s.iac[:10]]
    assert np.allclose(d[:10], dr[None, :] * (4.0 * m / 12.010)[:, None])


def test_mass_centre_force_quirk(sys_r):
    s = sys_r
    o = Oracle(s)
    x = s.x.copy()
    x[10:20] += np.array([-0.1, 0.25, 0.05])
    d, ep, _ = o.p_restrain(x, Restraints(seq=[(10, 19, 3.0, 1, 2)]), [0.5, 0.5])
    dr = np.array([-0.1, 0.25, 0.05])
    assert ep == pytest.approx(0.5 * 3.0 * dr @ dr)
    assert np.allclose(d[10:20], np.broadcast_to(dr * 3.0, (10, 3)))
