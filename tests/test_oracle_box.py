"""The periodic-box restatement (oracle/box.py; qdyn's *_box lists and
energies) pinned three ways: in a box far larger than the system every
shift is zero and the box energies equal the C oracle's sphere energies with
the same cut-offs; moving whole charge groups and water molecules by lattice
vectors changes no energy and no gradient; the gradient matches finite
differences of the energy in a box small enough that pairs wrap."""
import numpy as np
import pytest

from oracle.box import box_energies, box_lists, shift_of
from oracle.oracle import Oracle
from q6_gb300.system import make_system

LAM = [0.3, 0.7]


@pytest.fixture(scope="module")
def sysb():
    return make_system(R=11.0, n_solute=60, group_sizes=(3, 5), ntypes=5, nq=3, nstates=2, seed=404)


def total(E, EQ, lam=LAM):
    return sum(E.values()) + float(np.asarray(lam) @ EQ.sum(1))


def test_large_box_equals_sphere(sysb):
    s = sysb
    cut = dict(Rcq=99.0, RcLRF=99.0, Rcpp=9.0, Rcpw=9.0, Rcww=9.0)
    o = Oracle(s, use_lrf=False)
    _, E0, EQ0, _ = o.evaluate(s.x, LAM, cut=cut)
    _, EQs = o.nonbond_qq(s.x)   # the static Q-Q and Q-bonded-P part (no box variant)
    o.close()
    EQ0 = EQ0 - EQs
    qs = int(s.iqseq[0])
    d, E, EQ = box_energies(s, s.x, LAM, [1000.0] * 3, qs, cut)
    for k in E:
        assert E[k] == pytest.approx(E0[k], rel=1e-11, abs=1e-9), k
    np.testing.assert_allclose(EQ[:, 2:6], EQ0[:, 2:6], rtol=1e-11, atol=1e-9)


def wrapped_case(s):
    L = np.array([2 * 11.0 + 3.0] * 3)
    cut = dict(Rcq=12.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
    return L, cut


def test_lattice_moves_change_nothing(sysb):
    s = sysb
    L, cut = wrapped_case(s)
    qs = int(s.iqseq[0])
    d0, E0, EQ0 = box_energies(s, s.x, LAM, L, qs, cut)
    rng = np.random.default_rng(1)
    x = s.x.copy()
    qconn = np.asarray(s.qconn)
    near = set(np.nonzero((qconn <= 3).any(axis=(0, 2)))[0].tolist()) | set(np.asarray(s.iqseq).tolist())
    moved = 0
    for g in range(s.ncgp_solute):
        atoms = s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1]
        if near & set(atoms.tolist()):
            continue   # the static Q lists keep plain distances
        x[atoms] += L * rng.integers(-2, 3, 3)
        moved += 1
    for w in range(s.nwat):
        a = s.nat_solute + 3 * w
        x[a:a + 3] += L * rng.integers(-2, 3, 3)
    assert moved > 0
    d1, E1, EQ1 = box_energies(s, x, LAM, L, qs, cut)
    for k in E0:
        assert E1[k] == pytest.approx(E0[k], rel=1e-10, abs=1e-8), k
    np.testing.assert_allclose(EQ1, EQ0, rtol=1e-10, atol=1e-8)
    np.testing.assert_allclose(d1, d0, rtol=1e-8, atol=1e-7)


def test_pairs_wrap_and_gradient_matches_differences(sysb):
    s = sysb
    L, cut = wrapped_case(s)
    qs = int(s.iqseq[0])
    lists = box_lists(s, s.x, L, qs, cut)
    ns = s.nat_solute
    first = ns + 3 * np.asarray([p[1] for p in lists["ww"]])
    firsti = ns + 3 * np.asarray([p[0] for p in lists["ww"]])
    nwrap = int((np.abs(shift_of(L, s.x[firsti], s.x[first])).sum(1) > 0).sum())
    assert nwrap > 10 and len(lists["qw"]) > 0 and len(lists["qp"]) > 0 and len(lists["pw"]) > 0
    d, E, EQ = box_energies(s, s.x, LAM, L, qs, cut, lists)
    rng = np.random.default_rng(2)
    h = 1e-6
    for a in rng.choice(s.natom, 6, replace=False).tolist() + [int(s.iqseq[1])]:
        for c in range(3):
            xp = s.x.copy()
            xm = s.x.copy()
            xp[a, c] += h
            xm[a, c] -= h
            _, Ep, EQp = box_energies(s, xp, LAM, L, qs, cut, lists)
            _, Em, EQm = box_energies(s, xm, LAM, L, qs, cut, lists)
            fd = (total(Ep, EQp) - total(Em, EQm)) / (2 * h)
            assert d[a, c] == pytest.approx(fd, rel=1e-5, abs=1e-5), (a, c)
