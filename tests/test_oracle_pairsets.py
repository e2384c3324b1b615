"""The restated monitor-group energies and group-contribution exclusions
(oracle/pairsets.py; src/nonbondene.f90:4517-4680, 6825-6920,
src/simprep.f90:2879-2945) pinned to the C oracle's force loops, which the
golden fixtures pin: with no cut-off, excluding every solute atom removes the
whole Q-Q and Q-P energy of each state; monitoring the Q atoms against the
rest of the solute gives the Q-P energy; two halves of the non-Q solute
monitored against each other give the P-P energy between them (the C
oracle's P-P energy minus that with the halves pulled apart)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from oracle.pairsets import group_exclusions, monitor_energies
from q6_gb300.enefile import ELECTRO, FULL, NOGC, VDW, EnergyFileWriter, group_contribution_header, read_energy_file
from q6_gb300.system import make_system

CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=99.0, Rcpw=99.0, Rcww=99.0)


@pytest.fixture(scope="module")
def sysx():
    s = make_system(R=10.0, n_solute=24, group_sizes=(3, 4), ntypes=4, nq=5, nstates=2, seed=31,
                    soft_pairs=((0, 2),), el_scale=(((1, 3), (0.5, 0.8)),))
    return s


def oracle_eq(s, x):
    o = Oracle(s, use_lrf=False)
    _, E, EQ, _ = o.evaluate(x, [0.5, 0.5], cut=CUT)
    o.close()
    return E, EQ


def test_exclude_all_solute_is_whole_q_energy(sysx):
    s = sysx
    _, EQ = oracle_eq(s, s.x)
    exc = group_exclusions(s, s.x, [np.ones(s.nat_solute, bool)])[0]
    np.testing.assert_allclose(exc[:, 0:2], EQ[:, 0:2], rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(exc[:, 2:4], EQ[:, 2:4], rtol=1e-10, atol=1e-9)
    none = group_exclusions(s, s.x, [np.zeros(s.nat_solute, bool)])[0]
    assert not none.any()


def test_exclusions_add_over_disjoint_non_q_groups(sysx):
    s = sysx
    rng = np.random.default_rng(3)
    nonq = np.setdiff1d(np.arange(s.nat_solute), s.iqseq)
    pick = rng.random(len(nonq)) < 0.5
    m1 = np.zeros(s.nat_solute, bool)
    m2 = np.zeros(s.nat_solute, bool)
    m1[nonq[pick]] = True
    m2[nonq[~pick]] = True
    e1, e2, e12 = group_exclusions(s, s.x, [m1, m2, m1 | m2])
    np.testing.assert_allclose(e1[:, 2:4] + e2[:, 2:4], e12[:, 2:4], rtol=1e-12, atol=1e-10)
    assert not e12[:, 0:2].any()   # no Q atom in the groups: no Q-Q pair


def test_monitor_q_against_solute_is_qp_energy(sysx):
    s = sysx
    _, EQ = oracle_eq(s, s.x)
    nonq = np.setdiff1d(np.arange(s.nat_solute), s.iqseq)
    mon = monitor_energies(s, s.x, [list(s.iqseq), list(nonq)], [(0, 1), (1, 0)])
    np.testing.assert_allclose(mon[0], EQ[:, 2:4], rtol=1e-10, atol=1e-9)
    np.testing.assert_allclose(mon[1], mon[0], rtol=1e-13, atol=1e-12)


def test_monitor_q_halves_is_qq_between_them(sysx):
    s = sysx
    lo, hi = list(s.iqseq[:2]), list(s.iqseq[2:])
    mon = monitor_energies(s, s.x, [lo, hi], [(0, 1)])[0]
    # the Q-Q energy between the halves: every Q-Q pair, less each half's own
    full = group_exclusions(s, s.x, [np.isin(np.arange(s.nat_solute), s.iqseq)])[0]
    m_lo = np.zeros(s.nat_solute, bool)
    m_lo[lo] = True
    # excluding the low half removes its internal pairs and the cross pairs;
    # the remaining energy is the high half's internal one
    exc_lo = group_exclusions(s, s.x, [m_lo])[0]
    hi_internal = full[:, 0:2] - exc_lo[:, 0:2]
    m_hi = np.zeros(s.nat_solute, bool)
    m_hi[hi] = True
    exc_hi = group_exclusions(s, s.x, [m_hi])[0]
    lo_internal = full[:, 0:2] - exc_hi[:, 0:2]
    np.testing.assert_allclose(mon, full[:, 0:2] - hi_internal - lo_internal, rtol=1e-10, atol=1e-9)


def test_monitor_pp_between_halves(sysx):
    s = sysx
    nonq = set(np.setdiff1d(np.arange(s.nat_solute), s.iqseq).tolist())
    ncg = s.ncgp_solute
    far = np.zeros(s.natom, bool)
    g1, g2 = [], []
    for g in range(ncg):
        atoms = [int(a) for a in s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1]]
        (g2 if g % 2 else g1).extend(a for a in atoms if a in nonq)
        if g % 2:
            far[atoms] = True
    E0, _ = oracle_eq(s, s.x)
    x1 = s.x.copy()
    x1[far] += 1000.0
    E1, _ = oracle_eq(s, x1)   # P-P pairs across the halves beyond every cut-off
    mon = monitor_energies(s, s.x, [g1, g2], [(0, 1)])[0]
    assert np.allclose(mon[0], mon[1])   # P-P pairs do not depend on the state
    assert mon[0, 0] == pytest.approx(E0["pp_el"] - E1["pp_el"], rel=1e-9, abs=1e-9)
    assert mon[0, 1] == pytest.approx(E0["pp_vdw"] - E1["pp_vdw"], rel=1e-9, abs=1e-9)


def test_monitor_same_atom_rejected(sysx):
    with pytest.raises(ValueError):
        monitor_energies(sysx, sysx.x, [[3, 4], [4, 5]], [(0, 1)])


def test_group_contribution_header(tmp_path):
    h = group_contribution_header([(3, "full"), (2, "all")], resid=[[10, 11, 12], [20, 21]])
    assert h.arrays == 5
    assert h.types == [NOGC, FULL, FULL, ELECTRO, VDW]
    assert h.numres == [1, 3, 2, 2, 2] and h.gcnum == [-1, 1, 2, 2, 2]
    assert h.resid == [-1, 10, 11, 12, 20, 21, 20, 21, 20, 21]
    p = tmp_path / "gc.en"
    EQ = np.arange(2 * 5 * 6, dtype=np.float64).reshape(2, 30)
    with EnergyFileWriter(p, 2, header=h) as f:
        f.write_step([0.5, 0.5], EQ)
    ef = read_energy_file(p, 2)
    assert ef.header.types == h.types and ef.header.resid == h.resid
    np.testing.assert_array_equal(ef.qq[0, :, :, 0], EQ.reshape(2, 5, 6)[:, :, 0])
    assert group_contribution_header([]).arrays == 1
