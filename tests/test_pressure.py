"""Constant pressure (q6_gb300.pressure; MC_volume, src/md.f90:1976-2284) on
the CPU: the molecule scaling keeps every molecule's shape and scales its
mass centre about the box centre; the Metropolis rule on
dW = dE + P dV - nmol kB T ln(V_new/V_old) with scripted draws; a few moves
with the box oracle's energy; the cut-off check."""
import math

import numpy as np
import pytest

from oracle.box import box_energies
from q6_gb300.pressure import (BAR_TO_KCAL_MOL_A3, BOLTZ, PressureSetup, default_molecules, mc_volume_move,
                               scale_molecules)
from q6_gb300.system import make_system

CUT = dict(Rcq=11.0, Rcpp=9.0, Rcpw=9.0, Rcww=9.0)


@pytest.fixture(scope="module")
def sysp():
    return make_system(R=10.0, n_solute=30, group_sizes=(3, 5), ntypes=5, nq=3, nstates=2, seed=77)


class Draws:
    def __init__(self, values):
        self.values = list(values)

    def random(self):
        return self.values.pop(0)


def test_scaling_keeps_molecules_and_scales_centres(sysp):
    s = sysp
    mols = default_molecules(s)
    mass = np.asarray(s.mass)[np.asarray(s.iac)]
    L0, L1 = np.array([24.0] * 3), np.array([24.6] * 3)
    c = np.array([0.3, -0.2, 0.1])
    x1 = scale_molecules(s.x, mols, mass, L0, L1, c)
    for mol in mols[:5] + mols[-5:]:
        d0 = s.x[mol][:, None] - s.x[mol][None]
        d1 = x1[mol][:, None] - x1[mol][None]
        np.testing.assert_allclose(d1, d0, atol=1e-12)
        cm0 = (s.x[mol] * mass[mol][:, None]).sum(0) / mass[mol].sum()
        cm1 = (x1[mol] * mass[mol][:, None]).sum(0) / mass[mol].sum()
        np.testing.assert_allclose(cm1 - c, (cm0 - c) * L1 / L0, atol=1e-12)


def test_metropolis_rule():
    x = np.zeros((2, 3))
    mols = [[0], [1]]
    mass = np.ones(2)
    L = np.array([30.0] * 3)
    setup = PressureSetup(max_volume_displ=100.0, pressure_bar=1000.0)
    T = 300.0
    for dE in (-1.0, 0.0, 0.05, 2.0):
        for u1, u2 in ((0.9, 0.5), (0.1, 0.99), (0.5, 0.01)):
            calls = []

            def energy(xc, Lc, dE=dE, calls=calls):   # the old state first, then the trial
                calls.append(1)
                return 0.0 if len(calls) == 1 else dE
            acc, _, Ln, _, info = mc_volume_move(energy, x, L, mols, mass, np.zeros(3), setup, T, Draws([u1, u2]),
                                                 CUT)
            dV = (u1 * 2 - 1) * 100.0
            V0 = 27000.0
            dW = dE + 1000.0 * BAR_TO_KCAL_MOL_A3 * dV - 2 * BOLTZ * T * math.log((V0 + dV) / V0)
            assert info["dW"] == pytest.approx(dW, rel=1e-12, abs=1e-12)
            assert acc == (dW <= 0 or u2 <= math.exp(-dW / BOLTZ / T))
            if acc:
                assert np.prod(Ln) == pytest.approx(V0 + dV, rel=1e-12)
            else:
                assert np.array_equal(Ln, L)


def test_moves_with_the_box_oracle(sysp):
    s = sysp
    mols = default_molecules(s)
    mass = np.asarray(s.mass)[np.asarray(s.iac)]
    qs = int(s.iqseq[0])
    lam = [0.5, 0.5]

    def energy(xc, Lc):
        _, E, EQ = box_energies(s, xc, lam, Lc, qs, CUT)
        return sum(E.values()) + float(np.dot(lam, EQ.sum(1)))

    setup = PressureSetup(max_volume_displ=200.0, pressure_bar=1.0, seed=5)
    rng = np.random.default_rng(setup.seed)
    x, L = s.x.copy(), np.array([23.5] * 3)
    E = energy(x, L)
    n_acc = 0
    for _ in range(4):
        acc, x, L, E, info = mc_volume_move(energy, x, L, mols, mass, x[:s.nat_solute].mean(0), setup, 300.0,
                                            rng, CUT, E_old=E)
        n_acc += acc
        assert abs(info["dV"]) <= 200.0 and np.isfinite(E)
        assert E == pytest.approx(energy(x, L), rel=1e-12)
    with pytest.raises(ValueError):
        mc_volume_move(energy, x, np.array([18.0] * 3), mols, mass, np.zeros(3), setup, 300.0,
                       Draws([0.0, 0.5]), CUT)


class FakeNptEngine:
    """The host side of an engine as run_npt sees it: one window, a box, an
    MD set-up; md_run returns empty records and md_state the coordinates."""

    def __init__(self, s, nbcycle, cut, boxcentre=None):
        from q6_gb300.md import MdSetup
        self.s, self.nwin, self.use_lrf, self.qswitch = s, 1, False, int(s.iqseq[0])
        self.boxlength = np.array([23.5] * 3)
        self.md_setup = MdSetup(nbcycle=nbcycle, cut=cut)
        self.pb_boxcentre = None if boxcentre is None else np.asarray(boxcentre, np.float64)

    def md_run(self, n, istep):
        return np.zeros(n), None, None

    def md_state(self, w):
        return self.s.x.copy(), np.zeros_like(self.s.x)

    def set_box(self, L, qs):
        self.boxlength = np.array(L, np.float64)

    def set_coordinates_dev(self, x):
        pass


def test_npt_takes_the_md_cutoffs_nbcycle_multiple_and_rigid_centre(sysp, monkeypatch):
    """run_npt's trial energies use the MD run's cut-offs (a cut dict that
    differs is refused), volume moves come only on list-update steps
    (volume_change a multiple of nbcycle, src/md.f90:1661, 1724-1731), and the
    molecules scale about the rigid box centre given to put_back_in_box."""
    import q6_gb300.pressure as pr
    s = sysp
    mdcut = dict(Rcq=11.0, RcLRF=11.0, Rcpp=9.0, Rcpw=9.0, Rcww=9.0)
    setup = PressureSetup(max_volume_displ=100.0, volume_change=10)
    eng = FakeNptEngine(s, 5, mdcut, boxcentre=(1.0, 2.0, 3.0))
    assert pr.npt_cutoffs(eng, setup) == mdcut
    assert pr.npt_cutoffs(eng, setup, CUT) == mdcut          # RcLRF is not compared with LRF off
    with pytest.raises(ValueError, match="Rcpp"):
        pr.npt_cutoffs(eng, setup, dict(CUT, Rcpp=10.0))
    with pytest.raises(ValueError, match="nbcycle"):
        pr.npt_cutoffs(FakeNptEngine(s, 25, mdcut), setup)
    seen = []

    def fake_move(energy, x, L, molecules, mass, centre, setup_, temp0, rng, cut, E_old=None):
        seen.append((np.array(centre), dict(cut)))
        return False, x, L, 0.0, {}

    monkeypatch.setattr(pr, "mc_volume_move", fake_move)
    rec, moves, L = pr.run_npt(eng, setup, 30, temp0=300.0)
    assert len(rec) == 30 and len(moves) == 2
    for c, cut in seen:
        assert np.array_equal(c, [1.0, 2.0, 3.0]) and cut == mdcut
    seen.clear()
    pr.run_npt(FakeNptEngine(s, 5, mdcut), setup, 20, temp0=300.0)   # floating centre: the solute mean
    assert np.allclose(seen[0][0], s.x[:s.nat_solute].mean(0))
