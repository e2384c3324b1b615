"""Box LRF, excluded atoms and solvent internal pairs in a periodic box on
the GPU, against the box restatement (oracle/box.py: box_lrf, box_lrf_taylor,
box_energies) plus the C oracle's static Q-Q part.

The box LRF (lrf_update's lattice shift, the LRF branch of nbpplist_box_lrf /
nbpwlist_box_lrf / nbwwlist_box_lrf, lrf_taylor over all non-Q atoms) is
compared record by record (43 coefficients per group): the FP64 form within
1e-10 of each coefficient's scale, the mixed form (FP32 terms, double-float
sums) within 2e-5; energies and gradient as the other box tests.  Moving
whole groups and waters by lattice vectors leaves the LRF energy unchanged.
Excluded atoms take part in a box like any other atom (the box lists,
lrf_taylor under use_PBC and temperature() test no exclusion).  Solvent
internal pairs use the minimum image (nonbond_solvent_internal_box).  With
the switch-atom flag off the any-atom selection (nbpplis2_box_lrf /
nbpwlis2_box_lrf) feeds the moments."""
import dataclasses

import numpy as np
import pytest

from oracle.box import box_energies, box_lrf, box_lrf_taylor
from oracle.oracle import Oracle
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.system import lambdas_for_window, make_system

pytestmark = pytest.mark.gpu
R = 11.0
BOX = [2 * R + 3.0] * 3
CUT = dict(Rcq=12.0, RcLRF=12.0, Rcpp=8.0, Rcpw=8.0, Rcww=8.0)
OCUT = dict(Rcq=12.0, RcLRF=12.0, Rcpp=8.0, Rcpw=8.0, Rcww=8.0)


@pytest.fixture(scope="module")
def sysb():
    return make_system(R=R, n_solute=60, group_sizes=(3, 5), ntypes=5, nq=3, nstates=2, seed=404)


def reference(s, x, lam):
    qs = int(s.iqseq[0])
    d, E, EQ = box_energies(s, x, lam, BOX, qs, OCUT)
    rec = box_lrf(s, x, BOX, OCUT)
    elrf, dl = box_lrf_taylor(s, x, rec)
    E = dict(E, lrf=elrf)
    o = Oracle(s, use_lrf=False)
    o.set_lambda(lam)
    dq, EQs = o.nonbond_qq(x)
    o.close()
    return d + dl + dq, E, EQ + EQs, rec


def device(s, prec, xs, lams, box=BOX, nsi=None):
    W = len(xs)
    with NonbondedEngine(s, precision=prec, use_lrf=True, windows=W) as e:
        e.set_box(box)
        if nsi is not None:
            e.set_solvent_internal(*nsi)
        for w in range(W):
            e.set_lambda(lams[w], window=w)
        e.set_coordinates_dev(np.stack(xs))
        e.make_pair_lists_dev(**CUT)
        E, EQ, _ = e.compute_dev(sync=True)
        d = e.gradient_dev()
        rec = e.lrf() if W == 1 else None
    return d, E, EQ, rec


def record_scale(rec):
    """Per-coefficient scale: the largest magnitude of that coefficient over
    all groups (the centre columns excluded)."""
    return np.maximum(np.abs(rec[:, 3:]).max(0), 1e-12)


@pytest.mark.parametrize("prec,rtol,etol", [(PREC_FP64, 1e-10, 1e-10), (PREC_MIXED, 2e-5, 1e-4)])
def test_box_lrf_matches_oracle(sysb, prec, rtol, etol):
    s = sysb
    rng = np.random.default_rng(19)
    x = s.x + rng.normal(0, 0.03, s.x.shape)
    lam = lambdas_for_window(0.25, 2)
    d, E, EQ, rec = device(s, prec, [x], [lam])
    dr, Er, EQr, recr = reference(s, x, lam)
    np.testing.assert_allclose(rec[:, :3], recr[:, :3], rtol=0, atol=1e-12)
    err = np.abs(rec[:, 3:] - recr[:, 3:]) / record_scale(recr)
    assert err.max() <= rtol, (prec, err.max())
    assert abs(Er["lrf"]) > 1.0
    for k in Er:
        assert E[0][k] == pytest.approx(Er[k], rel=etol, abs=etol * 10), k
    np.testing.assert_allclose(EQ[0], EQr, rtol=etol, atol=etol * 10)
    scale = np.abs(dr).max()
    assert np.abs(d[0] - dr).max() < etol * 10 * scale


@pytest.mark.parametrize("prec,etol", [(PREC_FP64, 1e-10), (PREC_MIXED, 1e-4)])
def test_any_atom_box_lrf_matches_oracle(sysb, prec, etol):
    """Switch-atom flag off (nbpplis2_box_lrf / nbpwlis2_box_lrf): a unit pair
    feeds the LRF moments when no minimum-image atom pair is within the
    cut-off and one is within RcLRF.  The records are FP64 in both forms
    (1e-10 of each coefficient's scale); they differ from the switch-atom
    selection's on this system."""
    s = dataclasses.replace(sysb, iuse_switch_atom=0)
    rng = np.random.default_rng(23)
    x = s.x + rng.normal(0, 0.03, s.x.shape)
    lam = lambdas_for_window(0.75, 2)
    d, E, EQ, rec = device(s, prec, [x], [lam])
    dr, Er, EQr, recr = reference(s, x, lam)
    np.testing.assert_allclose(rec[:, :3], recr[:, :3], rtol=0, atol=1e-12)
    err = np.abs(rec[:, 3:] - recr[:, 3:]) / record_scale(recr)
    assert err.max() <= 1e-10, (prec, err.max())
    assert np.abs(box_lrf(sysb, x, BOX, OCUT)[:, 3:] - recr[:, 3:]).max() > 1e-6
    for k in Er:
        assert E[0][k] == pytest.approx(Er[k], rel=etol, abs=etol * 10), k
    np.testing.assert_allclose(EQ[0], EQr, rtol=etol, atol=etol * 10)
    scale = np.abs(dr).max()
    assert np.abs(d[0] - dr).max() < etol * 10 * scale


def test_box_lrf_lattice_moves_change_nothing(sysb):
    s = sysb
    L = np.asarray(BOX)
    rng = np.random.default_rng(2)
    x = s.x.copy()
    qconn = np.asarray(s.qconn)
    near = set(np.nonzero((qconn <= 3).any(axis=(0, 2)))[0].tolist()) | set(np.asarray(s.iqseq).tolist())
    for g in range(s.ncgp_solute):
        atoms = s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1]
        if not near & set(atoms.tolist()):
            x[atoms] += L * rng.integers(-2, 3, 3)
    for w in range(s.nwat):
        a = s.nat_solute + 3 * w
        x[a:a + 3] += L * rng.integers(-2, 3, 3)
    lam = lambdas_for_window(0.5, 2)
    _, E0, _, _ = device(s, PREC_FP64, [s.x], [lam])
    _, E1, _, _ = device(s, PREC_FP64, [x], [lam])
    assert E1[0]["lrf"] == pytest.approx(E0[0]["lrf"], rel=1e-9, abs=1e-8)


def test_box_excluded_atoms_take_part(sysb):
    s = sysb
    r = np.linalg.norm(s.x - s.x.mean(0), axis=1)
    excl = (r > 9.0).astype(np.uint8)
    for w in range(s.nwat):   # whole waters
        a = s.nat_solute + 3 * w
        excl[a:a + 3] = excl[a]
    assert excl.any()
    se = dataclasses.replace(s, excl=excl)
    lam = lambdas_for_window(0.5, 2)
    for prec in (PREC_FP64, PREC_MIXED):
        d0, E0, EQ0, rec0 = device(s, prec, [s.x], [lam])
        d1, E1, EQ1, rec1 = device(se, prec, [s.x], [lam])
        if prec == PREC_MIXED:   # fixed-point sums: bit for bit
            assert E1 == E0 and np.array_equal(EQ1, EQ0) and np.array_equal(d1, d0) and np.array_equal(rec1, rec0)
        else:                    # FP64 atomics: rounding follows the schedule
            for k in E0[0]:
                assert E1[0][k] == pytest.approx(E0[0][k], rel=1e-12, abs=1e-12), k
            np.testing.assert_allclose(EQ1, EQ0, rtol=1e-12, atol=1e-12)
            np.testing.assert_allclose(d1, d0, rtol=1e-10, atol=1e-10)
            np.testing.assert_allclose(rec1, rec0, rtol=1e-12, atol=1e-12)
    # and the sphere still honours the flags
    with NonbondedEngine(se, precision=PREC_FP64, use_lrf=True, windows=1) as e:
        e.set_lambda(lam)
        e.set_coordinates_dev(s.x[None])
        e.make_pair_lists_dev(**CUT)
        Es, _, _ = e.compute_dev(sync=True)
    assert Es[0]["ww_el"] != E0[0]["ww_el"]


def test_box_solvent_internal_pairs(sysb):
    """Intra-water pairs as a solvent with torsions would list them: with
    whole molecules the minimum image is the plain distance, so the box term
    equals the closed form of the pairs' Coulomb + LJ, and the rest of the
    evaluation is unchanged."""
    s = sysb
    pairs = [(1, 2)]
    A, B, el = [100.0], [10.0], [0.5]
    lam = lambdas_for_window(0.5, 2)
    d0, E0, _, _ = device(s, PREC_FP64, [s.x], [lam])
    d1, E1, _, _ = device(s, PREC_FP64, [s.x], [lam], nsi=(pairs, A, B, el))
    h1 = s.nat_solute + 3 * np.arange(s.nwat) + 1
    v = s.x[h1 + 1] - s.x[h1]
    r2 = (v * v).sum(1)
    r = np.sqrt(r2)
    eel = float((el[0] / r).sum())
    evdw = float((A[0] / r2 ** 6 - B[0] / r2 ** 3).sum())
    assert E1[0]["ww_el"] - E0[0]["ww_el"] == pytest.approx(eel, rel=1e-10)
    assert E1[0]["ww_vdw"] - E0[0]["ww_vdw"] == pytest.approx(evdw, rel=1e-10)
