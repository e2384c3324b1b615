"""Size-independent properties of the GPU path at the benchmark's full size
(the seeded 25 A, 2-state sphere: 6,060 atoms, 3,000-atom solute, 1,020 SPC
waters, 20 Q atoms; 10 A cut-offs), where the CPU oracle would take minutes:

* Newton's third law: with the LRF correction and the solvent restraints off,
  every remaining term (pp, pw, ww, qp, qw, qq) is a sum of pair forces, so
  the gradient sums to zero over the atoms; in the FP64 form to rounding
  (1e-9 of the gradient's scale), in the mixed form to the FP32 rounding of the
  per-atom sums (each pair is evaluated from both sides; 1e-5).
* Linearity in lambda: only the Q-atom gradient carries the state weights,
  d(lam) = d_nonQ + sum_s lam_s d_s, so d(0.25, 0.75) = 0.25 d(1, 0) +
  0.75 d(0, 1); and the per-state Q energies are unweighted, so they do not
  change with lambda at all (bit for bit in the mixed form, whose sums are
  fixed point).
* Translation invariance: moving every atom and both sphere centres by the
  same vector leaves the energies and the gradient unchanged up to the
  rounding of the moved coordinates.
* Permutation invariance: relabelling the water molecules (every water has
  the same parameters) maps the water-water rows onto the relabelled ones as
  sets, exactly (the cut-off decisions are FP64 on unchanged coordinates),
  and permutes the gradient, with the energies unchanged up to the order of
  the sums.
"""
import dataclasses

import numpy as np
import pytest

from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.system import config_window

pytestmark = pytest.mark.gpu

CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.fixture(scope="module")
def sphere():
    return config_window()


def _eval(s, lam, prec, x=None):
    x = s.x if x is None else x
    with NonbondedEngine(s, precision=prec, use_lrf=False) as e:
        d, E, EQ, _ = e.evaluate(x, lam, cut=CUT)
    return d, E, EQ


@pytest.mark.parametrize("prec,tol", [(PREC_FP64, 1e-9), (PREC_MIXED, 1e-5)])
def test_newton_third_law_full_size(sphere, prec, tol):
    d, E, _ = _eval(sphere, [0.4, 0.6], prec)
    scale = np.abs(d).sum(0)
    assert np.all(np.abs(d.sum(0)) <= tol * scale), (d.sum(0), scale)
    assert E["pp_el"] != 0.0 and E["ww_vdw"] != 0.0


@pytest.mark.parametrize("prec,tol", [(PREC_FP64, 1e-10), (PREC_MIXED, 1e-5)])
def test_q_gradient_linear_in_lambda_full_size(sphere, prec, tol):
    d10, _, EQ10 = _eval(sphere, [1.0, 0.0], prec)
    d01, _, EQ01 = _eval(sphere, [0.0, 1.0], prec)
    dmix, _, EQm = _eval(sphere, [0.25, 0.75], prec)
    lin = 0.25 * d10 + 0.75 * d01
    scale = np.abs(dmix).max()
    assert np.abs(dmix - lin).max() <= tol * scale
    if prec == PREC_MIXED:
        assert np.array_equal(EQ10, EQ01) and np.array_equal(EQ10, EQm)
    else:
        np.testing.assert_allclose(EQ10, EQm, rtol=1e-10, atol=1e-9)
        np.testing.assert_allclose(EQ01, EQm, rtol=1e-10, atol=1e-9)


@pytest.mark.parametrize("prec,etol,gtol", [(PREC_FP64, 1e-9, 1e-9), (PREC_MIXED, 2e-5, 2e-3)])
def test_translation_invariance_full_size(sphere, prec, etol, gtol):
    t = np.array([8.0, -4.0, 2.0])
    moved = dataclasses.replace(sphere, x=sphere.x + t, xpcent=np.asarray(sphere.xpcent) + t,
                                xwcent=np.asarray(sphere.xwcent) + t)
    d0, E0, EQ0 = _eval(sphere, [0.5, 0.5], prec)
    d1, E1, EQ1 = _eval(moved, [0.5, 0.5], prec)
    for k in E0:
        assert abs(E1[k] - E0[k]) <= etol * max(1.0, abs(E0[k])), (k, E1[k], E0[k])
    np.testing.assert_allclose(EQ1, EQ0, rtol=etol, atol=etol)
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    assert np.all(np.abs(d1 - d0) <= gtol * scale)


@pytest.mark.parametrize("prec,etol,gtol", [(PREC_FP64, 1e-9, 1e-9), (PREC_MIXED, 2e-5, 2e-3)])
def test_water_relabelling_full_size(sphere, prec, etol, gtol):
    from q6_gb300.qnb import ROWS_WW
    s = sphere
    ns, sa, W = s.nat_solute, s.solv_atom, s.nwat
    perm = np.random.default_rng(4).permutation(W)          # new water k holds old water perm[k]
    atom_map = np.arange(s.natom)
    atom_map[ns:] = (ns + sa * perm[:, None] + np.arange(sa)).reshape(-1)   # new atom -> old atom
    moved = dataclasses.replace(s, x=s.x[atom_map], excl=s.excl[atom_map])
    out = []
    for sysm in (s, moved):
        with NonbondedEngine(sysm, precision=prec, use_lrf=False) as e:
            d, E, EQ, _ = e.evaluate(sysm.x, [0.5, 0.5], cut=CUT)
            rows = None
            if prec == PREC_MIXED:
                r, p = e.export_rows(ROWS_WW, 0)
                rows = (r.astype(np.int64), p.astype(np.int64))
        out.append((d, E, EQ, rows))
    (d0, E0, EQ0, rows0), (d1, E1, EQ1, rows1) = out
    for k in E0:
        assert abs(E1[k] - E0[k]) <= etol * max(1.0, abs(E0[k])), (k, E1[k], E0[k])
    np.testing.assert_allclose(EQ1, EQ0, rtol=etol, atol=etol)
    scale = np.maximum(np.abs(d0), np.median(np.abs(d0)))
    assert np.all(np.abs(d1 - d0[atom_map]) <= gtol * scale[atom_map])
    if rows0 is not None:
        key0 = np.sort(rows0[0] * W + rows0[1])
        key1 = np.sort(perm[rows1[0]] * W + perm[rows1[1]])   # relabelled rows in the old numbering
        assert len(key0) > 0 and np.array_equal(key0, key1)
