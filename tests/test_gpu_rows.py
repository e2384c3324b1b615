"""The mixed form's gather rows, built by cell binning, equal the reference's
selections as sets.

With switch atoms on, nbpplist (src/nonbondene.f90:1777-1908) lists a solute
group pair when the FP64 distance of the two switch atoms is within Rcpp,
nbpwlist (2842-2955) a group and a water when the switch atom and the
oxygen are within Rcpw, nbwwlist (4274-4395) two waters when their oxygens
are within Rcww; excluded switch atoms / oxygens take part in none.  The
rows hold each selected pair from both sides (a group's row also holds the
group itself), Q atoms left out of the solute partners, and a group of Q
atoms only has an empty row (its atoms' pairs are the Q lists').  Expected sets are
computed here in FP64 from the coordinates (a k-d tree proposes pairs within
the cut-off plus 0.01 A, the FP64 squared distance decides); the water-water
set is also anchored to the CPU oracle's nbww list.

Cases: the benchmark droplets (R15, R25 with a 3,000-atom solute), excluded
atoms outside 13 A, a 2 A cut-off on the R25 sphere (the grid would need
more than 32,768 cells, so the cells grow), water only, unequal cut-offs
(the cells follow the largest), and a batch of three windows with different
coordinates; and in a periodic box (minimum image, wrapped stencil, or
every unit a candidate when a box edge holds fewer than 5 cells)."""
import numpy as np
import pytest

from q6_gb300.qnb import PREC_MIXED, ROWS_GP, ROWS_GW, ROWS_WG, ROWS_WW, NonbondedEngine
from q6_gb300.system import config_small, config_window, make_system

pytestmark = pytest.mark.gpu

CUT10 = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


def _pairs_within(a, b, rc, box=None):
    """(i, k) with |a_i - b_k|^2 <= rc^2 in FP64 (dx*dx + dy*dy + dz*dz); in a
    periodic box the minimum image (L nint(d / L) - d, as the box lists)."""
    from scipy.spatial import cKDTree
    if len(a) == 0 or len(b) == 0:
        return np.zeros((0, 2), np.int64)
    if box is None:
        lists = cKDTree(b).query_ball_point(a, rc + 0.01)
    else:
        L = np.asarray(box, np.float64)
        lists = cKDTree(np.mod(b, L) % L, boxsize=L).query_ball_point(np.mod(a, L) % L, rc + 0.01)
    ii = np.repeat(np.arange(len(a)), [len(v) for v in lists])
    kk = np.concatenate([np.asarray(v, np.int64) for v in lists]) if len(ii) else np.zeros(0, np.int64)
    d = a[ii] - b[kk]
    if box is not None:
        d = L * (np.sign(d / L) * np.floor(np.abs(d / L) + 0.5)) - d
    r2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]
    keep = r2 <= rc * rc
    return np.stack([ii[keep], kk[keep]], 1)


def expected_rows(s, x, Rcpp, Rcpw, Rcww, box=None):
    """Sets of (row, partner) keys of the four row kinds, in FP64 (in a box
    no atom is excluded: the box lists test no exclusion)."""
    ng, sa = s.ncgp_solute, s.solv_atom
    sw = s.cgp_iswitch[:ng].astype(np.int64)
    excl = np.zeros_like(s.excl) if box is not None else s.excl
    gin = np.nonzero(excl[sw] == 0)[0]
    oat = s.nat_solute + sa * np.arange(s.nwat)
    win = np.nonzero(excl[oat] == 0)[0]
    isq = np.zeros(s.natom, bool)
    isq[np.asarray(s.iqseq, np.int64)] = True
    # a group of Q atoms only has an empty row (its atoms' pairs are Q lists)
    allq = np.array([isq[s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1]].all() for g in range(ng)], bool)
    rows_g = np.nonzero((excl[sw] == 0) & ~allq)[0]
    out = {}
    # GP: group pairs by switch atoms (the group itself included), expanded to non-Q partner atoms
    gg = _pairs_within(x[sw[rows_g]], x[sw[gin]], Rcpp, box)
    keys = []
    for a, b in gg:
        g, g2 = rows_g[a], gin[b]
        atoms = s.cgpatom[s.cgp_first[g2]: s.cgp_last[g2] + 1]
        atoms = atoms[~isq[atoms]]
        keys.append(g * s.natom + atoms.astype(np.int64))
    out[ROWS_GP] = np.sort(np.concatenate(keys)) if keys else np.zeros(0, np.int64)
    gw = _pairs_within(x[sw[gin]], x[oat[win]], Rcpw, box)
    keep = ~allq[gin[gw[:, 0]]]
    out[ROWS_GW] = np.sort(gin[gw[keep, 0]] * s.natom + win[gw[keep, 1]])
    out[ROWS_WG] = np.sort(win[gw[:, 1]] * s.natom + gin[gw[:, 0]])
    ww = _pairs_within(x[oat[win]], x[oat[win]], Rcww, box)
    ww = ww[ww[:, 0] != ww[:, 1]]
    out[ROWS_WW] = np.sort(win[ww[:, 0]] * s.natom + win[ww[:, 1]])
    return out


def device_rows(eng, s, win=0):
    out = {}
    for kind in (ROWS_GP, ROWS_GW, ROWS_WW, ROWS_WG):
        r, p = eng.export_rows(kind, win)
        keys = r.astype(np.int64) * s.natom + p.astype(np.int64)
        assert len(np.unique(keys)) == len(keys), ("entry listed twice", kind)
        out[kind] = np.sort(keys)
    return out


def check_rows(s, cut, xs=None, box=None):
    xs = s.x[None] if xs is None else xs
    W = len(xs)
    with NonbondedEngine(s, precision=PREC_MIXED, windows=W, use_lrf=box is None) as eng:
        if box is not None:
            eng.set_box(box)
        for w in range(W):
            eng.set_lambda([0.5] * s.nstates, window=w)
        eng.set_coordinates_dev(xs)
        eng.make_pair_lists_dev(**cut)
        got = [device_rows(eng, s, w) for w in range(W)]
    for w in range(W):
        exp = expected_rows(s, xs[w], cut["Rcpp"], cut["Rcpw"], cut["Rcww"], box)
        for kind in exp:
            assert np.array_equal(got[w][kind], exp[kind]), (s.name, w, kind, len(got[w][kind]), len(exp[kind]))
    return got


def test_rows_r15_droplet_and_oracle_ww_anchor():
    from oracle.oracle import Oracle
    from q6_gb300.qnb import LIST_WW
    s = config_small()
    got = check_rows(s, CUT10)[0]
    o = Oracle(s)
    o.set_lambda([0.5, 0.5])
    o.make_pair_lists(s.x, **CUT10)
    i, j = o.export_pairs(LIST_WW)
    o.close()
    sa = s.solv_atom
    wi = (i.astype(np.int64) - s.nat_solute) // sa
    wj = (j.astype(np.int64) - s.nat_solute) // sa
    oo = np.unique(np.concatenate([wi * s.natom + wj, wj * s.natom + wi]))   # the listed water pairs, both orders
    assert np.array_equal(got[ROWS_WW], oo)


def test_rows_r25_sphere():
    check_rows(config_window(), CUT10)


def test_rows_with_excluded_atoms():
    s = make_system(R=18.0, n_solute=300, group_sizes=(3, 6), ntypes=6, nq=6, seed=31, excl_radius=13.0)
    assert s.excl.any()
    check_rows(s, CUT10)


def test_rows_small_cutoff_grows_the_cells():
    """2 A cut-offs on the R25 sphere: half-cut-off cells would number about
    50^3, more than the 32,768 a window holds."""
    check_rows(config_window(), dict(Rcq=99.0, RcLRF=99.0, Rcpp=2.0, Rcpw=2.0, Rcww=2.0))


def test_rows_water_only_and_unequal_cutoffs():
    check_rows(make_system(R=15.0, n_solute=0, nq=0, nstates=1, seed=5), CUT10)
    check_rows(config_small(), dict(Rcq=99.0, RcLRF=99.0, Rcpp=12.0, Rcpw=8.0, Rcww=9.0))


def test_rows_batch_of_windows_with_different_coordinates():
    s = config_small()
    rng = np.random.default_rng(3)
    xs = np.stack([s.x + rng.normal(0.0, 0.3, s.x.shape) for _ in range(3)])
    got = check_rows(s, CUT10, xs)
    assert not np.array_equal(got[0][ROWS_WW], got[1][ROWS_WW])


def test_rows_periodic_box_cells_and_all_candidates():
    """The box rows (switch atoms, minimum image): the R25 sphere's atoms in a
    55 A box, with cells (10 per edge) and with the excluded flags set (the
    box ignores them); and a 25 A box where 10 A cut-offs leave fewer than 5
    cells per edge, so every unit is a candidate; pairs wrap across the faces
    in both."""
    import dataclasses
    cut = dict(Rcq=12.0, RcLRF=12.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
    s = config_window()
    check_rows(s, cut, box=[55.0] * 3)
    r = np.linalg.norm(s.x - s.x.mean(0), axis=1)
    se = dataclasses.replace(s, excl=(r > 20.0).astype(np.uint8))
    check_rows(se, cut, box=[55.0] * 3)
    small = make_system(R=11.0, n_solute=60, group_sizes=(3, 5), ntypes=5, nq=3, nstates=2, seed=404)
    check_rows(small, cut, box=[25.0] * 3)
