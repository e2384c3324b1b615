"""Periodic box on the GPU (qnb_set_box; qdyn's *_box lists and energies)
against the oracle restatement (oracle/box.py) plus the C oracle's static
Q-Q lists, in a box small enough that pairs wrap: energies and gradient in
both forms, several windows at once; moving whole charge groups and waters
by lattice vectors changes nothing; a short MD run in the box; the
unsupported combinations fail with QNB_ERR_UNSUPPORTED / QNB_ERR_ARG.  The
box LRF, excluded atoms and solvent internal pairs in a box are in
test_gpu_box_lrf.py."""
import numpy as np
import pytest

from oracle.box import box_energies
from oracle.oracle import Oracle
from q6_gb300.md import MdSetup, maxwell_velocities
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine, QnbError
from q6_gb300.system import lambdas_for_window, make_system

pytestmark = pytest.mark.gpu
R = 11.0
BOX = [2 * R + 3.0] * 3
CUT = dict(Rcq=12.0, RcLRF=12.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
OCUT = dict(Rcq=12.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


@pytest.fixture(scope="module")
def sysb():
    return make_system(R=R, n_solute=60, group_sizes=(3, 5), ntypes=5, nq=3, nstates=2, seed=404)


def reference(s, x, lam):
    qs = int(s.iqseq[0])
    d, E, EQ = box_energies(s, x, lam, BOX, qs, OCUT)
    o = Oracle(s, use_lrf=False)
    o.set_lambda(lam)
    dq, EQs = o.nonbond_qq(x)
    o.close()
    return d + dq, E, EQ + EQs


def device(s, prec, xs, lams):
    W = len(xs)
    with NonbondedEngine(s, precision=prec, use_lrf=False, windows=W) as e:
        e.set_box(BOX)
        for w in range(W):
            e.set_lambda(lams[w], window=w)
        e.set_coordinates_dev(np.stack(xs))
        e.make_pair_lists_dev(**CUT)
        E, EQ, _ = e.compute_dev(sync=True)
        d = e.gradient_dev()
    return d, E, EQ


# the mixed form computes its pairs in FP32 (box terms and static Q lists)
@pytest.mark.parametrize("prec,tol,tolq", [(PREC_FP64, 1e-10, 1e-10), (PREC_MIXED, 1e-4, 1e-4)])
def test_box_matches_oracle(sysb, prec, tol, tolq):
    s = sysb
    rng = np.random.default_rng(9)
    xs = [s.x + rng.normal(0, 0.03, s.x.shape) for _ in range(2)]
    lams = [lambdas_for_window(0.25, 2), lambdas_for_window(0.75, 2)]
    d, E, EQ = device(s, prec, xs, lams)
    for w in range(2):
        dr, Er, EQr = reference(s, xs[w], lams[w])
        for k in Er:
            assert E[w][k] == pytest.approx(Er[k], rel=tol, abs=tol * 10), k
        np.testing.assert_allclose(EQ[w][:, 4:6], EQr[:, 4:6], rtol=tol, atol=tol * 10)
        np.testing.assert_allclose(EQ[w][:, 0:4], EQr[:, 0:4], rtol=tolq, atol=tolq * 10)
        scale = np.abs(dr).max()
        assert np.abs(d[w] - dr).max() < tolq * 10 * scale
    assert E[0]["ww_el"] != 0 and EQ[0][:, 4].any() and EQ[0][:, 2].any()


def test_lattice_moves_change_nothing(sysb):
    s = sysb
    L = np.asarray(BOX)
    rng = np.random.default_rng(1)
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
    d0, E0, EQ0 = device(s, PREC_FP64, [s.x], [lam])
    d1, E1, EQ1 = device(s, PREC_FP64, [x], [lam])
    for k in E0[0]:
        assert E1[0][k] == pytest.approx(E0[0][k], rel=1e-10, abs=1e-8), k
    np.testing.assert_allclose(EQ1, EQ0, rtol=1e-10, atol=1e-8)
    np.testing.assert_allclose(d1, d0, rtol=1e-7, atol=1e-6)


def test_md_in_box(sysb):
    s = sysb
    with NonbondedEngine(s, precision=PREC_MIXED, use_lrf=False, windows=1) as e:
        e.set_box(BOX)
        e.set_lambda([0.5, 0.5])
        e.set_coordinates_dev(s.x[None])
        e.md_init(MdSetup(stepsize=0.5, tau_t=1e12, nbcycle=5, cut=CUT))
        e.md_set_velocities(maxwell_velocities(s, 300.0, 7)[None])
        e.md_prepare(stop_cm=True)
        rec, EQ, _ = e.md_run(20)
        x, v = e.md_state(0)
    assert np.isfinite(x).all() and np.isfinite(rec["E"]).all()
    assert 0.0 < rec["temp"][-1] < 5000.0


def test_box_rejects_unsupported(sysb):
    import dataclasses
    s = sysb
    with NonbondedEngine(s, precision=PREC_FP64, use_lrf=False, windows=1) as e:
        e.set_box(BOX)
        e.set_coordinates_dev(s.x[None])
        with pytest.raises(QnbError):
            e.make_pair_lists_dev(**dict(CUT, Rcww=13.0))
        with pytest.raises(QnbError):
            e.set_box([0.0, 10.0, 10.0])
        e.set_box(None)   # back to the sphere
        e.make_pair_lists_dev(**CUT)
        e.compute_dev(sync=True)


def test_put_back_in_box(sysb):
    from oracle.box import put_back_in_box
    from q6_gb300.md import solute_molecules
    s = sysb
    L = np.asarray(BOX)
    mols = solute_molecules(s) + [list(range(s.nat_solute + 3 * w, s.nat_solute + 3 * w + 3))
                                  for w in range(s.nwat)]
    rng = np.random.default_rng(4)
    x = s.x.copy()
    # every third water one box away on each axis (a call moves a molecule by
    # at most one box length per axis, as the reference does)
    for mol in mols[len(mols) - s.nwat:][::3]:
        x[mol] += L * rng.integers(-1, 2, 3)
    mass = np.asarray(s.mass)[np.asarray(s.iac)]
    with NonbondedEngine(s, precision=PREC_FP64, use_lrf=False, windows=1) as e:
        e.set_box(BOX)
        e.set_coordinates_dev(x[None])
        e.md_init(MdSetup(cut=CUT))
        e.set_put_back_in_box()
        c = e.put_back_in_box()
        xd, _ = e.md_state(0)
    xr, cr = put_back_in_box(x, L, mols, mass, len(mols) - s.nwat, s.nat_solute)
    np.testing.assert_allclose(c[0], cr, rtol=1e-14, atol=1e-12)
    np.testing.assert_array_equal(xd, xr)
    assert np.abs(xd - x).max() > 0
    # every wrapped molecule's mass centre lies within half a box of the centre
    for mol in mols:
        cm = (xd[mol] * mass[mol][:, None]).sum(0) / mass[mol].sum()
        assert np.all(np.abs(cm - cr) <= L / 2 + 1e-9)


def test_any_atom_box_lists_match_oracle(sysb):
    import dataclasses
    s = dataclasses.replace(sysb, iuse_switch_atom=0)
    rng = np.random.default_rng(12)
    x = s.x + rng.normal(0, 0.03, s.x.shape)
    lam = lambdas_for_window(0.5, 2)
    d, E, EQ = device(s, PREC_FP64, [x], [lam])
    dr, Er, EQr = reference(s, x, lam)
    for k in Er:
        assert E[0][k] == pytest.approx(Er[k], rel=1e-10, abs=1e-9), k
    np.testing.assert_allclose(EQ[0], EQr, rtol=1e-10, atol=1e-9)
    assert np.abs(d[0] - dr).max() < 1e-9 * np.abs(dr).max()
    # more solute-water pairs than with switch atoms
    from oracle.box import box_lists
    n_any = len(box_lists(s, x, BOX, int(s.iqseq[0]), OCUT)["pw"])
    n_sw = len(box_lists(sysb, x, BOX, int(s.iqseq[0]), OCUT)["pw"])
    assert n_any > n_sw


def test_npt_volume_moves(sysb):
    # qdyn's MC_volume around the device MD (q6_gb300.pressure.run_npt): the
    # engine's potential energy equals the oracle's at the same box, and after
    # the run the lists and energies follow the final box
    from q6_gb300.pressure import PressureSetup, potential_energy, run_npt
    s = sysb
    lam = lambdas_for_window(0.5, 2)
    with NonbondedEngine(s, precision=PREC_FP64, use_lrf=False, windows=1) as e:
        e.set_box(BOX)
        e.set_lambda(lam)
        e.set_coordinates_dev(s.x[None])
        e.make_pair_lists_dev(**CUT)
        e.compute_dev(sync=True)
        dr, Er, EQr = reference(s, s.x, lam)
        u_ref = sum(Er.values()) + float(np.dot(lam, EQr.sum(1)))
        assert potential_energy(e) == pytest.approx(u_ref, rel=1e-10)
        e.md_init(MdSetup(stepsize=0.5, tau_t=100.0, nbcycle=5, cut=CUT))
        e.md_set_velocities(maxwell_velocities(s, 300.0, 3)[None])
        e.md_prepare(stop_cm=True)
        setup = PressureSetup(max_volume_displ=150.0, pressure_bar=1.0, volume_change=10, seed=11)
        rec, moves, L = run_npt(e, setup, 40, OCUT, 300.0)
        assert len(rec) == 40 and len(moves) == 3 and np.isfinite(rec["E"]).all()
        x, _ = e.md_state(0)
        e.make_pair_lists_dev(**CUT)
        e.compute_dev(sync=True)
        u_dev = potential_energy(e)
    assert np.allclose(L, e.boxlength)
    for m in moves:
        assert abs(m["dV"]) <= 150.0
    qs = int(s.iqseq[0])
    _, E1, EQ1 = box_energies(s, x, lam, L, qs, OCUT)
    o = Oracle(s, use_lrf=False)
    o.set_lambda(lam)
    _, EQs = o.nonbond_qq(x)
    o.close()
    u1 = sum(E1.values()) + float(np.dot(lam, (EQ1 + EQs).sum(1)))
    assert u_dev == pytest.approx(u1, rel=1e-9)
