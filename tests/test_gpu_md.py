"""Device-resident MD step (qnb_md_*) against the oracle's MD step.

FP64 form: per-step energies, temperatures and the final coordinates and
velocities of a 12-step run (list rebuilds every 5 steps, solvent restraint
with the device Tfree, watpol) within 1e-9 relative of the CPU oracle's run
(the integrator is written without fused multiply-adds, the pair sums differ
in order only).  Mixed form: within 1e-3 of the FP64 form.  Batched windows
bit-equal to single-window contexts; graph replay bit-equal to direct
launches; a SHAKE that cannot converge returns QNB_ERR_CONSTRAINT."""
import dataclasses

import numpy as np
import pytest

from oracle.oracle import Oracle, OracleMD
from q6_gb300.md import MdSetup, build_constraints, maxwell_velocities, md_params
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine, QnbError
from q6_gb300.system import default_solvent_params, lambdas_for_window, make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
SETUP = MdSetup(stepsize=1.0, temp0=300.0, tau_t=100.0, nbcycle=5, shake_solute=True, shake_heavy=True, cut=CUT)


@pytest.fixture(scope="module")
def system():
    return make_system(R=14.0, n_solute=40, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2, seed=5150)


def device_run(s, prec, nsteps, lams, setup=SETUP, graphs=True, v0=None, bonded=None, eb=None, shell=None):
    W = len(lams)
    sp = default_solvent_params(s, itdis=4.0)
    with NonbondedEngine(s, precision=prec, windows=W) as e:
        e.set_graphs(graphs)
        e.set_solvent_params(sp)
        for w in range(W):
            e.set_lambda(lams[w], window=w)
        e.set_coordinates_dev(np.stack([s.x] * W))
        if bonded is not None:
            e.set_bonded(bonded)
        if shell is not None:
            e.set_shell_restraint(*shell)
        e.md_init(setup)
        e.md_set_velocities(v0 if v0 is not None else np.stack([maxwell_velocities(s, 300.0, 11 + w)
                                                                 for w in range(W)]))
        e.md_prepare(stop_cm=True)
        rec, EQ, Eb = e.md_run(nsteps)
        st = [e.md_state(w) for w in range(W)]
    if eb is not None:
        eb.append(Eb)
    return rec, EQ, st


def test_fp64_md_matches_oracle(system):
    s = system
    lam = [0.6, 0.4]
    n = 12
    rec, EQ, st = device_run(s, PREC_FP64, n, [lam])
    sp = default_solvent_params(s, itdis=4.0)
    o = Oracle(s)
    o.set_solvent_params(sp)
    cons = build_constraints(s, SETUP)
    md = OracleMD(o, md_params(s, SETUP, cons), cons, sp=sp, lam=lam)
    x, v = md.prepare(s.x, maxwell_velocities(s, 300.0, 11))
    for k in range(n):
        r = md.step(x, v, k, CUT)
        for f, key in enumerate(("pp_el", "pp_vdw", "pw_el", "pw_vdw", "ww_el", "ww_vdw", "lrf")):
            assert abs(rec[k, 0]["E"][f] - r["E"][key]) <= 1e-9 * max(1.0, abs(r["E"][key])), (k, key)
        assert np.allclose(EQ[k, 0], r["EQ"], rtol=1e-9, atol=1e-9), k
        assert abs(rec[k, 0]["solvent_radial"] - r["erst"][0]) <= 1e-9 * max(1.0, abs(r["erst"][0])), k
        assert abs(rec[k, 0]["water_pol"] - r["erst"][1]) <= 1e-9 * max(1.0, abs(r["erst"][1])), k
        for key in ("ekin", "temp", "tfree"):
            assert abs(rec[k, 0][key] - r[key]) <= 1e-10 * abs(r[key]), (k, key)
        assert rec[k, 0]["shake_iterations"] == r["shake_iterations"], k
    xd, vd = st[0]
    assert np.allclose(xd, x, rtol=0, atol=1e-9)
    assert np.allclose(vd, v, rtol=1e-8, atol=1e-10)


def test_mixed_md_follows_fp64(system):
    s = system
    lam = [[0.6, 0.4]]
    r64, EQ64, st64 = device_run(s, PREC_FP64, 10, lam)
    r32, EQ32, st32 = device_run(s, PREC_MIXED, 10, lam)
    for k in range(10):
        assert np.allclose(r32[k, 0]["E"], r64[k, 0]["E"], rtol=1e-3, atol=1e-3), k
        assert abs(r32[k, 0]["temp"] - r64[k, 0]["temp"]) <= 1e-3 * r64[k, 0]["temp"], k
        assert np.allclose(EQ32[k], EQ64[k], rtol=1e-3, atol=1e-3), k
    assert np.abs(st32[0][0] - st64[0][0]).max() < 1e-4


def test_batched_windows_equal_single_contexts(system):
    s = system
    lams = [lambdas_for_window(l, 2) for l in (0.0, 0.5, 1.0)]
    v0 = np.stack([maxwell_velocities(s, 300.0, 11 + w) for w in range(3)])
    rb, EQb, stb = device_run(s, PREC_MIXED, 8, lams, v0=v0)
    for w in (0, 2):
        r1, EQ1, st1 = device_run(s, PREC_MIXED, 8, [lams[w]], v0=v0[w][None])
        assert np.array_equal(rb[:, w], r1[:, 0]) and np.array_equal(EQb[:, w], EQ1[:, 0]), w
        assert np.array_equal(stb[w][0], st1[0][0]) and np.array_equal(stb[w][1], st1[0][1]), w


def test_graph_replay_equals_direct_launches(system):
    s = system
    a = device_run(s, PREC_MIXED, 7, [[0.5, 0.5]], graphs=True)
    b = device_run(s, PREC_MIXED, 7, [[0.5, 0.5]], graphs=False)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[2][0][0], b[2][0][0])


def test_shake_failure_is_reported(system):
    s = system
    setup = dataclasses.replace(SETUP, shake_solute=False)
    with NonbondedEngine(s, precision=PREC_MIXED) as e:
        e.set_solvent_params(default_solvent_params(s))
        e.set_coordinates_dev(s.x[None])
        # an impossible triangle: O-H1 1 A, O-H2 1 A, H1-H2 3 A
        o = s.nat_solute
        from q6_gb300 import md as qmd
        cons = qmd.build_constraints(s, setup)
        cons.dist[2] = 3.0
        p = qmd.md_params(s, setup, cons)
        import ctypes
        mass = np.ascontiguousarray(s.mass[s.iac], dtype=np.float64)
        ij = np.ascontiguousarray(cons.ij, dtype=np.int32)
        e._check(e.lib.qnb_md_init(e.h, ctypes.byref(p), mass.ctypes.data_as(ctypes.c_void_p),
                                   len(cons.mol_first) - 1, cons.mol_first.ctypes.data_as(ctypes.c_void_p),
                                   ij.ctypes.data_as(ctypes.c_void_p), cons.dist.ctypes.data_as(ctypes.c_void_p)))
        assert cons.ij[2].tolist() == [o + 1, o + 2]
        with pytest.raises(QnbError, match="SHAKE failed in window 0, molecule 0"):
            e.md_prepare()


def test_fp64_md_with_bonded_terms_matches_oracle(system):
    """The step with solute bonded and Q bonded terms and fix_shell
    (constraints on the water only): 10 steps against the oracle's step with
    the same terms."""
    from q6_gb300.bonded import synthetic_bonded
    s = system
    lam = [0.6, 0.4]
    setup = dataclasses.replace(SETUP, shake_solute=False, stepsize=0.5)
    from q6_gb300.md import make_shell
    bt = synthetic_bonded(s, seed=21)
    shell = (s.x.copy(), make_shell(s, 3.0), 200.0, 10.0)
    eb = []
    rec, EQ, st = device_run(s, PREC_FP64, 10, [lam], setup=setup, bonded=bt, eb=eb, shell=shell)
    sp = default_solvent_params(s, itdis=4.0)
    o = Oracle(s)
    o.set_solvent_params(sp)
    cons = build_constraints(s, setup)
    md = OracleMD(o, md_params(s, setup, cons), cons, sp=sp, lam=lam, bonded=bt, shell=shell)
    x, v = md.prepare(s.x, maxwell_velocities(s, 300.0, 11))
    for k in range(10):
        r = md.step(x, v, k, CUT)
        assert np.allclose(eb[0][k, 0, :8], r["Eb"], rtol=1e-9, atol=1e-9), k
        assert np.allclose([rec[k, 0]["fix"], rec[k, 0]["shell"]], r["fix_shell"], rtol=1e-9, atol=1e-12), k
        assert np.allclose(eb[0][k, 0, 8:].reshape(2, 4), r["EQb"], rtol=1e-9, atol=1e-9), k
        assert abs(rec[k, 0]["temp"] - r["temp"]) <= 1e-10 * r["temp"], k
    assert np.allclose(st[0][0], x, rtol=0, atol=1e-9)


def test_fp64_minimize_matches_oracle(system):
    """qnb_md_minimize against the oracle's restatement of Qmin's steepest
    descent (30 steps, move cap off and on): coordinates within 1e-9 A."""
    from q6_gb300.bonded import synthetic_bonded
    s = system
    lam = [0.6, 0.4]
    setup = dataclasses.replace(SETUP, shake_solute=False)
    bt = synthetic_bonded(s, seed=22)
    sp = default_solvent_params(s, itdis=4.0)
    for cap in (0.0, 0.02):
        with NonbondedEngine(s, precision=PREC_FP64) as e:
            e.set_solvent_params(sp)
            e.set_lambda(lam)
            e.set_bonded(bt)
            e.set_coordinates_dev(s.x[None])
            e.md_init(setup)
            maxf = e.md_minimize(30, initial_step=1e-4, force_cutoff=1.0, max_move=cap)
            xd, _ = e.md_state(0)
        o = Oracle(s)
        o.set_solvent_params(sp)
        cons = build_constraints(s, setup)
        md = OracleMD(o, md_params(s, setup, cons), cons, sp=sp, lam=lam, bonded=bt)
        xo, mfo, _ = md.minimize(s.x, 30, CUT, step0=1e-4, fcut=1.0, max_move=cap)
        assert np.allclose(xd, xo, rtol=0, atol=1e-9), cap
        assert abs(maxf[0] - mfo) <= 1e-6 * mfo, cap
