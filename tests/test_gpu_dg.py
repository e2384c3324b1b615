"""Free-energy accuracy of the mixed form: per-window dG from Qfep's
exponential averaging (q6_gb300.fep, Q6 src/qfep.f90:587-644) on identical
frames must agree with the FP64 form within 0.02 kcal/mol per window, the
tolerance the mixed form is specified to."""
import numpy as np
import pytest

from q6_gb300.fep import BOLTZ, qfep_dg, state_energies, window_increments
from q6_gb300.qnb import PREC_FP64, PREC_MIXED, NonbondedEngine
from q6_gb300.system import default_solvent_params, lambdas_for_window, make_system

pytestmark = pytest.mark.gpu
CUT = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


def window_energies(s, prec, frames, lams):
    W, K = frames.shape[0], frames.shape[1]
    v = np.zeros((W, K, s.nstates))
    with NonbondedEngine(s, precision=prec, windows=W) as eng:
        eng.set_solvent_params(default_solvent_params(s))
        for w in range(W):
            eng.set_lambda(lams[w], window=w)
        for k in range(K):
            eng.set_coordinates_dev(frames[:, k])
            eng.make_pair_lists_dev(**CUT)
            E, EQ, R = eng.compute_dev(sync=True)
            v[:, k, :] = state_energies(EQ)
    return v


def test_mixed_dg_within_0p02_of_fp64():
    s = make_system(R=15.0, n_solute=40, group_sizes=(3, 5), ntypes=6, nq=8, nstates=2, q_sigma=0.4,
                    seed=777)
    W, K = 11, 8
    lam_w = np.linspace(0.0, 1.0, W)
    lams = np.array([lambdas_for_window(l, 2) for l in lam_w])
    rng = np.random.default_rng(3)
    frames = np.stack([np.stack([s.x + rng.normal(0, 0.05, s.x.shape) for _ in range(K)]) for _ in range(W)])
    rt = BOLTZ * 300.0
    v64 = window_energies(s, PREC_FP64, frames, lams)
    v32 = window_energies(s, PREC_MIXED, frames, lams)
    inc64 = window_increments(qfep_dg(v64, lams, rt)[2])
    inc32 = window_increments(qfep_dg(v32, lams, rt)[2])
    err = np.abs(inc32 - inc64)
    assert err.max() <= 0.02, err


def test_dg_through_energy_files(tmp_path):
    """The engine's per-state records written as qdyn energy files (one per
    window) and summed by the Qfep restatement from those files give the same
    dG as the in-memory sums, and the mixed form stays within 0.02 kcal/mol."""
    from q6_gb300.enefile import EnergyFileWriter, qfep_files
    s = make_system(R=14.0, n_solute=30, group_sizes=(3, 5), ntypes=6, nq=6, nstates=2, seed=4040)
    W, K = 5, 6
    lams = np.array([lambdas_for_window(l, 2) for l in np.linspace(0.0, 1.0, W)])
    rng = np.random.default_rng(4)
    frames = np.stack([np.stack([s.x + rng.normal(0, 0.05, s.x.shape) for _ in range(K)]) for _ in range(W)])
    rt = BOLTZ * 300.0
    inc = {}
    for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED)):
        paths = [tmp_path / ("%s_%d.en" % (name, w)) for w in range(W)]
        files = [EnergyFileWriter(p, 2) for p in paths]
        v = np.zeros((W, K, 2))
        with NonbondedEngine(s, precision=prec, windows=W) as eng:
            eng.set_solvent_params(default_solvent_params(s))
            for w in range(W):
                eng.set_lambda(lams[w], window=w)
            for k in range(K):
                eng.set_coordinates_dev(frames[:, k])
                eng.make_pair_lists_dev(**CUT)
                _, EQ, _ = eng.compute_dev(sync=True)
                v[:, k, :] = state_energies(EQ)
                for w in range(W):
                    files[w].write_step(lams[w], EQ[w])
        for f in files:
            f.close()
        _, _, _, dg = qfep_files(paths, 2, rt=rt)
        assert np.allclose(dg, qfep_dg(v, lams, rt)[2], rtol=1e-12, atol=1e-10), name
        inc[name] = window_increments(dg)
    assert np.abs(inc["mixed"] - inc["fp64"]).max() <= 0.02


def test_mixed_dg_on_fp64_md_frames():
    """The primary check of the specification: frames of each window's own
    FP64 trajectory (the device FP64 MD path at the window's lambda, 300 K,
    bonded and Q bonded terms, SHAKE) re-evaluated in both forms; per-window
    dG within 0.02 kcal/mol."""
    from q6_gb300.bonded import remove_shaken, synthetic_bonded
    from q6_gb300.md import MdSetup, maxwell_velocities
    s = make_system(R=15.0, n_solute=40, group_sizes=(3, 5), ntypes=6, nq=8, nstates=2, q_sigma=0.4,
                    seed=778)
    W, K, every, equil = 11, 20, 10, 60
    lams = np.array([lambdas_for_window(l, 2) for l in np.linspace(0.0, 1.0, W)])
    sp = default_solvent_params(s)
    bt = remove_shaken(synthetic_bonded(s, seed=5), np.asarray(s.heavy).astype(bool), s.nat_solute)
    setup = MdSetup(stepsize=1.0, temp0=300.0, tau_t=10.0, nbcycle=25, cut=dict(CUT))
    with NonbondedEngine(s, precision=PREC_MIXED, windows=W) as e:     # relax the generated start
        e.set_solvent_params(sp)
        for w in range(W):
            e.set_lambda(lams[w], window=w)
        e.set_bonded(bt)
        e.set_coordinates_dev(np.stack([s.x] * W))
        e.md_init(setup)
        e.md_minimize(1500, initial_step=1e-4, force_cutoff=1.0, max_move=0.05)
        x0 = np.stack([e.md_state(w)[0] for w in range(W)])
    frames = np.zeros((W, K, s.natom, 3))
    with NonbondedEngine(s, precision=PREC_FP64, windows=W) as e:
        e.set_solvent_params(sp)
        for w in range(W):
            e.set_lambda(lams[w], window=w)
        e.set_bonded(bt)
        e.set_coordinates_dev(x0)
        e.md_init(setup)
        e.md_set_velocities(np.stack([maxwell_velocities(s, 300.0, 40 + w) for w in range(W)]))
        e.md_prepare(stop_cm=True)
        e.md_run(equil, 0, records=False)
        for k in range(K):
            e.md_run(every, equil + k * every, records=False)
            for w in range(W):
                frames[w, k] = e.md_state(w)[0]
    assert np.all(np.isfinite(frames))
    rt = BOLTZ * 300.0
    inc = {}
    for prec in (PREC_FP64, PREC_MIXED):
        v = np.zeros((W, K, s.nstates))
        with NonbondedEngine(s, precision=prec, windows=W) as e:
            e.set_solvent_params(sp)
            e.set_bonded(bt)
            for w in range(W):
                e.set_lambda(lams[w], window=w)
            for k in range(K):
                e.set_coordinates_dev(frames[:, k])
                e.make_pair_lists_dev(**CUT)
                _, EQ, _ = e.compute_dev(sync=True)
                _, EQb = e.bonded_energies()
                v[:, k, :] = state_energies(EQ) + EQb.sum(-1)
        inc[prec] = window_increments(qfep_dg(v, lams, rt)[2])
    err = np.abs(inc[PREC_MIXED] - inc[PREC_FP64])
    assert err.max() <= 0.02, err
