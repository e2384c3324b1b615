"""Constant pressure for the periodic box: qdyn's Monte Carlo volume move
(MC_volume, Q6 src/md.f90:1976-2284; settings 550-572; called every
volume_change steps at a list update, 1720-1731).

A move draws dV uniformly in [-max_volume_displ, max_volume_displ], scales
the box edges by (V_new/V_old)^(1/3) and every molecule's mass centre about
the box centre (the molecules keep their shape), evaluates the potential
energy in the new box and accepts with the Metropolis rule on

    dW = dE + P dV - nmol kB T0 ln(V_new / V_old)

(P in kcal/(mol A^3): the input's bar times 1.43836e-5).  The uniform draws
come from numpy's seeded generator, not qdyn's randm stream.  The reference's
atom_based_scaling option (scaling every atom, then SHAKE) is not supported.
One box per context: run_npt wants a single-window engine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

BAR_TO_KCAL_MOL_A3 = 1.43836e-5   # src/md.f90:571
BOLTZ = 0.001986                  # src/globals.f90:46


@dataclass
class PressureSetup:
    max_volume_displ: float          # A^3 (required by qdyn)
    pressure_bar: float = 1.0
    volume_change: int = 10          # ivolume_cycle_default, src/globals.f90:231
    seed: int = 3781                 # pressure_seed default, src/md.f90:561-563
    atom_based_scaling: bool = False


def scale_molecules(x, molecules, mass, L_old, L_new, centre):
    """Moves every molecule so its mass centre scales about the box centre
    with the box (src/md.f90:2131-2143); returns the new coordinates."""
    x = np.array(x, dtype=np.float64)
    L_old = np.asarray(L_old, np.float64)
    L_new = np.asarray(L_new, np.float64)
    c = np.asarray(centre, np.float64)
    for mol in molecules:
        mol = np.asarray(mol)
        cm = (x[mol] * mass[mol][:, None]).sum(0) * (1.0 / mass[mol].sum())
        move = ((cm - c) * L_new / L_old + c) - cm
        x[mol] += move
    return x


def check_cutoffs(L, cut):
    """The box must stay larger than twice every cut-off (src/md.f90:2114-2125)."""
    box_min = float(np.min(L))
    for k in ("Rcpp", "Rcww", "Rcpw", "Rcq"):
        if k in cut and not box_min > 2.0 * cut[k]:
            raise ValueError(f"{k} cut-off too large for a box edge of {box_min:.3f} A")


def mc_volume_move(energy, x, L, molecules, mass, centre, setup: PressureSetup, temp0, rng, cut, E_old=None):
    """One MC_volume trial.  energy(x, L) is the potential energy; returns
    (accepted, x, L, E, info) with the accepted state (the old one when
    rejected)."""
    L = np.asarray(L, np.float64)
    if setup.atom_based_scaling:
        raise NotImplementedError("atom_based_scaling is not supported")
    if E_old is None:
        E_old = energy(x, L)
    V_old = float(np.prod(L))
    dV = (rng.random() * 2.0 - 1.0) * setup.max_volume_displ
    V_new = V_old + dV
    L_new = L * (V_new / V_old) ** (1.0 / 3.0)
    check_cutoffs(L_new, cut)
    x_new = scale_molecules(x, molecules, mass, L, L_new, centre)
    E_new = energy(x_new, L_new)
    P = setup.pressure_bar * BAR_TO_KCAL_MOL_A3
    dW = (E_new - E_old) + P * dV - len(molecules) * BOLTZ * temp0 * math.log(V_new / V_old)
    acc = dW <= 0.0 or not (rng.random() > math.exp(-dW / BOLTZ / temp0))
    info = dict(dV=dV, dE=E_new - E_old, dW=dW, V_new=V_new, V_old=V_old)
    if acc:
        return True, x_new, L_new, E_new, info
    return False, np.array(x, dtype=np.float64), L, E_old, info


def potential_energy(engine, window=0):
    """E%potential of the engine's last evaluation: the classical nonbonded,
    bonded and restraint energies plus the lambda-weighted Q energies."""
    E, EQ, R = engine.energies_dev()
    lam = np.asarray(engine.lambdas[window], np.float64)
    u = sum(E[window].values()) + float(lam @ EQ[window].sum(1))
    if getattr(engine, "bonded_terms", None) is not None:
        Eb, EQb = engine.bonded_energies()
        u += float(np.sum(Eb[window])) + float(lam @ np.asarray(EQb[window]).sum(1))
    Er = engine.restraint_energies()[window]
    S = engine.S
    u += float(np.sum(Er[:5])) + float(lam @ Er[5:5 + S])
    return u


def default_molecules(s):
    """The topology's molecules: the solute's bonded molecules, then each
    solvent molecule (istart_mol order)."""
    from .md import solute_molecules
    return solute_molecules(s) + [list(range(s.nat_solute + s.solv_atom * w, s.nat_solute + s.solv_atom * (w + 1)))
                                  for w in range(s.nwat)]


_CUT_DEFAULTS = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


def npt_cutoffs(engine, setup: PressureSetup, cut=None):
    """The cut-offs of the trial energies: those the MD run builds its lists
    with (the engine's MD set-up), so that a trial compares energies under the
    same lists.  A cut dict that is passed must agree with them.  qdyn tries a
    volume move only inside the list-update block of the step loop
    (src/md.f90:1661, 1724-1731), so volume_change must be a multiple of
    nbcycle."""
    md = getattr(engine, "md_setup", None)
    if md is None:
        raise ValueError("constant pressure needs an initialised MD state (md_init)")
    if setup.volume_change <= 0 or setup.volume_change % md.nbcycle != 0:
        raise ValueError(f"volume_change {setup.volume_change} is not a multiple of nbcycle {md.nbcycle}")
    mdcut = {k: md.cut.get(k, v) for k, v in _CUT_DEFAULTS.items()}
    if cut is not None:
        keys = [k for k in _CUT_DEFAULTS if k != "RcLRF" or getattr(engine, "use_lrf", True)]
        for k in keys:
            if k in cut and float(cut[k]) != float(mdcut[k]):
                raise ValueError(f"{k} = {cut[k]} differs from the MD run's {mdcut[k]}")
    return mdcut


def run_npt(engine, setup: PressureSetup, nsteps, cut=None, temp0=300.0, istep0=0, molecules=None,
            boxcentre=None):
    """Device MD (qnb_md_run) with an MC volume move every volume_change
    steps, before that step's evaluation as md_run does.  The engine holds
    one window, a periodic box (set_box) and an initialised MD state.  The
    trial energies use the MD run's cut-offs (npt_cutoffs); molecules scale
    about boxcentre, by default the rigid box centre given to
    set_put_back_in_box, else the mean of the solute atoms at the move (the
    floating centre put_back_in_box uses).
    Returns (records, per-move info dicts, final box edges)."""
    if engine.nwin != 1:
        raise ValueError("constant pressure needs a single-window engine (one box per context)")
    if getattr(engine, "boxlength", None) is None:
        raise ValueError("constant pressure needs a periodic box (set_box)")
    cut = npt_cutoffs(engine, setup, cut)
    if boxcentre is None:
        boxcentre = getattr(engine, "pb_boxcentre", None)
    s = engine.s
    molecules = molecules if molecules is not None else default_molecules(s)
    mass = np.asarray(s.mass, np.float64)[np.asarray(s.iac)]
    rng = np.random.default_rng(setup.seed)
    L = np.array(engine.boxlength, dtype=np.float64)
    qs = engine.qswitch
    recs, moves = [], []
    istep = istep0

    def energy(xc, Lc):
        engine.set_box(Lc, qs)
        engine.set_coordinates_dev(np.asarray(xc)[None])
        engine.make_pair_lists_dev(**cut)
        engine.compute_dev(istep=istep, sync=True)
        return potential_energy(engine)

    while istep < istep0 + nsteps:
        n = min(setup.volume_change - (istep % setup.volume_change), istep0 + nsteps - istep)
        rec, _, _ = engine.md_run(n, istep)
        recs.append(rec)
        istep += n
        if istep % setup.volume_change == 0 and istep < istep0 + nsteps:
            x, _ = engine.md_state(0)
            n_sol = s.nat_solute if s.nat_solute > 0 else s.natom
            centre = np.asarray(boxcentre, np.float64) if boxcentre is not None else x[:n_sol].mean(0)
            acc, xn, Ln, _, info = mc_volume_move(energy, x, L, molecules, mass, centre, setup, temp0, rng, cut)
            if not acc:   # back to the old box and coordinates; the next md_run rebuilds the lists
                engine.set_box(L, qs)
                engine.set_coordinates_dev(x[None])
            L = Ln
            info.update(accepted=acc, istep=istep, box=L.copy())
            moves.append(info)
    return np.concatenate(recs) if recs else np.zeros(0), moves, L
