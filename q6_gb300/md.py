"""Set-up of the device-resident MD step (qnb_md_*): constraints, degrees of
freedom, temperature groups and start velocities as qdyn derives them.

References (Q6 src/):
  constraint molecules     simprep.f90:2180-2380 (init_constraints; SHAKE of
                           solvent and/or solute bonds, per molecule in bond
                           order; exclshk counts half a degree of freedom per
                           excluded atom of a constrained bond)
  degrees of freedom       simprep.f90:2439-2448
  temperature groups       md.f90:470-520 (separate_scaling: solute and
                           solvent are two groups, else one)
  start velocities         simprep.f90 maxwell + initial_constraint
                           (bondene.f90:1025-1048) + stop_cm_translation
                           (simprep.f90:4496-4518)
The Maxwell draw here uses numpy's seeded generator, not qdyn's random
number stream, so start velocities match qdyn's in distribution only.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

BOLTZ = 0.001986          # kcal/(mol K), src/globals.f90:46
MAGIC_STEP_CONV = 0.020462   # fs -> internal time unit, src/globals.f90:47
MAX_TGROUPS = 4


class QnbMdParams(ctypes.Structure):
    _fields_ = [("stepsize", ctypes.c_double), ("temp0", ctypes.c_double), ("tau_t", ctypes.c_double),
                ("ndegf", ctypes.c_double), ("ndegfree", ctypes.c_double),
                ("ntgroups", ctypes.c_int32), ("nbcycle", ctypes.c_int32),
                ("tg_first", ctypes.c_int32 * MAX_TGROUPS), ("tg_last", ctypes.c_int32 * MAX_TGROUPS),
                ("tg_ndegf", ctypes.c_double * MAX_TGROUPS), ("tg_ndegfree", ctypes.c_double * MAX_TGROUPS),
                ("rq", ctypes.c_double), ("rcq", ctypes.c_double), ("rclrf", ctypes.c_double),
                ("rcpp", ctypes.c_double), ("rcpw", ctypes.c_double), ("rcww", ctypes.c_double)]


# qnb_md_record
MD_RECORD = np.dtype([("E", "<f8", 7), ("solvent_radial", "<f8"), ("water_pol", "<f8"), ("ekin", "<f8"),
                      ("temp", "<f8"), ("tfree", "<f8"), ("shake_iterations", "<f8"), ("fix", "<f8"),
                      ("shell", "<f8"), ("protein", "<f8")])


@dataclass
class MdSetup:
    stepsize: float = 1.0           # fs
    temp0: float = 300.0            # K
    tau_t: float = 100.0            # fs (bath_coupling)
    separate_scaling: bool = True   # solute and solvent coupled separately
    nbcycle: int = 25
    shake_solvent: bool = True
    shake_solute: bool = False
    shake_hydrogens: bool = True    # bonds to hydrogens (qdyn's default on)
    shake_heavy: bool = False       # heavy-atom bonds (qdyn's default off)
    cut: dict = field(default_factory=lambda: dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0))


@dataclass
class Constraints:
    mol_first: np.ndarray   # [nmol+1]
    ij: np.ndarray          # [ncons, 2]
    dist: np.ndarray        # [ncons]
    exclshk: np.ndarray     # per temperature group (filled by degrees_of_freedom)


def water_bonds(s):
    """(i, j, b0) of one solvent molecule as offsets: SPC O-H1, O-H2, H1-H2
    at the system's own geometry (its first water)."""
    if s.nwat == 0:
        return []
    o = s.nat_solute
    x = s.x[o:o + s.solv_atom]
    pairs = [(0, 1), (0, 2), (1, 2)] if s.solv_atom == 3 else \
        [(a, b) for a in range(s.solv_atom) for b in range(a + 1, s.solv_atom)]
    return [(a, b, float(np.linalg.norm(x[a] - x[b]))) for a, b in pairs]


def solute_molecules(s):
    """Connected components of the solute bond graph, as atom sets (each a
    qdyn molecule)."""
    parent = list(range(s.nat_solute))

    def root(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a

    for i, j in np.asarray(s.bonds).reshape(-1, 2):
        ri, rj = root(int(i)), root(int(j))
        if ri != rj:
            parent[max(ri, rj)] = min(ri, rj)
    comp = {}
    for a in range(s.nat_solute):
        comp.setdefault(root(a), []).append(a)
    return [comp[k] for k in sorted(comp)]


def build_constraints(s, setup: MdSetup, bonded=None) -> Constraints:
    """Constraint molecules in qdyn's order: solute molecules (bonds in
    topology order, hydrogen / heavy selection as init_constraints), then one
    molecule per water.

    With ``bonded`` (the topology's BondedTerms, redefined terms already
    removed but shaken bonds not), the constrained bonds and their lengths
    are the topology's own, as init_constraints takes them: every bond of a
    non-removed code in topology order, of length bondlib(code) b0
    (src/simprep.f90:2196-2345).  Without it, a generated system's bonds and
    water geometry give them."""
    if bonded is not None:
        return _constraints_from_topology(s, setup, bonded)
    starts, ij, dist = [0], [], []
    if setup.shake_solute and s.nat_solute:
        mass = s.mass[s.iac]
        heavy = mass >= 4.0
        by_mol = {min(m): [] for m in solute_molecules(s)}
        owner = {}
        for m in solute_molecules(s):
            for a in m:
                owner[a] = min(m)
        for i, j in np.asarray(s.bonds).reshape(-1, 2):
            i, j = int(i), int(j)
            hyd = not heavy[i] or not heavy[j]
            if (hyd and setup.shake_hydrogens) or (not hyd and setup.shake_heavy):
                by_mol[owner[i]].append((i, j, float(np.linalg.norm(s.x[i] - s.x[j]))))
        for k in sorted(by_mol):
            if by_mol[k]:
                for i, j, d in by_mol[k]:
                    ij.append((i, j))
                    dist.append(d)
                starts.append(len(ij))
    if setup.shake_solvent and s.nwat:
        hv = np.asarray(s.mass)[np.asarray(s.iac)[s.nat_solute:s.nat_solute + s.solv_atom]] >= 4.0
        wb = [(a, b, d) for a, b, d in water_bonds(s)
              if (setup.shake_hydrogens if (not hv[a] or not hv[b]) else setup.shake_heavy)]
        for w in range(s.nwat):
            o = s.nat_solute + s.solv_atom * w
            for a, b, d in wb:
                ij.append((o + a, o + b))
                dist.append(d)
            if wb:
                starts.append(len(ij))
    return Constraints(np.array(starts, np.int32), np.array(ij, np.int32).reshape(-1, 2),
                       np.array(dist, np.float64), np.zeros(MAX_TGROUPS))


def _constraints_from_topology(s, setup: MdSetup, bt) -> Constraints:
    heavy = np.asarray(s.mass)[np.asarray(s.iac)] >= 4.0
    mols = solute_molecules(s)
    owner = {}
    for m in mols:
        for a in m:
            owner[a] = min(m)
    per_mol = {}
    for i, j, c in np.asarray(bt.bonds).reshape(-1, 3).tolist():
        if c < 0:
            continue
        hyd = not heavy[i] or not heavy[j]
        pick = setup.shake_hydrogens if hyd else setup.shake_heavy
        if i < s.nat_solute:
            if not (setup.shake_solute and pick):
                continue
            key = (0, owner[i])
        else:
            if not (setup.shake_solvent and pick):
                continue
            key = (1, (i - s.nat_solute) // s.solv_atom)
        per_mol.setdefault(key, []).append((i, j, float(bt.bondlib[c][1])))
    starts, ij, dist = [0], [], []
    for key in sorted(per_mol):
        for i, j, b0 in per_mol[key]:
            ij.append((i, j))
            dist.append(b0)
        starts.append(len(ij))
    return Constraints(np.array(starts, np.int32), np.array(ij, np.int32).reshape(-1, 2),
                       np.array(dist, np.float64), np.zeros(MAX_TGROUPS))


def temperature_groups(s, setup: MdSetup):
    """(first, last) inclusive atom ranges: solute and solvent separately
    when separate_scaling and both exist, else all atoms."""
    if setup.separate_scaling and s.nat_solute > 0 and s.nwat > 0:
        return [(0, s.nat_solute - 1), (s.nat_solute, s.natom - 1)]
    return [(0, s.natom - 1)]


def degrees_of_freedom(s, cons: Constraints, groups):
    """Ndegf, Ndegfree and the per-group values (simprep.f90:2194-2253,
    2402-2448): Ndegf = 3N - constraints; Ndegfree = Ndegf - 3 nexcl +
    exclshk, exclshk adding 1/2 per excluded end of a constrained bond; a
    group counts the constraints of every molecule that overlaps its range."""
    ncons = len(cons.dist)
    excl = np.asarray(s.excl).astype(bool)
    nmol = len(cons.mol_first) - 1
    mol_lo = [int(cons.ij[cons.mol_first[m]:cons.mol_first[m + 1]].min()) for m in range(nmol)]
    mol_hi = [int(cons.ij[cons.mol_first[m]:cons.mol_first[m + 1]].max()) for m in range(nmol)]
    tg = []
    exclshk_tot = 0.0
    for a, b in groups:
        shake = sum(cons.mol_first[m + 1] - cons.mol_first[m] for m in range(nmol)
                    if mol_hi[m] >= a and mol_lo[m] <= b)
        exclshk = 0.0
        for i, j in cons.ij:
            exclshk += 0.5 * (excl[i] and a <= i <= b) + 0.5 * (excl[j] and a <= j <= b)
        exclshk_tot += exclshk
        ndegf = 3 * (b - a + 1) - shake
        nexcl = int(excl[a:b + 1].sum())
        tg.append((float(ndegf), float(int(ndegf - 3 * nexcl + exclshk))))
    ndegf = 3 * s.natom - ncons
    ndegfree = float(int(ndegf - 3 * int(excl.sum()) + exclshk_tot))
    return float(ndegf), ndegfree, tg


def md_params(s, setup: MdSetup, cons: Constraints) -> QnbMdParams:
    groups = temperature_groups(s, setup)
    ndegf, ndegfree, tg = degrees_of_freedom(s, cons, groups)
    p = QnbMdParams()
    p.stepsize, p.temp0, p.tau_t = setup.stepsize, setup.temp0, setup.tau_t
    p.ndegf, p.ndegfree = ndegf, ndegfree
    p.ntgroups, p.nbcycle = len(groups), setup.nbcycle
    for g, ((a, b), (nd, ndf)) in enumerate(zip(groups, tg)):
        p.tg_first[g], p.tg_last[g] = a, b
        p.tg_ndegf[g], p.tg_ndegfree[g] = nd, ndf
    c = setup.cut
    p.rq, p.rcq, p.rclrf = c.get("Rcq", 99.0), c.get("Rcq", 99.0), c.get("RcLRF", 99.0)
    p.rcpp, p.rcpw, p.rcww = c.get("Rcpp", 10.0), c.get("Rcpw", 10.0), c.get("Rcww", 10.0)
    return p


def maxwell_velocities(s, temperature: float, seed: int):
    """Gaussian velocities with sd sqrt(Boltz T / m) per component, in qdyn's
    internal units (A per internal time unit)."""
    rng = np.random.default_rng(seed)
    m = s.mass[s.iac]
    return rng.normal(0.0, 1.0, (s.natom, 3)) * np.sqrt(BOLTZ * temperature / m)[:, None]


def make_shell(s, rexcl_i: float, xtop=None):
    """Shell atoms of fix_shell as make_shell (switch atoms, src/topo.f90:1426-1449)
    or make_shell2 (group centres, 1455-1491) mark them: every atom of a solute
    charge group whose (non-excluded, heavy) switch atom, or whose centre in
    any-atom mode, lies beyond rexcl_i of xpcent in the topology coordinates.
    rexcl_i <= 1 is a fraction of rexcl_o (src/simprep.f90:2670-2672)."""
    xt = np.asarray(s.x if xtop is None else xtop, dtype=np.float64)
    r = float(rexcl_i)
    if r <= 1.0:
        r = r * float(s.rexcl_o)
    rin2 = r * r
    shell = np.zeros(s.natom, np.uint8)
    excl = np.asarray(s.excl).astype(bool)
    heavy = np.asarray(s.heavy).astype(bool)
    for g in range(s.ncgp_solute):
        sw = int(s.cgp_iswitch[g])
        if excl[sw] or not heavy[sw]:
            continue
        atoms = s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1]
        p = xt[sw] if s.iuse_switch_atom == 1 else xt[atoms].mean(0)
        if float(((p - s.xpcent) ** 2).sum()) > rin2:
            shell[atoms] = 1
    return shell
