"""Seeded synthetic spherical systems in the layout of ``include/qnb.h``.

The nonbonded engine reads a 0-based mirror of qdyn's module globals
(``qnb_topology``).  This module builds such a model the way Qprep and qdyn's
set-up would for a spherical droplet, without any file input:

* SPC water on a seeded, jittered cubic lattice (density 0.0334 / A^3),
  O -0.82 / H +0.41, O-H 1.0 A, H-O-H 109.47 deg, random orientation.
* A solute grown as a random tree of 1.5 A bonds from the sphere centre with
  clash rejection; charge groups of consecutive atoms whose first atom is the
  switch atom; charges N(0, sigma) shifted to zero net charge per group.
* Exclusions from bonds and angles and a 1-4 list from torsion paths, with the
  semantics of Q6 src/prep.f90:1209-1271 (make14list) and 1564-1638
  (makeexlist).  In a tree the torsion ends are the atoms 3 bonds apart.
* Q atoms: a connected set of solute atoms with per-state charges and Q atom
  types (qvdw_flag on), plain soft-core alphas (Q6 src/qatom.f90:1866-1991)
  and the Q-atom connectivity matrix qconn of make_qconn/find_bonded
  (Q6 src/nonbondene.f90:3087-3187): 1 for the Q atom itself, 1 + bond count
  up to 4, else 9.

Charges are returned already scaled by sqrt(332), as qdyn holds them after
prep_sim (Q6 src/simprep.f90:3714-3721).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

COULOMB = 332.0
SQRT_COULOMB = math.sqrt(COULOMB)
WATER_DENSITY = 0.0334          # molecules / A^3
OW_A, OW_B = 629.4, 24.97       # SPC oxygen per-atom geometric LJ factors


@dataclass
class QSystem:
    natom: int
    nat_solute: int
    nwat: int
    solv_atom: int
    solvent_type: int
    x: np.ndarray              # (natom, 3) float64
    crg: np.ndarray            # (natom,) scaled
    iac: np.ndarray            # (natom,) int32
    excl: np.ndarray           # (natom,) uint8
    heavy: np.ndarray          # (natom,) uint8
    avdw: np.ndarray           # (natyps, 3)
    bvdw: np.ndarray           # (natyps, 3)
    ljcod: np.ndarray          # (natyps, natyps) uint8
    ivdw_rule: int
    el14_scale: float
    cgp_first: np.ndarray
    cgp_last: np.ndarray
    cgp_iswitch: np.ndarray
    cgpatom: np.ndarray
    ncgp_solute: int
    excl_pairs: np.ndarray     # (n, 2)
    pairs14: np.ndarray        # (n, 2)
    bonds: np.ndarray          # (n, 2) solute bonds (for reference)
    nqat: int
    nstates: int
    iqseq: np.ndarray
    qcrg: np.ndarray           # (nqat, nstates) scaled
    qiac: np.ndarray           # (nqat, nstates)
    qavdw: np.ndarray          # (nqlib, 3)
    qbvdw: np.ndarray
    qvdw_flag: int
    qq_use_library_charges: int
    sc_lookup: np.ndarray      # (nqat, natyps+nqat, nstates)
    qconn: np.ndarray          # (nstates, nat_solute, nqat) int8
    el_scale_pairs: np.ndarray  # (n, 2)
    el_scale: np.ndarray        # (n, nstates)
    qexpnb_pairs: np.ndarray    # (n, 2)
    xpcent: np.ndarray
    xwcent: np.ndarray
    rexcl_o: float
    rwat: float
    mass: np.ndarray = field(default=None)   # (natyps,)
    iuse_switch_atom: int = 1
    name: str = ""

    @property
    def natyps(self) -> int:
        return int(self.avdw.shape[0])

    @property
    def ncgp(self) -> int:
        return int(self.cgp_first.shape[0])

    def summary(self) -> dict:
        return {"name": self.name, "natom": self.natom, "nat_solute": self.nat_solute,
                "nwat": self.nwat, "ncgp": self.ncgp, "ncgp_solute": self.ncgp_solute,
                "nqat": self.nqat, "nstates": self.nstates}


# --------------------------------------------------------------------------
# ctypes mirror of qnb_topology (field order must match include/qnb.h)
# --------------------------------------------------------------------------
_P = ctypes.c_void_p


class QnbTopology(ctypes.Structure):
    _fields_ = [
        ("natom", ctypes.c_int32), ("nat_solute", ctypes.c_int32),
        ("nwat", ctypes.c_int32), ("solv_atom", ctypes.c_int32),
        ("solvent_type", ctypes.c_int32),
        ("crg", _P), ("iac", _P), ("excl", _P), ("heavy", _P),
        ("natyps", ctypes.c_int32),
        ("avdw", _P), ("bvdw", _P), ("ljcod", _P),
        ("ivdw_rule", ctypes.c_int32), ("el14_scale", ctypes.c_double),
        ("ncgp", ctypes.c_int32), ("ncgp_solute", ctypes.c_int32),
        ("cgp_first", _P), ("cgp_last", _P), ("cgp_iswitch", _P), ("cgpatom", _P),
        ("iuse_switch_atom", ctypes.c_int32),
        ("nexcl_pairs", ctypes.c_int32), ("excl_pairs", _P),
        ("n14_pairs", ctypes.c_int32), ("pairs14", _P),
        ("nqat", ctypes.c_int32), ("nstates", ctypes.c_int32),
        ("iqseq", _P), ("qcrg", _P), ("qiac", _P),
        ("nqlib", ctypes.c_int32), ("qavdw", _P), ("qbvdw", _P),
        ("qvdw_flag", ctypes.c_int32), ("qq_use_library_charges", ctypes.c_int32),
        ("sc_lookup", _P), ("qconn", _P),
        ("nel_scale", ctypes.c_int32), ("el_scale_pairs", _P), ("el_scale", _P),
        ("nqexpnb", ctypes.c_int32), ("qexpnb_pairs", _P),
        ("xpcent", ctypes.c_double * 3), ("xwcent", ctypes.c_double * 3),
        ("rexcl_o", ctypes.c_double),
    ]


class QnbSolventParams(ctypes.Structure):
    _fields_ = [
        ("fk_wsphere", ctypes.c_double), ("Dwmz", ctypes.c_double), ("awmz", ctypes.c_double),
        ("rwat", ctypes.c_double), ("boltz", ctypes.c_double),
        ("wpol_restr", ctypes.c_int32), ("nwpolr_shell", ctypes.c_int32),
        ("fkwpol", ctypes.c_double), ("itdis", ctypes.c_double),
        ("shell_rout", ctypes.c_double * 16), ("shell_dr", ctypes.c_double * 16),
        ("shell_cstb", ctypes.c_double * 16), ("theta_corr", ctypes.c_double * 16),
    ]


class TopologyHandle:
    """Owns the contiguous arrays a ``QnbTopology`` points into."""

    def __init__(self, s: QSystem):
        keep = []

        def arr(a, dt):
            a = np.ascontiguousarray(a, dtype=dt)
            keep.append(a)
            return a.ctypes.data_as(_P) if a.size else None

        t = QnbTopology()
        t.natom, t.nat_solute, t.nwat = s.natom, s.nat_solute, s.nwat
        t.solv_atom, t.solvent_type = s.solv_atom, s.solvent_type
        t.crg = arr(s.crg, np.float64)
        t.iac = arr(s.iac, np.int32)
        t.excl = arr(s.excl, np.uint8)
        t.heavy = arr(s.heavy, np.uint8)
        t.natyps = s.natyps
        t.avdw = arr(s.avdw, np.float64)
        t.bvdw = arr(s.bvdw, np.float64)
        t.ljcod = arr(s.ljcod, np.uint8)
        t.ivdw_rule, t.el14_scale = s.ivdw_rule, s.el14_scale
        t.ncgp, t.ncgp_solute = s.ncgp, s.ncgp_solute
        t.cgp_first = arr(s.cgp_first, np.int32)
        t.cgp_last = arr(s.cgp_last, np.int32)
        t.cgp_iswitch = arr(s.cgp_iswitch, np.int32)
        t.cgpatom = arr(s.cgpatom, np.int32)
        t.iuse_switch_atom = s.iuse_switch_atom
        t.nexcl_pairs = len(s.excl_pairs)
        t.excl_pairs = arr(s.excl_pairs, np.int32)
        t.n14_pairs = len(s.pairs14)
        t.pairs14 = arr(s.pairs14, np.int32)
        t.nqat, t.nstates = s.nqat, s.nstates
        t.iqseq = arr(s.iqseq, np.int32)
        # Fortran layouts: qcrg(iq,s) at iq + nqat*s
        t.qcrg = arr(np.asfortranarray(s.qcrg).ravel(order="F"), np.float64)
        t.qiac = arr(np.asfortranarray(s.qiac).ravel(order="F"), np.int32)
        t.nqlib = int(s.qavdw.shape[0])
        t.qavdw = arr(s.qavdw, np.float64)
        t.qbvdw = arr(s.qbvdw, np.float64)
        t.qvdw_flag, t.qq_use_library_charges = s.qvdw_flag, s.qq_use_library_charges
        t.sc_lookup = arr(s.sc_lookup.ravel(order="F"), np.float64)
        t.qconn = arr(s.qconn.ravel(order="F"), np.int8)
        t.nel_scale = len(s.el_scale_pairs)
        t.el_scale_pairs = arr(s.el_scale_pairs, np.int32)
        t.el_scale = arr(s.el_scale, np.float64)
        t.nqexpnb = len(s.qexpnb_pairs)
        t.qexpnb_pairs = arr(s.qexpnb_pairs, np.int32)
        for k in range(3):
            t.xpcent[k] = float(s.xpcent[k])
            t.xwcent[k] = float(s.xwcent[k])
        t.rexcl_o = s.rexcl_o
        self.struct = t
        self._keep = keep

    def ptr(self):
        return ctypes.byref(self.struct)


def default_solvent_params(s: QSystem, wpol: bool = True, fk_wsphere: float = 60.0,
                           fkwpol: float = 20.0, drout: float = 0.5,
                           wpolr_layer: float = 3.0001, itdis: float = 100.0,
                           dielectric: float = 80.0, mu_w: float | None = None,
                           crg_qtot: float = 0.0, rho_wat: float = 0.0335) -> QnbSolventParams:
    """Boundary parameters as wat_sphere / wat_shells derive them
    (Q6 src/simprep.f90:4613-4891): Dwmz/awmz "magic" defaults from the
    solvent radius, shells of widths drout, 2 drout, ... from rwat inwards,
    cstb from the Born term.  crg_qtot is wat_sphere's crgQtot (born_charge;
    0 turns the Born correction off) and mu_w its water dipole (water_dipole
    from a topology; by default -q_O b0 cos(theta0/2) of SPC geometry)."""
    p = QnbSolventParams()
    rwat = s.rwat
    p.fk_wsphere = fk_wsphere
    p.Dwmz = 0.26 * math.exp(-0.19 * (rwat - 15.0)) + 0.74
    p.awmz = 0.2 / (1.0 + math.exp(0.4 * (rwat - 25.0))) + 0.3
    p.rwat = rwat
    p.boltz = 0.001986
    p.wpol_restr = 1 if wpol else 0
    p.fkwpol = fkwpol
    p.itdis = itdis
    drs = wpolr_layer / drout
    nsh = int(-0.5 + math.sqrt(2.0 * drs + 0.25))
    nsh = max(1, min(16, nsh))
    p.nwpolr_shell = nsh
    if mu_w is None:
        # -q_O * b0 * cos(theta0/2) for SPC geometry (1.0 A, 109.47 deg)
        mu_w = 0.82 * 1.0 * math.cos(math.radians(109.47) / 2.0)
    eps = 1.0 - 1.0 / dielectric
    rout = rwat
    for i in range(nsh):
        dr = drout * (i + 1)
        ri = rout - dr
        rshell = (0.5 * (rout ** 3 + ri ** 3)) ** (1.0 / 3.0)
        p.shell_rout[i] = rout
        p.shell_dr[i] = dr
        p.shell_cstb[i] = crg_qtot * eps / (rho_wat * mu_w * 4.0 * math.pi * rshell ** 2)
        p.theta_corr[i] = 0.0
        rout = rout - dr
    return p


def born_charge(s: QSystem, lam, coulomb: float = 332.0) -> float:
    """crgQtot of wat_sphere (Q6 src/simprep.f90:4638-4646): the Q atoms'
    charges summed over states with the lambda weights, in elementary charges.
    wat_sphere runs before prep_sim scales the charges by sqrt(coulomb)
    (src/simprep.f90:3628-3631, 3714-3721), so the scaled charges held here
    are divided back.  qdyn's Born correction (charge_correction, on by
    default whenever polarisation is) uses it as default_solvent_params'
    crg_qtot; with the correction off, crg_qtot is 0."""
    lam = np.asarray(lam, dtype=np.float64)
    q = np.asarray(s.qcrg, dtype=np.float64).reshape(s.nqat, s.nstates)
    return float((q * lam[None, :]).sum() / math.sqrt(coulomb))


def water_dipole(s: QSystem, bonded, coulomb: float = 332.0) -> float:
    """mu_w of wat_shells (Q6 src/simprep.f90:4748-4751): minus the first
    solvent atom's charge (elementary charges) times b0 of the bond code of
    the topology's last bond times cos(theta0/2) of the angle code of its
    last angle.  ``bonded`` is the topology's BondedTerms (anglib in radians)
    before SHAKE removes any bond.  For a water topology whose last bond is
    the H-H constraint, as Qprep writes SPC and TIP3P, b0 is the H-H distance
    rather than O-H; this is the value qdyn's Born term uses."""
    q1 = float(s.crg[s.nat_solute]) / math.sqrt(coulomb)
    b_code = int(np.asarray(bonded.bonds)[-1][2])
    a_code = int(np.asarray(bonded.angles)[-1][3])
    return -q1 * float(bonded.bondlib[b_code][1]) * math.cos(float(bonded.anglib[a_code][1]) / 2.0)


# --------------------------------------------------------------------------
# generator
# --------------------------------------------------------------------------
def _rand_rot(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def _grow_tree(rng, n, rmax, bond=1.5, clash=2.0, max_deg=4):
    """Random tree of `n` atoms with `bond` bonds inside radius `rmax`, no two
    atoms closer than `clash`.  Compact growth: of a few random open atoms,
    the one nearest the centre is extended, so the solute fills a core and
    water the outer shell.  Atoms are then numbered in depth-first order from
    the root, so runs of consecutive atoms are bonded neighbourhoods (charge
    groups cut from them are spatially compact, as in real topologies)."""
    if n == 0:
        return np.zeros((0, 3)), np.zeros((0, 2), dtype=np.int64)
    pos = np.zeros((n, 3))
    parent = -np.ones(n, dtype=np.int64)
    deg = np.zeros(n, dtype=np.int64)
    fails = np.zeros(n, dtype=np.int64)
    cells: dict = {}

    def cell(c):
        return (int(math.floor(c[0] / clash)), int(math.floor(c[1] / clash)), int(math.floor(c[2] / clash)))

    def clashes(c, skip):
        cx, cy, cz = cell(c)
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    for j in cells.get((cx + dx, cy + dy, cz + dz), ()):
                        if j != skip and np.sum((pos[j] - c) ** 2) < clash * clash:
                            return True
        return False

    cells.setdefault(cell(pos[0]), []).append(0)
    k = 1
    tries = 0
    while k < n:
        tries += 1
        if tries > 200 * n:
            raise RuntimeError("solute growth failed: sphere too small")
        cand = rng.integers(0, k, size=6)
        cand = cand[deg[cand] < max_deg]
        if cand.size == 0:
            continue
        p = int(cand[np.argmin(np.linalg.norm(pos[cand], axis=1))])
        fails[p] += 1
        if fails[p] > 30:          # crowded atom: stop growing from it
            deg[p] = max_deg
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        c = pos[p] + bond * v
        if np.linalg.norm(c) > rmax or clashes(c, p):
            continue
        pos[k] = c
        cells.setdefault(cell(c), []).append(k)
        parent[k] = p
        deg[p] += 1
        deg[k] = 1
        k += 1
    # depth-first numbering from the root (children in creation order)
    children = [[] for _ in range(n)]
    for i in range(1, n):
        children[parent[i]].append(i)
    order, stack = [], [0]
    while stack:
        i = stack.pop()
        order.append(i)
        stack.extend(reversed(children[i]))
    new_of = np.empty(n, dtype=np.int64)
    new_of[np.array(order)] = np.arange(n)
    pos = pos[np.array(order)]
    bonds = np.array([(new_of[parent[i]], new_of[i]) for i in range(1, n)], dtype=np.int64).reshape(-1, 2)
    return pos, bonds


def _compact_groups(rng, pos, sizes_range, bonds=None, reach=4.0):
    """Charge groups as connected pieces of the solute's bond tree (bonded
    groups stay compact in dynamics; a group of unbonded neighbours can drift
    apart, and the switch-atom list test then misses its atoms' close
    contacts).  The tree is cut bottom-up: every atom collects itself and the
    still-open pieces of its children, a child's piece is closed as a group
    when adding it would pass the drawn size, and an atom's piece is closed
    once it reaches that size.  Returns the atom order with groups
    consecutive (each group in tree order), and the group sizes."""
    n = len(pos)
    adj = [[] for _ in range(n)]
    for a, b in (bonds if bonds is not None else []):
        adj[int(a)].append(int(b))
        adj[int(b)].append(int(a))
    lo, hi = sizes_range
    seen = np.zeros(n, dtype=bool)
    groups = []
    for root in range(n):   # one pass per connected component
        if seen[root]:
            continue
        parent = {root: -1}
        pre = [root]
        seen[root] = True
        stack = [root]
        while stack:   # pre-order of the component
            u = stack.pop()
            for w in sorted(adj[u], reverse=True):
                if not seen[w]:
                    seen[w] = True
                    parent[w] = u
                    pre.append(w)
                    stack.append(w)
        open_piece = {}
        target = {u: int(rng.integers(lo, hi + 1)) for u in pre}
        for u in reversed(pre):   # children before parents
            piece = [u]
            for w in adj[u]:
                if parent.get(w) == u and w in open_piece:
                    cp = open_piece.pop(w)
                    if len(piece) + len(cp) > max(target[u], hi):
                        groups.append(cp)
                    else:
                        piece.extend(cp)
            if len(piece) >= target[u]:
                groups.append(piece)
            else:
                open_piece[u] = piece
        for piece in open_piece.values():
            groups.append(piece)
    groups.sort(key=lambda g: min(g))
    order = [a for g in groups for a in sorted(g)]
    return np.array(order, dtype=np.int64), [len(g) for g in groups]


def _graph_dist(n, bonds, maxd=3):
    """All pairs within maxd bonds: dict (i<j) -> distance."""
    adj = [[] for _ in range(n)]
    for a, b in bonds:
        adj[a].append(b)
        adj[b].append(a)
    out = {}
    for s in range(n):
        frontier = [s]
        seen = {s: 0}
        for d in range(1, maxd + 1):
            nxt = []
            for u in frontier:
                for w in adj[u]:
                    if w not in seen:
                        seen[w] = d
                        nxt.append(w)
            frontier = nxt
        for w, d in seen.items():
            if w > s:
                out[(s, w)] = d
    return out, adj


def make_system(R: float = 15.0, n_solute: int = 20, group_sizes=(3, 5), ntypes: int = 6,
                nq: int = 6, nstates: int = 2, q_sigma: float = 0.3, crg_sigma: float = 0.3,
                lognormal_q: bool = False, alpha: float = 0.5, seed: int = 1,
                excl_radius: float | None = None, soft_pairs=(), el_scale=(),
                type2_pairs=((0, 1),), jitter: float = 0.25, name: str = "") -> QSystem:
    rng = np.random.default_rng(seed)
    # ---- atom types: solute types, then OW, HW --------------------------
    natyps = ntypes + 2
    avdw = np.zeros((natyps, 3))
    bvdw = np.zeros((natyps, 3))
    mass = np.zeros(natyps)
    for t in range(ntypes):
        a1 = rng.uniform(300.0, 1500.0)
        b1 = rng.uniform(5.0, 30.0)
        avdw[t] = (a1, 0.8 * a1, a1 / math.sqrt(2.0))
        bvdw[t] = (b1, 0.8 * b1, b1 / math.sqrt(2.0))
        mass[t] = rng.choice([12.01, 14.01, 16.0, 32.06])
    tOW, tHW = ntypes, ntypes + 1
    avdw[tOW] = (OW_A, OW_A, OW_A / math.sqrt(2.0))
    bvdw[tOW] = (OW_B, OW_B, OW_B / math.sqrt(2.0))
    mass[tOW], mass[tHW] = 16.0, 1.008
    ljcod = np.ones((natyps, natyps), dtype=np.uint8)
    for (ta, tb) in type2_pairs:
        if ta < ntypes and tb < ntypes:
            ljcod[ta, tb] = ljcod[tb, ta] = 2

    # ---- solute -----------------------------------------------------------
    pos, bonds = _grow_tree(rng, n_solute, rmax=max(R - 2.0, 3.0))
    # charge groups of adjacent atoms, numbered consecutively
    order, sizes = _compact_groups(rng, pos, group_sizes, bonds) if n_solute else (np.zeros(0, np.int64), [])
    new_of = np.empty(n_solute, dtype=np.int64)
    new_of[order] = np.arange(n_solute)
    pos = pos[order]
    bonds = np.sort(new_of[bonds], axis=1) if len(bonds) else bonds
    iac_s = rng.integers(0, ntypes, size=n_solute)
    crg_s = np.zeros(n_solute)
    cgp_first, cgp_last, cgp_sw = [], [], []
    k = 0
    for g in sizes:
        c = rng.normal(0.0, crg_sigma, size=g)
        c -= c.mean()
        crg_s[k:k + g] = c
        cgp_first.append(k)
        cgp_last.append(k + g - 1)
        cgp_sw.append(k)
        k += g
    ncgp_solute = len(sizes)
    gd, adj = _graph_dist(n_solute, bonds, 3)
    excl_pairs = np.array(sorted(p for p, d in gd.items() if d <= 2), dtype=np.int32).reshape(-1, 2)
    pairs14 = np.array(sorted(p for p, d in gd.items() if d == 3), dtype=np.int32).reshape(-1, 2)

    # ---- water --------------------------------------------------------------
    a = (1.0 / WATER_DENSITY) ** (1.0 / 3.0)
    m = int(math.ceil(R / a)) + 1
    g1 = np.arange(-m, m + 1) * a
    grid = np.stack(np.meshgrid(g1, g1, g1, indexing="ij"), -1).reshape(-1, 3)
    grid = grid + rng.uniform(-jitter, jitter, size=grid.shape)
    grid = grid[np.linalg.norm(grid, axis=1) <= R]
    if n_solute:
        keep = np.ones(len(grid), bool)
        for i0 in range(0, len(grid), 4096):
            blk = grid[i0:i0 + 4096]
            dmin = np.sqrt(((blk[:, None, :] - pos[None, :, :]) ** 2).sum(-1)).min(1)
            keep[i0:i0 + 4096] = dmin > 2.4
        grid = grid[keep]
    nwat = len(grid)
    th = math.radians(109.47)
    tmpl = np.array([[0.0, 0.0, 0.0],
                     [1.0, 0.0, 0.0],
                     [math.cos(th), math.sin(th), 0.0]])
    wat = np.zeros((nwat, 3, 3))
    for w in range(nwat):
        wat[w] = grid[w] + tmpl @ _rand_rot(rng).T
    natom = n_solute + 3 * nwat
    x = np.concatenate([pos, wat.reshape(-1, 3)], 0)
    crg = np.concatenate([crg_s, np.tile([-0.82, 0.41, 0.41], nwat)])
    iac = np.concatenate([iac_s, np.tile([tOW, tHW, tHW], nwat)]).astype(np.int32)
    heavy = (mass[iac] >= 4.0).astype(np.uint8)
    cgp_first = np.array(cgp_first + [n_solute + 3 * w for w in range(nwat)], dtype=np.int32)
    cgp_last = np.array(cgp_last + [n_solute + 3 * w + 2 for w in range(nwat)], dtype=np.int32)
    cgp_sw = np.array(cgp_sw + [n_solute + 3 * w for w in range(nwat)], dtype=np.int32)
    cgpatom = np.arange(natom, dtype=np.int32)
    excl = np.zeros(natom, dtype=np.uint8)
    if excl_radius is not None:
        r = np.linalg.norm(x, axis=1)
        excl[:n_solute] = r[:n_solute] > excl_radius
        wo = r[n_solute::3] > excl_radius
        excl[n_solute:] = np.repeat(wo, 3)

    # ---- Q atoms ---------------------------------------------------------
    nq = min(nq, n_solute)
    iqseq = np.arange(nq, dtype=np.int32)
    qcrg = rng.normal(0.0, q_sigma, size=(nq, nstates))
    nqlib = nq * nstates
    qiac = np.zeros((nq, nstates), dtype=np.int32)
    qavdw = np.zeros((nqlib, 3))
    qbvdw = np.zeros((nqlib, 3))
    for s in range(nstates):
        for iq in range(nq):
            t = iq + nq * s
            qiac[iq, s] = t
            base = int(rng.integers(0, ntypes))
            fa = math.exp(rng.normal(0.0, 0.25)) if lognormal_q else 1.0
            fb = math.exp(rng.normal(0.0, 0.25)) if lognormal_q else 1.0
            qavdw[t] = avdw[base] * fa
            qbvdw[t] = bvdw[base] * fb
    sc = np.zeros((nq, natyps + nq, nstates))
    for s in range(nstates):
        sc[:, :natyps, s] = alpha
        sc[:, natyps:, s] = alpha   # max(alpha_i, alpha_j) for plain alphas
    qconn = np.full((nstates, n_solute, nq), 9, dtype=np.int8)
    for iq in range(nq):
        src = int(iqseq[iq])
        qconn[:, src, iq] = 1
        for (p, q_), d in gd.items():
            if p == src:
                qconn[:, q_, iq] = d + 1
            elif q_ == src:
                qconn[:, p, iq] = d + 1
    qexp = np.array(list(soft_pairs), dtype=np.int32).reshape(-1, 2)
    elp = np.array([p for p, _ in el_scale], dtype=np.int32).reshape(-1, 2)
    elv = np.array([v for _, v in el_scale], dtype=np.float64).reshape(-1, nstates)

    return QSystem(
        natom=natom, nat_solute=n_solute, nwat=nwat, solv_atom=3, solvent_type=0,
        x=x, crg=crg * SQRT_COULOMB, iac=iac, excl=excl, heavy=heavy,
        avdw=avdw, bvdw=bvdw, ljcod=ljcod, ivdw_rule=1, el14_scale=0.5,
        cgp_first=cgp_first, cgp_last=cgp_last, cgp_iswitch=cgp_sw, cgpatom=cgpatom,
        ncgp_solute=ncgp_solute, excl_pairs=excl_pairs, pairs14=pairs14,
        bonds=bonds.astype(np.int32),
        nqat=nq, nstates=nstates, iqseq=iqseq, qcrg=qcrg * SQRT_COULOMB, qiac=qiac,
        qavdw=qavdw, qbvdw=qbvdw, qvdw_flag=1, qq_use_library_charges=0,
        sc_lookup=sc, qconn=qconn, el_scale_pairs=elp, el_scale=elv, qexpnb_pairs=qexp,
        xpcent=np.zeros(3), xwcent=np.zeros(3), rexcl_o=float(R), rwat=float(R),
        mass=mass, name=name or f"sphere_R{R:g}")


# ---- the workloads named by the benchmark configurations ------------------
def config_small(seed: int = 1000) -> QSystem:
    """R 15 A droplet (~470 SPC), 20-atom solute in groups of 3-5, 6 LJ types,
    6 Q atoms, 2 states, charges N(0, 0.3)."""
    return make_system(R=15.0, n_solute=20, group_sizes=(3, 5), ntypes=6, nq=6,
                       nstates=2, q_sigma=0.3, seed=seed, name="R15_small")


def config_window(seed: int = 2000) -> QSystem:
    """R 25 A sphere: SPC water plus a 3,000-atom solute in groups of 3-6,
    12 LJ types, 20 Q atoms, 2 states, Q charges N(0, 0.4)."""
    return make_system(R=25.0, n_solute=3000, group_sizes=(3, 6), ntypes=12, nq=20,
                       nstates=2, q_sigma=0.4, seed=seed, name="R25_window")


def config_adjoint(seed: int = 4000) -> QSystem:
    """Config-1 system with a 40-atom solute, 30 Q atoms in 4 states,
    log-normal Q LJ parameters around the 12-type table."""
    return make_system(R=15.0, n_solute=40, group_sizes=(3, 5), ntypes=12, nq=30,
                       nstates=4, q_sigma=0.4, lognormal_q=True, seed=seed,
                       name="R15_adjoint")


def config_large(seed: int = 5000) -> QSystem:
    """R 40 A sphere with an 8,000-atom solute and 40 Q atoms in 4 states."""
    return make_system(R=40.0, n_solute=8000, group_sizes=(3, 6), ntypes=12, nq=40,
                       nstates=4, q_sigma=0.4, seed=seed, name="R40_large")


def lambdas_for_window(lam: float, nstates: int) -> np.ndarray:
    """Two-state lambda vector (lam, 1-lam); extra states get zero weight."""
    out = np.zeros(nstates)
    out[0] = lam
    if nstates > 1:
        out[1] = 1.0 - lam
    return out
