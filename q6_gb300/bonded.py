"""Bonded terms for qnb_set_bonded: the topology's bond, angle, torsion and
improper lists with their libraries, and the Q-atom bonded terms of the FEP
file, as qdyn prepares them.

qdyn removes from the topology lists (src/simprep.f90:1050-1135, 2330-2345,
4395-4491): terms redefined in the FEP file ([change_bonds] etc., matched in
either atom order; impropers in the orders listed there), and bonds that
SHAKE constrains (shake_solvent / shake_solute with the hydrogen / heavy
selection of init_constraints).  ``prepare_bonded`` applies those rules;
removed terms get code -1.  Libraries are converted as topology() does
(src/simprep.f90:4547-4550): angles to radians, torsion paths inverted.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np

DEG2RAD = math.pi / 180.0   # pi = 4 atan(1), src/math.f90:621-623

I32P = ctypes.POINTER(ctypes.c_int32)
F64P = ctypes.POINTER(ctypes.c_double)


class QnbBonded(ctypes.Structure):
    _fields_ = [
        ("nbonds", ctypes.c_int32), ("nbonds_solute", ctypes.c_int32), ("bonds", I32P),
        ("nbondlib", ctypes.c_int32), ("bondlib", F64P),
        ("nangles", ctypes.c_int32), ("nangles_solute", ctypes.c_int32), ("angles", I32P),
        ("nanglib", ctypes.c_int32), ("anglib", F64P),
        ("ntors", ctypes.c_int32), ("ntors_solute", ctypes.c_int32), ("torsions", I32P),
        ("ntorlib", ctypes.c_int32), ("torlib", F64P),
        ("nimps", ctypes.c_int32), ("nimps_solute", ctypes.c_int32), ("impropers", I32P),
        ("nimplib", ctypes.c_int32), ("implib", F64P),
        ("imp_type", ctypes.c_int32), ("urey_bradley", ctypes.c_int32),
        ("nqbonds", ctypes.c_int32), ("qbonds", I32P), ("qbond_code", I32P),
        ("nqbondlib", ctypes.c_int32), ("qbondlib", F64P),
        ("nqangles", ctypes.c_int32), ("qangles", I32P), ("qangle_code", I32P),
        ("nqanglib", ctypes.c_int32), ("qanglib", F64P),
        ("nqtors", ctypes.c_int32), ("qtorsions", I32P), ("qtorsion_code", I32P),
        ("nqtorlib", ctypes.c_int32), ("qtorlib", F64P),
        ("nqimps", ctypes.c_int32), ("qimpropers", I32P), ("qimproper_code", I32P),
        ("nqimplib", ctypes.c_int32), ("qimplib", F64P),
        ("nang_coupl", ctypes.c_int32), ("ang_coupl", I32P),
        ("ntor_coupl", ctypes.c_int32), ("tor_coupl", I32P),
        ("nimp_coupl", ctypes.c_int32), ("imp_coupl", I32P),
    ]


def _i(a, w):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32).reshape(-1, w))


def _f(a, w):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, w))


@dataclass
class BondedTerms:
    """0-based atoms and codes; code -1 = removed.  Libraries in internal
    units: bondlib [fk, b0]; anglib [fk, theta0(rad), ureyfk, ureyr0];
    torlib [fk, rmult, delta(rad), 1/paths]; implib [fk, phi0(rad)];
    qbondlib [Dmz, amz, r0, fk]; qanglib as anglib; qtorlib [fk, rmult,
    delta(rad)]; qimplib [fk, phi0(rad)].  Q codes: [nterms, nstates]."""
    bonds: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    nbonds_solute: int = 0
    bondlib: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))
    angles: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))
    nangles_solute: int = 0
    anglib: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))
    torsions: np.ndarray = field(default_factory=lambda: np.zeros((0, 5), np.int32))
    ntors_solute: int = 0
    torlib: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))
    impropers: np.ndarray = field(default_factory=lambda: np.zeros((0, 5), np.int32))
    nimps_solute: int = 0
    implib: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))
    imp_type: int = 1
    urey_bradley: int = 0
    qbonds: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    qbond_code: np.ndarray = field(default_factory=lambda: np.zeros((0, 1), np.int32))
    qbondlib: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))
    qangles: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    qangle_code: np.ndarray = field(default_factory=lambda: np.zeros((0, 1), np.int32))
    qanglib: np.ndarray = field(default_factory=lambda: np.zeros((0, 4)))
    qtorsions: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))
    qtorsion_code: np.ndarray = field(default_factory=lambda: np.zeros((0, 1), np.int32))
    qtorlib: np.ndarray = field(default_factory=lambda: np.zeros((0, 3)))
    qimpropers: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.int32))
    qimproper_code: np.ndarray = field(default_factory=lambda: np.zeros((0, 1), np.int32))
    qimplib: np.ndarray = field(default_factory=lambda: np.zeros((0, 2)))
    # Morse couplings: rows (Q term, Q bond, breaking flag), 0-based
    ang_coupl: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    tor_coupl: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    imp_coupl: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))

    def to_struct(self, nstates: int):
        """(QnbBonded, keep-alive list of arrays)."""
        keep = []

        def ip(a, w):
            a = _i(a, w)
            keep.append(a)
            return a.ctypes.data_as(I32P), len(a)

        def fp(a, w):
            a = _f(a, w)
            keep.append(a)
            return a.ctypes.data_as(F64P), len(a)

        def codes(c, n):
            c = np.ascontiguousarray(np.asarray(c, np.int32).reshape(n, nstates) if n else
                                     np.zeros((0, nstates), np.int32))
            keep.append(c)
            return c.ctypes.data_as(I32P)

        b = QnbBonded()
        b.bonds, b.nbonds = ip(self.bonds, 3)
        b.nbonds_solute = self.nbonds_solute
        b.bondlib, b.nbondlib = fp(self.bondlib, 2)
        b.angles, b.nangles = ip(self.angles, 4)
        b.nangles_solute = self.nangles_solute
        b.anglib, b.nanglib = fp(self.anglib, 4)
        b.torsions, b.ntors = ip(self.torsions, 5)
        b.ntors_solute = self.ntors_solute
        b.torlib, b.ntorlib = fp(self.torlib, 4)
        b.impropers, b.nimps = ip(self.impropers, 5)
        b.nimps_solute = self.nimps_solute
        b.implib, b.nimplib = fp(self.implib, 2)
        b.imp_type, b.urey_bradley = int(self.imp_type), int(self.urey_bradley)
        b.qbonds, b.nqbonds = ip(self.qbonds, 2)
        b.qbond_code = codes(self.qbond_code, b.nqbonds)
        b.qbondlib, b.nqbondlib = fp(self.qbondlib, 4)
        b.qangles, b.nqangles = ip(self.qangles, 3)
        b.qangle_code = codes(self.qangle_code, b.nqangles)
        b.qanglib, b.nqanglib = fp(self.qanglib, 4)
        b.qtorsions, b.nqtors = ip(self.qtorsions, 4)
        b.qtorsion_code = codes(self.qtorsion_code, b.nqtors)
        b.qtorlib, b.nqtorlib = fp(self.qtorlib, 3)
        b.qimpropers, b.nqimps = ip(self.qimpropers, 4)
        b.qimproper_code = codes(self.qimproper_code, b.nqimps)
        b.qimplib, b.nqimplib = fp(self.qimplib, 2)
        b.ang_coupl, b.nang_coupl = ip(self.ang_coupl, 3)
        b.tor_coupl, b.ntor_coupl = ip(self.tor_coupl, 3)
        b.imp_coupl, b.nimp_coupl = ip(self.imp_coupl, 3)
        return b, keep


def remove_redefined(bt: BondedTerms) -> BondedTerms:
    """Topology terms redefined by Q terms get code -1 (src/simprep.f90:1050-1135,
    default force-field branch for impropers)."""
    bonds = bt.bonds.copy()
    qb = {tuple(p) for p in bt.qbonds.tolist()} | {tuple(p[::-1]) for p in bt.qbonds.tolist()}
    for k, (i, j, c) in enumerate(bonds.tolist()):
        if (i, j) in qb:
            bonds[k, 2] = -1
    angles = bt.angles.copy()
    qa = {tuple(p) for p in bt.qangles.tolist()} | {tuple(p[::-1]) for p in bt.qangles.tolist()}
    for k, (i, j, kk, c) in enumerate(angles.tolist()):
        if (i, j, kk) in qa:
            angles[k, 3] = -1
    tors = bt.torsions.copy()
    qt = {tuple(p) for p in bt.qtorsions.tolist()} | {tuple(p[::-1]) for p in bt.qtorsions.tolist()}
    for k, t in enumerate(tors.tolist()):
        if t[4] >= 0 and tuple(t[:4]) in qt:
            tors[k, 4] = -1
    imps = bt.impropers.copy()
    orders = []
    for i, j, k_, l_ in bt.qimpropers.tolist():
        orders += [(i, j, k_, l_), (k_, j, i, l_), (k_, j, l_, i), (l_, j, i, k_), (l_, j, k_, i)]
    qi = set(orders)
    for k, t in enumerate(imps.tolist()):
        if tuple(t[:4]) in qi:
            imps[k, 4] = -1
    out = BondedTerms(**{**bt.__dict__})
    out.bonds, out.angles, out.torsions, out.impropers = bonds, angles, tors, imps
    return out


def remove_shaken(bt: BondedTerms, heavy, nat_solute: int, shake_solvent=True, shake_solute=False,
                  shake_hydrogens=True, shake_heavy=False) -> BondedTerms:
    """Bonds SHAKE constrains get code -1 (src/simprep.f90:2300-2345); bonds
    already removed (code -1) are not constrained.  Then, as init_constraints
    does (src/simprep.f90:2461-2473), each constraint clears the first angle in
    list order whose end atoms (i, k) are the constrained pair: the H-O-H angle
    of a rigid water whose H-H distance is constrained contributes nothing."""
    bonds = bt.bonds.copy()
    constrained = []
    for k, (i, j, c) in enumerate(bonds.tolist()):
        if c < 0:
            continue
        hyd = not heavy[i] or not heavy[j]
        pick = (shake_hydrogens if hyd else shake_heavy)
        if (shake_solute and i < nat_solute and pick) or (shake_solvent and i >= nat_solute and pick):
            bonds[k, 2] = -1
            constrained.append((i, j))
    angles = bt.angles.copy()
    if len(angles) and constrained:
        first = {}
        for a, (i, _, k, _) in enumerate(angles.tolist()):
            first.setdefault((min(i, k), max(i, k)), a)
        for i, j in constrained:
            a = first.get((min(i, j), max(i, j)))
            if a is not None:
                angles[a, 3] = -1
    out = BondedTerms(**{**bt.__dict__})
    out.bonds = bonds
    out.angles = angles
    return out


def angles_from_bonds(bonds, natom):
    nb = [[] for _ in range(natom)]
    for i, j in bonds:
        nb[i].append(j)
        nb[j].append(i)
    out = []
    for j in range(natom):
        ns = sorted(nb[j])
        for a in range(len(ns)):
            for b in range(a + 1, len(ns)):
                out.append((ns[a], j, ns[b]))
    return out, nb


def torsions_from_bonds(bonds, nb):
    out = []
    for j, k in bonds:
        for i in nb[j]:
            if i == k:
                continue
            for l in nb[k]:
                if l == j or l == i:
                    continue
                out.append((i, j, k, l))
    return out


def synthetic_bonded(s, seed: int = 7, q_bonded: bool = True) -> BondedTerms:
    """Bonded terms for a generated system (q6_gb300.system.make_system): its
    solute bonds at their generated lengths, every angle and torsion of the
    bond graph, and one improper per branch atom, with seeded force
    constants; bond lengths, angles and impropers at their generated values
    and torsion phases that put the generated dihedrals at a minimum (the
    Q terms get per-state offsets).  With q_bonded,
    the terms whose atoms are all Q atoms move to the Q lists with per-state
    force constants (redefining the topology terms).  Waters get harmonic
    O-H / H-H bonds and an H-O-H angle."""
    rng = np.random.default_rng(seed)
    x = s.x
    nat = s.nat_solute
    sb = [tuple(map(int, b)) for b in np.asarray(s.bonds).reshape(-1, 2)]
    ang, nb = angles_from_bonds(sb, nat)
    tor = torsions_from_bonds(sb, nb)
    imp = [(ns[0], j, ns[1], ns[2]) for j in range(nat) for ns in [sorted(nb[j])] if len(ns) >= 3]

    def ang_of(i, j, k):
        a, b = x[i] - x[j], x[k] - x[j]
        return float(np.arccos(np.clip(a @ b / np.linalg.norm(a) / np.linalg.norm(b), -1, 1)))

    # the random tree has some nearly straight angles; angle_calc's gradient
    # (1/sin theta) is singular at 180 degrees and dihedrals through a straight
    # angle are undefined, so those terms are left out (force fields treat
    # linear angles separately)
    lin = np.deg2rad(160.0)
    ang = [t for t in ang if ang_of(*t) < lin]
    tor = [t for t in tor if ang_of(t[0], t[1], t[2]) < lin and ang_of(t[1], t[2], t[3]) < lin]
    imp = [t for t in imp if max(ang_of(t[0], t[1], t[2]), ang_of(t[2], t[1], t[3]), ang_of(t[0], t[1], t[3])) < lin]

    def dist(i, j):
        return float(np.linalg.norm(x[i] - x[j]))

    def angle(i, j, k):
        a, b = x[i] - x[j], x[k] - x[j]
        return float(np.arccos(np.clip(a @ b / np.linalg.norm(a) / np.linalg.norm(b), -1, 1)))

    def dihedral(i, j, k, l):   # torsion_calc's angle and sign convention
        ab, bc, cd = x[i] - x[j], x[k] - x[j], x[l] - x[k]
        c1, c2 = np.cross(ab, bc), np.cross(-bc, cd)
        phi = float(np.arccos(np.clip(c1 @ c2 / np.linalg.norm(c1) / np.linalg.norm(c2), -1, 1)))
        return -phi if bc @ np.cross(c1, c2) < 0 else phi

    def tor_min(n, phi):   # delta putting the generated dihedral at the minimum of fk (1 + cos(n phi - delta))
        return n * phi - np.pi

    bondlib = [(float(rng.uniform(300, 600)), dist(i, j)) for i, j in sb]
    bonds = [(i, j, k) for k, (i, j) in enumerate(sb)]
    anglib = [(float(rng.uniform(50, 120)), angle(i, j, k), 0.0, 0.0) for i, j, k in ang]
    angles = [(i, j, k, c) for c, (i, j, k) in enumerate(ang)]
    torlib = []
    for t in tor:
        n = float(rng.choice([1.0, 2.0, 3.0]))
        torlib.append((float(rng.uniform(0.1, 2.0)), n, tor_min(n, dihedral(*t)), 1.0))
    tors = [(i, j, k, l, c) for c, (i, j, k, l) in enumerate(tor)]
    implib = [(float(rng.uniform(5, 20)), dihedral(*t)) for t in imp]
    imps = [(i, j, k, l, c) for c, (i, j, k, l) in enumerate(imp)]
    # waters
    wb = len(bonds)
    wlib_b = len(bondlib)
    if s.nwat:
        o = nat
        bondlib += [(1000.0, dist(o, o + 1)), (0.0, dist(o + 1, o + 2))]
        wa_lib = len(anglib)
        anglib += [(100.0, angle(o + 1, o, o + 2), 0.0, 0.0)]
        for w in range(s.nwat):
            a0 = nat + 3 * w
            bonds += [(a0, a0 + 1, wlib_b), (a0, a0 + 2, wlib_b), (a0 + 1, a0 + 2, wlib_b + 1)]
            angles += [(a0 + 1, a0, a0 + 2, wa_lib)]
    bt = BondedTerms(bonds=_i(bonds, 3), nbonds_solute=wb, bondlib=_f(bondlib, 2),
                     angles=_i(angles, 4), nangles_solute=len(ang), anglib=_f(anglib, 4),
                     torsions=_i(tors, 5), ntors_solute=len(tors), torlib=_f(torlib, 4),
                     impropers=_i(imps, 5), nimps_solute=len(imps), implib=_f(implib, 2), imp_type=1)
    if q_bonded and s.nqat:
        S = s.nstates
        isq = np.zeros(s.natom, bool)
        isq[s.iqseq] = True
        qb = [(i, j) for i, j in sb if isq[i] and isq[j]]
        qa = [t for t in ang if all(isq[list(t)])]
        qt = [t for t in tor if all(isq[list(t)])]
        qi = [t for t in imp if all(isq[list(t)])]
        qbl, qal, qtl, qil = [], [], [], []
        qbc, qac, qtc, qic = [], [], [], []
        for i, j in qb:
            row = []
            for st in range(S):
                if st % 2 == 0:   # Morse in even states
                    qbl.append((float(rng.uniform(80, 120)), float(rng.uniform(1.5, 2.5)), dist(i, j), 0.0))
                else:
                    qbl.append((0.0, 0.0, dist(i, j) * float(rng.uniform(0.97, 1.03)), float(rng.uniform(300, 600))))
                row.append(len(qbl) - 1)
            qbc.append(row)
        for i, j, k in qa:
            row = []
            for st in range(S):
                qal.append((float(rng.uniform(50, 120)), angle(i, j, k) + float(rng.normal(0, 0.05)), 0.0, 0.0))
                row.append(len(qal) - 1)
            qac.append(row)
        for t in qt:
            row = []
            for st in range(S):
                n = float(rng.choice([1.0, 2.0, 3.0]))
                qtl.append((float(rng.uniform(0.1, 2.0)), n, tor_min(n, dihedral(*t)) + float(rng.normal(0, 0.2))))
                row.append(len(qtl) - 1)
            qtc.append(row)
        for t in qi:
            row = []
            for st in range(S):
                qil.append((float(rng.uniform(5, 20)), dihedral(*t) + float(rng.normal(0, 0.1))))
                row.append(len(qil) - 1)
            qic.append(row)
        bt.qbonds, bt.qbond_code, bt.qbondlib = _i(qb, 2), _i(qbc, S), _f(qbl, 4)
        bt.qangles, bt.qangle_code, bt.qanglib = _i(qa, 3), _i(qac, S), _f(qal, 4)
        bt.qtorsions, bt.qtorsion_code, bt.qtorlib = _i(qt, 4), _i(qtc, S), _f(qtl, 3)
        bt.qimpropers, bt.qimproper_code, bt.qimplib = _i(qi, 4), _i(qic, S), _f(qil, 2)
        bt = remove_redefined(bt)
    return bt
