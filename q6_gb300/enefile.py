"""Qdyn energy files: the binary per-window files Qfep reads, written from
the engine's per-state Q-atom records, and Qfep's free-energy summary taken
from such files.

Layout (Fortran unformatted sequential access as gfortran writes it: every
record is framed by its payload length as a little-endian int32 before and
after the payload):

header, once (prep_sim_version, src/simprep.f90:4145-4168)
    int32 canary (137 single, 1337 double, 13337 quadruple precision),
    int32 arrays, int32 totresid, int32 types[arrays], int32 numres[arrays],
    int32 resid[totresid], int32 gcnum[arrays], char version[80]
    Without group contributions (src/simprep.f90:3787-3800): arrays 1,
    totresid 2, types [NOGC], numres [1], resid [-1, -1], gcnum [-1].

per saved step (put_ene, src/nrgy.f90:127-156), one record per state s
    int32 s (1-based), f64 lambda, f64 total[arrays],
    f64 q[arrays][4] (bond, angle, torsion, improper), f64 qx[arrays][2],
    f64 qq[arrays][2], f64 qp[arrays][2], f64 qw[arrays][2] (el, vdw),
    f64 restraint[arrays]
then one record holding the off-diagonal elements, {int32 i, j; f64 Hij,
rkl} each (OFFDIAG_SAVE, src/nrgy.f90:74-79); empty without EVB couplings.

The per-state sums follow the Q-atom energy summary of pot_energy
(src/potene.f90:224-231): qx = qq + qp + qw and
total = q.bond + q.angle + q.torsion + q.improper + qx.el + qx.vdw + restraint.
Bonded Q terms and Q restraints are outside the nonbonded engine; callers
that have them pass them in, otherwise they are written as zeros.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

from .fep import BOLTZ, qfep_dg

# group-contribution types (ENUM in src/misc.f90:33-35)
ELECTRO, VDW, FULL, NOGC = 0, 1, 2, 3
CANARY_DOUBLE = 1337
_CANARIES = (137, 1337, 13337)
VERSION_LEN = 80

# per-state record after the state index and lambda, in f64 per array
_FIELDS_PER_ARRAY = 1 + 4 + 2 + 2 + 2 + 2 + 1   # total, q(4), qx, qq, qp, qw, restraint
_OFFD = np.dtype([("i", "<i4"), ("j", "<i4"), ("Hij", "<f8"), ("rkl", "<f8")])


def _record(payload: bytes) -> bytes:
    n = struct.pack("<i", len(payload))
    return n + payload + n


@dataclass
class EnergyHeader:
    arrays: int = 1
    types: list = field(default_factory=lambda: [NOGC])
    numres: list = field(default_factory=lambda: [1])
    resid: list = field(default_factory=lambda: [-1, -1])
    gcnum: list = field(default_factory=lambda: [-1])
    version: str = "qnb"
    canary: int = CANARY_DOUBLE

    def pack(self) -> bytes:
        if not (len(self.types) == len(self.numres) == len(self.gcnum) == self.arrays) or self.arrays < 1:
            raise ValueError("header arrays do not match 'arrays'")
        v = self.version.encode("ascii")[:VERSION_LEN].ljust(VERSION_LEN, b" ")
        body = struct.pack("<3i", self.canary, self.arrays, len(self.resid))
        body += np.asarray(self.types, "<i4").tobytes() + np.asarray(self.numres, "<i4").tobytes()
        body += np.asarray(self.resid, "<i4").tobytes() + np.asarray(self.gcnum, "<i4").tobytes() + v
        return _record(body)


def group_contribution_header(groups, resid=None) -> EnergyHeader:
    """The header of a run with [group_contribution] sections
    (src/simprep.f90:3722-3808): array 1 is the whole system (NOGC), then one
    array per group with its calculation type, three (FULL, ELECTRO, VDW) for
    'all'; numres = the group's selection count, gcnum = the 1-based group,
    resid = -1 for array 1 and then each selection's residue or atom number
    (resid[g], a list per group, -1 when not given)."""
    types, numres, gcnum, res = [NOGC], [1], [-1], [-1]
    code = {"full": FULL, "electro": ELECTRO, "vdw": VDW}
    for g, (count, caltype) in enumerate(groups):
        kinds = [FULL, ELECTRO, VDW] if caltype == "all" else [code[caltype]]
        for t in kinds:
            types.append(t)
            numres.append(int(count))
            gcnum.append(g + 1)
            ids = list(resid[g]) if resid is not None else [-1] * int(count)
            res.extend(ids[:int(count)])
    if len(types) == 1:
        res = [-1, -1]
    return EnergyHeader(len(types), types, numres, res, gcnum)


def state_record(state: int, lam: float, qx_terms, q_bonded=None, restraint=None, arrays: int = 1) -> bytes:
    """One put_ene record of a state: qx_terms[arrays][6] = qq el, qq vdw,
    qp el, qp vdw, qw el, qw vdw (the engine's qnb_qenergies order);
    q_bonded[arrays][4] and restraint[arrays] default to zeros."""
    t = np.asarray(qx_terms, np.float64).reshape(arrays, 6)
    qb = np.zeros((arrays, 4)) if q_bonded is None else np.asarray(q_bonded, np.float64).reshape(arrays, 4)
    rs = np.zeros(arrays) if restraint is None else np.asarray(restraint, np.float64).reshape(arrays)
    qq, qp, qw = t[:, 0:2], t[:, 2:4], t[:, 4:6]
    qx = np.empty((arrays, 2))
    qx[:, 0] = qq[:, 0] + qp[:, 0] + qw[:, 0]
    qx[:, 1] = qq[:, 1] + qp[:, 1] + qw[:, 1]
    total = qb[:, 0] + qb[:, 1] + qb[:, 2] + qb[:, 3] + qx[:, 0] + qx[:, 1] + rs
    body = struct.pack("<id", state, lam)
    for part in (total, qb, qx, qq, qp, qw, rs):
        body += np.ascontiguousarray(part, "<f8").tobytes()
    return _record(body)


class EnergyFileWriter:
    """Writes one window's energy file: the header on open, then one step
    (all states plus the off-diagonal record) per ``write_step``."""

    def __init__(self, path, nstates: int, header: EnergyHeader | None = None):
        self.nstates = int(nstates)
        self.header = header or EnergyHeader()
        self.f = open(path, "wb")
        self.f.write(self.header.pack())

    def write_step(self, lambdas, EQ, q_bonded=None, restraint=None, offd=None):
        """EQ[nstates][arrays*6] per-state Q energies of the step (one
        window's slice of the engine's EQ output); offd: array of
        (i, j, Hij, rkl) rows or None."""
        a = self.header.arrays
        EQ = np.asarray(EQ, np.float64).reshape(self.nstates, a, 6)
        for s in range(self.nstates):
            self.f.write(state_record(s + 1, float(lambdas[s]), EQ[s],
                                      None if q_bonded is None else np.asarray(q_bonded)[s],
                                      None if restraint is None else np.asarray(restraint)[s], a))
        rows = np.zeros(0, _OFFD) if offd is None else np.array([tuple(r) for r in offd], _OFFD)
        self.f.write(_record(rows.tobytes()))

    def close(self):
        if self.f:
            self.f.close()
            self.f = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def _records(buf: bytes):
    p = 0
    while p < len(buf):
        if p + 4 > len(buf):
            raise ValueError("truncated record marker")
        (n,) = struct.unpack_from("<i", buf, p)
        if n < 0 or p + 8 + n > len(buf):
            raise ValueError("bad record length %d at byte %d" % (n, p))
        (n2,) = struct.unpack_from("<i", buf, p + 4 + n)
        if n2 != n:
            raise ValueError("record markers differ at byte %d" % p)
        yield buf[p + 4:p + 4 + n]
        p += 8 + n


@dataclass
class EnergyFile:
    header: EnergyHeader
    lambdas: np.ndarray      # [nstates] from the first step (Qfep takes them from there)
    total: np.ndarray        # [npts][nstates][arrays]
    q: np.ndarray            # [npts][nstates][arrays][4]
    qx: np.ndarray           # [npts][nstates][arrays][2]
    qq: np.ndarray
    qp: np.ndarray
    qw: np.ndarray
    restraint: np.ndarray    # [npts][nstates][arrays]
    offd: list               # per step: structured array of off-diagonal elements


def read_energy_file(path, nstates: int) -> EnergyFile:
    """Reads a file written by qdyn's put_ene (or by EnergyFileWriter) the way
    Qfep does (src/qfep.f90:259-300, get_ene src/nrgy.f90:160-200): the
    header, then steps of nstates state records and one off-diagonal record
    until the end of the file; a step cut short by the end is dropped."""
    with open(path, "rb") as f:
        recs = list(_records(f.read()))
    if not recs:
        raise ValueError("empty energy file")
    h = recs[0]
    canary, arrays, totresid = struct.unpack_from("<3i", h, 0)
    if canary not in _CANARIES:
        raise ValueError("no energy file header (canary %d)" % canary)
    if canary != CANARY_DOUBLE:
        raise ValueError("energy file precision differs from double (canary %d)" % canary)
    if arrays < 1:
        raise ValueError("number of arrays < 1")
    o = 12
    ints = lambda k: (np.frombuffer(h, "<i4", k, o).tolist(), o + 4 * k)
    types, o = ints(arrays)
    numres, o = ints(arrays)
    resid, o = ints(totresid)
    gcnum, o = ints(arrays)
    version = h[o:o + VERSION_LEN].decode("ascii", "replace").rstrip()
    header = EnergyHeader(arrays, types, numres, resid, gcnum, version, canary)
    nf = _FIELDS_PER_ARRAY * arrays
    size = 12 + 8 * nf
    steps = []
    k = 1
    while k + nstates < len(recs):
        st = []
        for s in range(nstates):
            r = recs[k + s]
            if len(r) < size:
                raise ValueError("state record of %d bytes, %d expected" % (len(r), size))
            idx, lam = struct.unpack_from("<id", r, 0)
            st.append((lam, np.frombuffer(r, "<f8", nf, 12)))
        offd = np.frombuffer(recs[k + nstates], _OFFD)
        steps.append((st, offd))
        k += nstates + 1
    npts = len(steps)
    vals = np.array([[v for _, v in st] for st, _ in steps]).reshape(npts, nstates, nf)
    lam = np.array([l for l, _ in steps[0][0]]) if npts else np.zeros(nstates)
    a = arrays
    cut = np.cumsum([0, a, 4 * a, 2 * a, 2 * a, 2 * a, 2 * a, a])
    part = lambda i: vals[:, :, cut[i]:cut[i + 1]]
    return EnergyFile(header, lam, part(0), part(1).reshape(npts, nstates, a, 4),
                      part(2).reshape(npts, nstates, a, 2), part(3).reshape(npts, nstates, a, 2),
                      part(4).reshape(npts, nstates, a, 2), part(5).reshape(npts, nstates, a, 2),
                      part(6), [o for _, o in steps])


def qfep_files(paths, nstates: int, rt: float = BOLTZ * 300.0, nskip: int = 0, gas: bool = False,
               alfa=None, array: int = 0):
    """Qfep's free-energy perturbation summary (src/qfep.f90:587-644) over the
    energy files of consecutive windows: returns (lambdas[w][s], dgf, dgr, dG)
    for group-contribution array ``array`` (0: the whole system).  ``rt`` is
    Qfep's input kT in kcal/mol; the first ``nskip`` points of every file are
    left out; ``gas`` replaces each state's total by its bonded + Q-Q +
    restraint energy (src/qfep.f90:373-380); ``alfa[s]`` shifts state s
    (alfa[0] is forced to 0 as at src/qfep.f90:448-452)."""
    shift = np.zeros(nstates) if alfa is None else np.asarray(alfa, np.float64).copy()
    shift[0] = 0.0
    files = [read_energy_file(p, nstates) for p in paths]
    v, lams = [], []
    for ef in files:
        if ef.total.shape[0] <= nskip:
            raise ValueError("file holds %d points, cannot skip %d" % (ef.total.shape[0], nskip))
        if gas:
            tot = ef.q[:, :, array].sum(-1) + ef.qq[:, :, array].sum(-1) + ef.restraint[:, :, array]
        else:
            tot = ef.total[:, :, array]
        v.append(tot[nskip:] + shift)
        lams.append(ef.lambdas)
    dgf, dgr, dg = qfep_dg(v, lams, rt)
    return np.array(lams), dgf, dgr, dg
