"""Build tests/golden/lig_w.npz and lig_w_pbc.npz from Q6's own regression-test
inputs.

Reads tests/basic_tests/prep_SPH/lig_w.top and lig_w.fep of the Q6 tree (its
root directory is the required command-line argument) with a reader written for
the Q topology text format as Q6 src/topo.f90:471-1115 parses it, and stores
the arrays the nonbonded path needs; likewise prep_PBC (the same solute in a
49.633 A periodic box of 4,072 SPC waters, box size and centre from the
topology, the FEP file's [PBC] switching_atom).  The fixtures are what the
golden tests use; the Q6 tree is not needed at test time.

The step-0 energies that the Q6 regression test checks for the sphere
(tests/basic_tests/eval_test.sh:99 and row 1 of
SPH_leap-frog_berendsen_benchmark.en) are stored beside the arrays:
Q-surr. el 3.12, vdW 139.43 (Q-atom state 1, lambda 1), the sums of the
solute, solvent and solute-solvent rows, EL -7.30, VdW -413.17, and the
bonded columns of that row: solute bond 31.61, angle 30.69, torsion 6.28,
improper 0.05; Q-atom bond -122.04, angle 0.68, torsion 2.17, improper 0.00.
The same row's last six columns, read from the file, are the reference's
bands (mean -/+ one standard deviation over the 20 random seeds of its
benchmark runs, run_test.sh:197-440) of the step-0 total, kinetic and
potential energy: golden_tot_band, golden_kin_band, golden_pot_band.  For
the box, row 1 of PBC_leap-frog_berendsen_benchmark.en (eval_test.sh:101:
Q-surr. el -31.30, vdW 228.64; EL 380.33, VdW -1990.55; POT -1512.62 with a
zero-width band; run with q_atom 24 and lrf 24, run_test.sh:173-176).

Usage: python tests/golden/make_lig_w_fixture.py Q6_ROOT
"""
from __future__ import annotations

import os
import sys

import numpy as np

MAX_NBR_RANGE = 25  # src/topo.f90:37


class Reader:
    def __init__(self, path):
        with open(path) as f:
            self.lines = f.read().splitlines()
        self.k = 0

    def line(self):
        s = self.lines[self.k]
        self.k += 1
        return s

    def head_ints(self, n_max):
        """Leading integers of one record (list-directed read that stops at text)."""
        out = []
        for tok in self.line().split():
            try:
                out.append(int(tok))
            except ValueError:
                break
            if len(out) == n_max:
                break
        return out

    def head_floats(self, n_max):
        out = []
        for tok in self.line().split():
            try:
                out.append(float(tok))
            except ValueError:
                break
            if len(out) == n_max:
                break
        return out

    def values(self, n, conv=float):
        """List-directed read of n values spanning records."""
        out = []
        while len(out) < n:
            for tok in self.line().split():
                out.append(conv(tok))
                if len(out) == n:
                    break
        return out

    def digits(self, n):
        out = []
        while len(out) < n:
            s = self.line()
            out.extend(int(c) for c in s.strip())
        return out[:n]

    def logicals(self, n):
        out = []
        while len(out) < n:
            s = self.line().strip()
            out.extend(c in "Tt" for c in s)
        return out[:n]


def read_top(path):
    r = Reader(path)
    assert r.line().strip() == "Q topology file"
    ff_type = 1   # FF_GROMOS unless the header names another (src/topo.f90:567)
    while True:
        ln = r.line().strip()
        if ln.upper().startswith("END"):
            break
        if ln.upper().startswith("FF_TYPE"):
            ff_type = int(ln.split()[1])
    nat_pro, nat_solute = r.head_ints(2)
    solv_atom = 3
    x = np.array(r.values(3 * nat_pro), dtype=np.float64).reshape(nat_pro, 3)
    r.line()
    iac = np.array(r.values(nat_pro, int), dtype=np.int32) - 1
    nb = r.head_ints(2)
    nbonds = nb[0]
    nbonds_solute = nb[1] if len(nb) > 1 else nbonds
    bnd = np.array(r.values(3 * nbonds, int), dtype=np.int64).reshape(nbonds, 3)
    nbndcod = r.head_ints(1)[0]
    bondlib = [r.head_floats(3) for _ in range(nbndcod)]
    na = r.head_ints(2)
    nangles = na[0]
    ang = np.array(r.values(4 * nangles, int), dtype=np.int64).reshape(nangles, 4)
    nangles_solute = na[1] if len(na) > 1 else nangles
    nangcod = r.head_ints(1)[0]
    anglib = [(r.head_floats(5)[1:] + [0.0, 0.0])[:4] for _ in range(nangcod)]   # fk theta0 [ureyfk ureyr0]
    nt = r.head_ints(2)
    ntors = nt[0]
    ntors_solute = nt[1] if len(nt) > 1 else ntors
    tor = np.array(r.values(5 * ntors, int), dtype=np.int64).reshape(ntors, 5)
    ntorcod = r.head_ints(1)[0]
    torlib = [r.head_floats(5)[1:5] for _ in range(ntorcod)]   # fk rmult deltor paths
    ni = r.head_ints(2)
    nimps = ni[0]
    nimps_solute = ni[1] if len(ni) > 1 else nimps
    imp = np.array(r.values(5 * nimps, int), dtype=np.int64).reshape(nimps, 5)
    nic = r.head_ints(2)
    nimpcod = nic[0]
    imp_type = nic[1] if len(nic) > 1 else 1
    implib = [r.head_floats(3)[1:3] for _ in range(nimpcod)]   # fk imp0
    nq = r.head_ints(1)[0]
    crg = np.array(r.values(nq), dtype=np.float64)
    cg = r.head_ints(3)
    ncgp, ncgp_solute = cg[0], cg[1]
    iuse_switch = cg[2] if len(cg) > 2 else 1
    first, last, sw, atoms = [], [], [], []
    k = 0
    for _ in range(ncgp):
        n, isw = r.values(2, int)
        members = r.values(n, int)
        first.append(k)
        last.append(k + n - 1)
        sw.append(isw - 1)
        atoms.extend(m - 1 for m in members)
        k += n
    natyps = r.head_ints(1)[0]
    ivdw_rule = r.head_ints(1)[0]
    el14_scale, coulomb = r.head_floats(2)
    r.line()
    mass = np.array(r.values(natyps), dtype=np.float64)
    avdw = np.zeros((natyps, 3))
    bvdw = np.zeros((natyps, 3))
    for j in range(3):
        r.line()
        avdw[:, j] = r.values(natyps)
        r.line()
        bvdw[:, j] = r.values(natyps)
    nlj2 = r.head_ints(1)[0]
    lj2 = [r.values(2, int) for _ in range(nlj2)]
    r.head_ints(1)
    l14 = np.array(r.digits(MAX_NBR_RANGE * nat_solute)).reshape(nat_solute, MAX_NBR_RANGE)
    n14long = r.head_ints(1)[0]
    p14long = [r.values(2, int) for _ in range(n14long)]
    r.head_ints(1)
    lex = np.array(r.digits(MAX_NBR_RANGE * nat_solute)).reshape(nat_solute, MAX_NBR_RANGE)
    nexlong = r.head_ints(1)[0]
    pexlong = [r.values(2, int) for _ in range(nexlong)]
    # skip residue / molecule / type-name blocks up to the solvent type record
    while "solvent type" not in r.lines[r.k]:
        r.k += 1
    solvent_type = r.head_ints(1)[0]
    boxl = boxc = None
    if "PBC" in r.lines[r.k] and "boundary" in r.lines[r.k]:   # src/topo.f90: box size and centre, no exclusions
        r.line()
        boxl = np.array(r.head_floats(3))
        boxc = np.array(r.head_floats(3))
        rexcl_o = rwat = 0.0
        xpcent = xwcent = boxc.copy()
        excl = np.zeros(nat_pro, dtype=np.uint8)
    else:
        rexcl_o, rwat = r.head_floats(2)
        xpcent = np.array(r.head_floats(3))
        xwcent = np.array(r.head_floats(3))
        nexats, nexwat = r.head_ints(2)
        excl = np.array(r.logicals(nat_pro), dtype=np.uint8)

    pairs14 = [(i, i + o + 1) for i in range(nat_solute) for o in range(MAX_NBR_RANGE) if l14[i, o]]
    pairs14 += [(a - 1, b - 1) for a, b in p14long]
    expairs = [(i, i + o + 1) for i in range(nat_solute) for o in range(MAX_NBR_RANGE) if lex[i, o]]
    expairs += [(a - 1, b - 1) for a, b in pexlong]
    ljcod = np.ones((natyps, natyps), dtype=np.uint8)
    for a, b in lj2:
        ljcod[a - 1, b - 1] = ljcod[b - 1, a - 1] = 2
    return dict(
        natom=nat_pro, nat_solute=nat_solute, solv_atom=solv_atom, x=x, iac=iac,
        bonds=bnd[:nbonds_solute, :2] - 1, bond_codes=bnd[:nbonds_solute, 2],
        crg=crg, coulomb=coulomb,
        cgp_first=np.array(first, np.int32), cgp_last=np.array(last, np.int32),
        cgp_iswitch=np.array(sw, np.int32), cgpatom=np.array(atoms, np.int32),
        ncgp_solute=ncgp_solute, iuse_switch_atom=iuse_switch,
        mass=mass, avdw=avdw, bvdw=bvdw, ljcod=ljcod, ivdw_rule=ivdw_rule,
        el14_scale=el14_scale, pairs14=np.array(pairs14, np.int32).reshape(-1, 2),
        excl_pairs=np.array(expairs, np.int32).reshape(-1, 2), solvent_type=solvent_type,
        rexcl_o=rexcl_o, rwat=rwat, xpcent=xpcent, xwcent=xwcent, excl=excl,
        **({} if boxl is None else dict(boxlength=boxl, boxcentre=boxc)),
        # solvent bonds in topology order with their equilibrium lengths: the
        # SHAKE constraints qdyn applies at start-up (shake_solvent defaults on)
        wbond_ij=(bnd[nbonds_solute:, :2] - 1).astype(np.int32),
        wbond_b0=np.array([bondlib[int(c) - 1][2] for c in bnd[nbonds_solute:, 2]]),
        wbond_code=bnd[nbonds_solute:, 2].astype(np.int32),
        # bonded lists (0-based atoms and codes) and libraries as the topology
        # holds them (degrees, torsion paths not inverted)
        ff_type=ff_type, top_bonds=(bnd - 1).astype(np.int32), nbonds_solute=nbonds_solute,
        bondlib=np.array([b[1:3] for b in bondlib], np.float64),
        top_angles=(ang - 1).astype(np.int32), nangles_solute=nangles_solute,
        anglib=np.array(anglib, np.float64),
        top_torsions=(tor - 1).astype(np.int32), ntors_solute=ntors_solute,
        torlib=np.array(torlib, np.float64),
        top_impropers=(imp - 1).astype(np.int32), nimps_solute=nimps_solute,
        implib=np.array(implib, np.float64), imp_type=imp_type)


def read_fep_atoms(path):
    """[FEP] states and [atoms] (Q index -> topology atom); this FEP file has
    no charge/type/soft-core sections, so Q atoms keep their topology charges
    (qcrg = crg, src/simprep.f90:1029) and there is no soft-core."""
    states, atoms, sec = 1, [], None
    with open(path) as f:
        for ln in f:
            s = ln.split("!")[0].strip()
            if not s:
                continue
            if s.startswith("["):
                sec = s.strip("[]").lower()
                continue
            if sec == "fep" and s.split()[0] == "states":
                states = int(s.split()[1])
            elif sec == "atoms":
                q, a = s.split()[:2]
                atoms.append(int(a) - 1)
    return states, np.array(atoms, np.int32)


def read_fep_bonded(path, nstates):
    """Q bonded sections of the FEP file as qatom_load_fep reads them
    (src/qatom.f90:950-1510): [bond_types] id Dmz amz r0 (Morse) or id fk r0
    (harmonic); [angle_types] id fk theta0 [ureyfk ureyr0]; [torsion_types]
    id fk rmult deltor; [improper_types] id fk imp0; [change_*] atoms then one
    type per state (0 = absent).  Comments after '!' are dropped."""
    secs = {}
    sec = None
    with open(path) as f:
        for ln in f:
            t = ln.split("!")[0].strip()
            if not t:
                continue
            if t.startswith("["):
                sec = t.strip("[]").lower()
                secs[sec] = []
                continue
            if sec:
                secs[sec].append(t.split())
    out = {}
    bl = {}
    for v in secs.get("bond_types", []):
        if len(v) >= 4:
            bl[int(v[0])] = (float(v[1]), float(v[2]), float(v[3]), 0.0)   # Dmz amz r0 fk
        else:
            bl[int(v[0])] = (0.0, 0.0, float(v[2]), float(v[1]))
    al = {int(v[0]): (float(v[1]), float(v[2]), float(v[3]) if len(v) > 4 else 0.0,
                      float(v[4]) if len(v) > 4 else 0.0) for v in secs.get("angle_types", [])}
    tl = {int(v[0]): (float(v[1]), float(v[2]), float(v[3])) for v in secs.get("torsion_types", [])}
    il = {int(v[0]): (float(v[1]), float(v[2])) for v in secs.get("improper_types", [])}
    for name, lib, nat in (("bond", bl, 2), ("angle", al, 3), ("torsion", tl, 4), ("improper", il, 4)):
        keys = sorted(lib)
        index = {k: n for n, k in enumerate(keys)}
        out["fep_%slib" % name] = np.array([lib[k] for k in keys], np.float64).reshape(len(keys), -1)
        rows = secs.get("change_%ss" % name, [])
        atoms = np.array([[int(a) - 1 for a in v[:nat]] for v in rows], np.int32).reshape(-1, nat)
        codes = np.array([[index[int(c)] if int(c) > 0 else -1 for c in v[nat:nat + nstates]] for v in rows],
                         np.int32).reshape(-1, nstates)
        out["fep_q%ss" % name] = atoms
        out["fep_q%s_code" % name] = codes
    return out


def read_step0_bands(path):
    """(TOT, KIN, POT) (lower, upper) bounds of the first data row of a
    *_benchmark.en file (columns 26-31 after the step number)."""
    for ln in open(path):
        if ln.startswith("#") or not ln.strip():
            continue
        v = [float(t) for t in ln.split()[1:]]
        return (v[24], v[25]), (v[26], v[27]), (v[28], v[29])
    raise ValueError("no data row in " + path)


def read_switching_atom(path):
    """[PBC] switching_atom of an FEP file (src/qatom.f90:700-716), 0-based."""
    sec = None
    with open(path) as f:
        for ln in f:
            t = ln.split("!")[0].strip()
            if t.startswith("["):
                sec = t.strip("[]").lower()
            elif sec == "pbc" and t.split() and t.split()[0] == "switching_atom":
                return int(t.split()[1]) - 1
    raise ValueError("no [PBC] switching_atom in " + path)


def read_step0_row(path):
    """Lower bounds of the first data row of a *_benchmark.en file in column
    order (QEL QVdW EL VdW QBND QANG QTOR QIMP BND ANG TOR IMP TOT KIN POT)."""
    for ln in open(path):
        if ln.startswith("#") or not ln.strip():
            continue
        v = [float(t) for t in ln.split()[1:]]
        return v[0::2]
    raise ValueError("no data row in " + path)


def build(root, kind):
    bt = os.path.join(root, "tests", "basic_tests")
    d = os.path.join(bt, "prep_" + kind)
    top = read_top(os.path.join(d, "lig_w.top"))
    fep = os.path.join(d, "lig_w.fep")
    nstates, iqseq = read_fep_atoms(fep)
    fepb = read_fep_bonded(fep, nstates)
    en = os.path.join(bt, kind + "_leap-frog_berendsen_benchmark.en")
    tot, kin, pot = read_step0_bands(en)
    row = read_step0_row(en)
    extra = {}
    if kind == "PBC":
        extra["qswitch"] = read_switching_atom(fep)
    name = "lig_w.npz" if kind == "SPH" else "lig_w_pbc.npz"
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), name)
    np.savez_compressed(
        out, **top, **fepb, **extra, nstates=nstates, iqseq=iqseq,
        golden_tot_band=np.array(tot), golden_kin_band=np.array(kin), golden_pot_band=np.array(pot),
        # row 1 of <kind>_leap-frog_berendsen_benchmark.en (zero-width bands):
        # Q-surr. el and vdW (the eval_test.sh line), the solute + solvent +
        # solute-solvent EL and VdW, the solute row's bond, angle, torsion,
        # improper and the Q-atom row's (state 1)
        golden_qsurr_el=row[0], golden_qsurr_vdw=row[1], golden_el=row[2], golden_vdw=row[3],
        golden_qbnd=row[4], golden_qang=row[5], golden_qtor=row[6], golden_qimp=row[7],
        golden_bnd=row[8], golden_ang=row[9], golden_tor=row[10], golden_imp=row[11])
    print("wrote", out, "atoms", top["natom"], "solute", top["nat_solute"],
          "groups", len(top["cgp_first"]), "Q", len(iqseq), "row", row)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_lig_w_fixture.py Q6_ROOT")
    for kind in ("SPH", "PBC"):
        build(sys.argv[1], kind)


if __name__ == "__main__":
    main()
