"""Build tests/golden/lig_w.npz from Q6's own regression-test inputs.

Reads tests/basic_tests/prep_SPH/lig_w.top and lig_w.fep of the Q6 tree (path
given on the command line, default /root/reference) with a reader written for
the Q topology text format as Q6 src/topo.f90:471-1115 parses it, and stores
the arrays the nonbonded path needs.  The fixture is what the golden test uses;
the Q6 tree is not needed at test time.

The step-0 energies that the Q6 regression test checks for this system
(tests/basic_tests/eval_test.sh:99 and row 1 of
SPH_leap-frog_berendsen_benchmark.en) are stored beside the arrays:
Q-surr. el 3.12, vdW 139.43 (Q-atom state 1, lambda 1) and the sums of the
solute, solvent and solute-solvent rows, EL -7.30, VdW -413.17.

Usage: python tests/golden/make_lig_w_fixture.py [Q6_ROOT]
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
    while not r.line().strip().upper().startswith("END"):
        pass
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
    nangcod = r.head_ints(1)[0]
    anglib = [r.head_floats(3) for _ in range(nangcod)]
    nt = r.head_ints(2)
    ntors = nt[0]
    r.values(5 * ntors, int)
    ntorcod = r.head_ints(1)[0]
    for _ in range(ntorcod):
        r.line()
    ni = r.head_ints(2)
    nimps = ni[0]
    r.values(5 * nimps, int)
    nimpcod = r.head_ints(2)[0]
    for _ in range(nimpcod):
        r.line()
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
        # solvent bonds in topology order with their equilibrium lengths: the
        # SHAKE constraints qdyn applies at start-up (shake_solvent defaults on)
        wbond_ij=(bnd[nbonds_solute:, :2] - 1).astype(np.int32),
        wbond_b0=np.array([bondlib[int(c) - 1][2] for c in bnd[nbonds_solute:, 2]]),
        wbond_code=bnd[nbonds_solute:, 2].astype(np.int32))


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


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    d = os.path.join(root, "tests", "basic_tests", "prep_SPH")
    top = read_top(os.path.join(d, "lig_w.top"))
    nstates, iqseq = read_fep_atoms(os.path.join(d, "lig_w.fep"))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lig_w.npz")
    np.savez_compressed(
        out, **top, nstates=nstates, iqseq=iqseq,
        golden_qsurr_el=3.12, golden_qsurr_vdw=139.43,
        golden_el=-7.30, golden_vdw=-413.17)
    print("wrote", out, "atoms", top["natom"], "solute", top["nat_solute"],
          "groups", len(top["cgp_first"]), "Q", len(iqseq))


if __name__ == "__main__":
    main()
