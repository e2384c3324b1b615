"""Build tests/golden/cjp.npz from the reference's realistic FEP test inputs.

Reads tests/exclude_tests/inputs/2cjpFH_ionres_oplsa.top and lig.fep of the
Q6 tree (its root directory is the command-line argument): a protein with a
ligand in a 20 A sphere (5,622 atoms, 1,167 charge groups, 1,875 excluded
atoms), 40 Q atoms in 2 states.  The topology reader is the lig_w fixture's
(Q6 src/topo.f90:471-1115).  From the FEP file (the sections qatom_load_fep
reads, src/qatom.f90:690-1100): [FEP] states, [atoms] (Q index -> topology
atom), [change_charges] (charge per state), [atom_types] (name, then
(A, B) for the three LJ codes - normal, polar (the soft-pair exponential's
C and a), 1-4 - and the mass), [change_atoms] (type name per state) and
[soft_pairs] (Q index pairs with the exponential repulsion).  The reference
has no golden numbers for this system: the fixture gives the GPU-versus-
oracle parity tests a real topology.

Usage: python tests/golden/make_2cjp_fixture.py Q6_ROOT
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_lig_w_fixture import read_top  # noqa: E402


def read_fep(path):
    sec, out = None, {"states": 1, "atoms": [], "charges": {}, "types": [], "change_atoms": {}, "soft": []}
    with open(path) as f:
        for ln in f:
            t = ln.split("!")[0].strip()
            if not t:
                continue
            if t.startswith("["):
                sec = t.strip("[]").lower()
                continue
            w = t.split()
            if sec == "fep" and w[0] == "states":
                out["states"] = int(w[1])
            elif sec == "atoms":
                out["atoms"].append(int(w[1]) - 1)
            elif sec == "change_charges":
                out["charges"][int(w[0]) - 1] = [float(v) for v in w[1:1 + out["states"]]]
            elif sec == "atom_types":
                out["types"].append((w[0], [float(v) for v in w[1:7]], float(w[7])))
            elif sec == "change_atoms":
                out["change_atoms"][int(w[0]) - 1] = w[1:1 + out["states"]]
            elif sec == "soft_pairs":
                out["soft"].append((int(w[0]) - 1, int(w[1]) - 1))
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_2cjp_fixture.py Q6_ROOT")
    d = os.path.join(sys.argv[1], "tests", "exclude_tests", "inputs")
    top = read_top(os.path.join(d, "2cjpFH_ionres_oplsa.top"))
    fep = read_fep(os.path.join(d, "lig.fep"))
    S, nq = fep["states"], len(fep["atoms"])
    names = [n for n, _, _ in fep["types"]]
    qavdw = np.array([[v[0], v[2], v[4]] for _, v, _ in fep["types"]])   # A: normal, polar (C), 1-4
    qbvdw = np.array([[v[1], v[3], v[5]] for _, v, _ in fep["types"]])   # B: normal, polar (a), 1-4
    qcrg = np.array([fep["charges"][iq] for iq in range(nq)])
    qiac = np.array([[names.index(fep["change_atoms"][iq][s]) for s in range(S)] for iq in range(nq)], np.int32)
    out = os.path.join(HERE, "cjp.npz")
    keep = {k: v for k, v in top.items() if not k.startswith("top_") and k not in (
        "bondlib", "anglib", "torlib", "implib", "wbond_ij", "wbond_b0", "wbond_code")}
    np.savez_compressed(out, **keep, nstates=S, iqseq=np.array(fep["atoms"], np.int32), qcrg=qcrg,
                        qiac=qiac, qavdw=qavdw, qbvdw=qbvdw, qexpnb_pairs=np.array(fep["soft"], np.int32))
    print("wrote", out, "atoms", top["natom"], "solute", top["nat_solute"], "groups", len(top["cgp_first"]),
          "Q", nq, "states", S, "Q types", len(names), "soft pairs", len(fep["soft"]))


if __name__ == "__main__":
    main()
