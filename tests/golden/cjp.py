"""Load the 2cjp fixture (Q6 tests/exclude_tests/inputs: a protein and its
ligand in a 20 A sphere, 40 Q atoms in 2 states) as a QSystem.

Q charges per state from [change_charges] (scaled by sqrt(Coulomb) as the
topology charges are), Q LJ from the FEP file's [atom_types] / [change_atoms]
(qvdw_flag on), the two [soft_pairs], no [softcore] (zero alphas).  qconn
follows make_qconn over the solute bonds (Q6 src/nonbondene.f90:3087-3187).
"""
from __future__ import annotations

import math
import os

import numpy as np

from q6_gb300.system import QSystem

HERE = os.path.dirname(os.path.abspath(__file__))


def load_cjp() -> QSystem:
    f = np.load(os.path.join(HERE, "cjp.npz"))
    natom, nsol = int(f["natom"]), int(f["nat_solute"])
    sa = int(f["solv_atom"])
    scale = math.sqrt(float(f["coulomb"]))
    crg = f["crg"] * scale
    iqseq = f["iqseq"].astype(np.int32)
    nq, S = len(iqseq), int(f["nstates"])
    natyps = f["avdw"].shape[0]
    adj = [[] for _ in range(nsol)]
    for a, b in f["bonds"]:
        adj[int(a)].append(int(b))
        adj[int(b)].append(int(a))
    qconn = np.full((S, nsol, nq), 9, np.int8)
    for iq, src in enumerate(iqseq):
        dist = {int(src): 1}
        frontier = [int(src)]
        for lev in (2, 3, 4):
            nxt = []
            for u in frontier:
                for w in adj[u]:
                    if w not in dist:
                        dist[w] = lev
                        nxt.append(w)
            frontier = nxt
        for a, lev in dist.items():
            qconn[:, a, iq] = lev
    mass = f["mass"]
    heavy = (mass[f["iac"]] >= 4.0).astype(np.uint8)
    return QSystem(
        natom=natom, nat_solute=nsol, nwat=(natom - nsol) // sa, solv_atom=sa,
        solvent_type=int(f["solvent_type"]), x=f["x"].copy(), crg=crg,
        iac=f["iac"].astype(np.int32), excl=f["excl"].astype(np.uint8), heavy=heavy,
        avdw=f["avdw"], bvdw=f["bvdw"], ljcod=f["ljcod"], ivdw_rule=int(f["ivdw_rule"]),
        el14_scale=float(f["el14_scale"]), cgp_first=f["cgp_first"], cgp_last=f["cgp_last"],
        cgp_iswitch=f["cgp_iswitch"], cgpatom=f["cgpatom"], ncgp_solute=int(f["ncgp_solute"]),
        excl_pairs=f["excl_pairs"], pairs14=f["pairs14"], bonds=f["bonds"].astype(np.int32),
        nqat=nq, nstates=S, iqseq=iqseq, qcrg=f["qcrg"] * scale, qiac=f["qiac"].astype(np.int32),
        qavdw=f["qavdw"], qbvdw=f["qbvdw"], qvdw_flag=1, qq_use_library_charges=0,
        sc_lookup=np.zeros((nq, natyps + nq, S)), qconn=qconn,
        el_scale_pairs=np.zeros((0, 2), np.int32), el_scale=np.zeros((0, S)),
        qexpnb_pairs=f["qexpnb_pairs"].astype(np.int32), xpcent=f["xpcent"], xwcent=f["xwcent"],
        rexcl_o=float(f["rexcl_o"]), rwat=float(f["rwat"]), mass=mass,
        iuse_switch_atom=int(f["iuse_switch_atom"]), name="2cjp")
