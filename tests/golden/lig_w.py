"""Load the lig_w golden fixture (Q6 tests/basic_tests/prep_SPH) as a QSystem.

The FEP file of that test makes every solute atom a Q atom in one state with
the topology charges and atom types (no [change_charges], no [atom_types], no
[softcore]), so qcrg = crg (Q6 src/simprep.f90:1029), qvdw_flag is off and all
soft-core alphas are zero.  qconn follows make_qconn over the solute bonds
(Q6 src/nonbondene.f90:3087-3187).
"""
from __future__ import annotations

import math
import os

import numpy as np

from q6_gb300.system import QSystem

HERE = os.path.dirname(os.path.abspath(__file__))


def load_lig_w() -> tuple[QSystem, dict]:
    f = np.load(os.path.join(HERE, "lig_w.npz"))
    natom, nsol = int(f["natom"]), int(f["nat_solute"])
    sa = int(f["solv_atom"])
    scale = math.sqrt(float(f["coulomb"]))
    crg = f["crg"] * scale
    iqseq = f["iqseq"].astype(np.int32)
    nq, S = len(iqseq), int(f["nstates"])
    natyps = f["avdw"].shape[0]
    # qconn: 1 for the Q atom itself, 1 + bond distance up to 4, else 9
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
    s = QSystem(
        natom=natom, nat_solute=nsol, nwat=(natom - nsol) // sa, solv_atom=sa,
        solvent_type=int(f["solvent_type"]), x=f["x"].copy(), crg=crg,
        iac=f["iac"].astype(np.int32), excl=f["excl"].astype(np.uint8), heavy=heavy,
        avdw=f["avdw"], bvdw=f["bvdw"], ljcod=f["ljcod"], ivdw_rule=int(f["ivdw_rule"]),
        el14_scale=float(f["el14_scale"]), cgp_first=f["cgp_first"], cgp_last=f["cgp_last"],
        cgp_iswitch=f["cgp_iswitch"], cgpatom=f["cgpatom"], ncgp_solute=int(f["ncgp_solute"]),
        excl_pairs=f["excl_pairs"], pairs14=f["pairs14"], bonds=f["bonds"].astype(np.int32),
        nqat=nq, nstates=S, iqseq=iqseq, qcrg=np.repeat(crg[iqseq][:, None], S, 1),
        qiac=np.zeros((nq, S), np.int32), qavdw=np.zeros((1, 3)), qbvdw=np.zeros((1, 3)),
        qvdw_flag=0, qq_use_library_charges=0, sc_lookup=np.zeros((nq, natyps + nq, S)),
        qconn=qconn, el_scale_pairs=np.zeros((0, 2), np.int32), el_scale=np.zeros((0, S)),
        qexpnb_pairs=np.zeros((0, 2), np.int32), xpcent=f["xpcent"], xwcent=f["xwcent"],
        rexcl_o=float(f["rexcl_o"]), rwat=float(f["rwat"]), mass=mass,
        iuse_switch_atom=int(f["iuse_switch_atom"]), name="lig_w")
    golden = {k: float(f[k]) for k in ("golden_qsurr_el", "golden_qsurr_vdw", "golden_el", "golden_vdw",
                                       "golden_bnd", "golden_ang", "golden_tor", "golden_imp",
                                       "golden_qbnd", "golden_qang", "golden_qtor", "golden_qimp")}
    golden["wbond_ij"] = f["wbond_ij"]
    golden["wbond_b0"] = f["wbond_b0"]
    golden["wbond_code"] = f["wbond_code"]
    return s, golden


def lig_w_bonded(s):
    """The bonded terms qdyn evaluates for lig_w: the topology lists with
    the FEP-redefined terms and the SHAKE-constrained bonds removed
    (defaults shake_solvent on, shake_solute off, shake_hydrogens on,
    shake_heavy off), libraries converted as topology() does."""
    from q6_gb300.bonded import DEG2RAD, BondedTerms, remove_redefined, remove_shaken
    f = np.load(os.path.join(HERE, "lig_w.npz"))
    anglib = f["anglib"].copy()
    anglib[:, 1] *= DEG2RAD
    torlib = f["torlib"].copy()
    torlib[:, 2] *= DEG2RAD
    torlib[:, 3] = 1.0 / torlib[:, 3]
    implib = f["implib"].copy()
    implib[:, 1] *= DEG2RAD
    qanglib = f["fep_anglelib"].copy()
    qanglib[:, 1] *= DEG2RAD
    qtorlib = f["fep_torsionlib"].copy()
    qtorlib[:, 2] *= DEG2RAD
    qimplib = f["fep_improperlib"].copy()
    qimplib[:, 1] *= DEG2RAD
    bt = BondedTerms(
        bonds=f["top_bonds"], nbonds_solute=int(f["nbonds_solute"]), bondlib=f["bondlib"],
        angles=f["top_angles"], nangles_solute=int(f["nangles_solute"]), anglib=anglib,
        torsions=f["top_torsions"], ntors_solute=int(f["ntors_solute"]), torlib=torlib,
        impropers=f["top_impropers"], nimps_solute=int(f["nimps_solute"]), implib=implib,
        imp_type=int(f["imp_type"]), urey_bradley=int(int(f["ff_type"]) == 3),
        qbonds=f["fep_qbonds"], qbond_code=f["fep_qbond_code"], qbondlib=f["fep_bondlib"],
        qangles=f["fep_qangles"], qangle_code=f["fep_qangle_code"], qanglib=qanglib,
        qtorsions=f["fep_qtorsions"], qtorsion_code=f["fep_qtorsion_code"], qtorlib=qtorlib,
        qimpropers=f["fep_qimpropers"], qimproper_code=f["fep_qimproper_code"], qimplib=qimplib)
    bt = remove_redefined(bt)
    return remove_shaken(bt, np.asarray(s.heavy).astype(bool), s.nat_solute)
