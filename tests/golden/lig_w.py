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


FIXTURES = {"lig_w": "lig_w.npz", "lig_w_pbc": "lig_w_pbc.npz"}


def load_lig_w(kind: str = "sph") -> tuple[QSystem, dict]:
    """kind "sph": prep_SPH (the 20 A droplet); "pbc": prep_PBC (the same
    solute in a 49.633 A periodic box; golden also holds boxlength, boxcentre
    and the FEP file's switching atom qswitch, 0-based)."""
    name = {"sph": "lig_w", "pbc": "lig_w_pbc"}[kind]
    f = np.load(os.path.join(HERE, FIXTURES[name]))
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
        iuse_switch_atom=int(f["iuse_switch_atom"]), name=name)
    golden = {k: float(f[k]) for k in ("golden_qsurr_el", "golden_qsurr_vdw", "golden_el", "golden_vdw",
                                       "golden_bnd", "golden_ang", "golden_tor", "golden_imp",
                                       "golden_qbnd", "golden_qang", "golden_qtor", "golden_qimp")}
    for k in ("golden_pot_band", "golden_kin_band", "golden_tot_band"):
        golden[k] = tuple(float(v) for v in f[k])
    golden["wbond_ij"] = f["wbond_ij"]
    golden["wbond_b0"] = f["wbond_b0"]
    golden["wbond_code"] = f["wbond_code"]
    if "boxlength" in f.files:
        golden["boxlength"] = f["boxlength"].copy()
        golden["boxcentre"] = f["boxcentre"].copy()
        golden["qswitch"] = int(f["qswitch"])
    return s, golden


def lig_w_bonded(s):
    """The bonded terms qdyn evaluates for lig_w: the topology lists with
    the FEP-redefined terms and the SHAKE-constrained bonds removed
    (defaults shake_solvent on, shake_solute off, shake_hydrogens on,
    shake_heavy off) together with the angles those constraints clear,
    libraries converted as topology() does."""
    from q6_gb300.bonded import remove_shaken
    return remove_shaken(lig_w_topology_terms(s), np.asarray(s.heavy).astype(bool), s.nat_solute)


def lig_w_topology_terms(s):
    """The topology's bonded terms with the FEP-redefined ones removed, before
    SHAKE removes any bond: what init_constraints and wat_shells read."""
    from q6_gb300.bonded import DEG2RAD, BondedTerms, remove_redefined
    f = np.load(os.path.join(HERE, FIXTURES[s.name]))
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
    return remove_redefined(bt)


def lig_w_eq1_inputs(s):
    """What qdyn derives from the regression run's first input (eq1.inp with
    run_test.sh's sphere settings, tests/basic_tests/run_test.sh:172-179):
    stepsize 0.1 fs, temperature 0.1 K, bath_coupling 1 fs, separate scaling,
    non_bond 25, cut-offs 10 / q_atom 99 / lrf 99, LRF on; [solvent] with only
    pol_update 100, so radial_force 60, polarisation on, polarisation_force 20
    and charge_correction (the Born term) on by default (src/md.f90:730-790,
    src/globals.f90:220-229), crgQtot of the ligand and mu_w from the
    topology's last bond and angle codes (src/simprep.f90:4638-4646, 4748-4751).
    Returns (MdSetup, QnbSolventParams, topology terms, evaluated bonded terms)."""
    from q6_gb300.md import MdSetup
    from q6_gb300.system import born_charge, default_solvent_params, water_dipole
    top = lig_w_topology_terms(s)
    cut = dict(Rcq=99.0, RcLRF=99.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)
    setup = MdSetup(stepsize=0.1, temp0=0.1, tau_t=1.0, separate_scaling=True, nbcycle=25, cut=cut)
    sp = default_solvent_params(s, fk_wsphere=60.0, fkwpol=20.0, itdis=100.0,
                                crg_qtot=born_charge(s, [1.0]), mu_w=water_dipole(s, top))
    return setup, sp, top, lig_w_bonded(s)


def lig_w_pbc_step0_coordinates(s, g):
    """qdyn's step-0 coordinates of the box run: the start-up SHAKE of the
    solvent bonds (initial_constraint, src/bondene.f90:1025-1048), then
    put_back_in_box at the first list update (src/md.f90:1666-1671;
    put_solvent_back_in_box on, put_solute_back_in_box off, the box centred on
    the solute's mean position since rigid_box_centre defaults off)."""
    from oracle.box import put_back_in_box
    from oracle.oracle import shake
    mols = {}
    for (i, j), b0 in zip(g["wbond_ij"], g["wbond_b0"]):
        mols.setdefault((int(i) - s.nat_solute) // s.solv_atom, []).append((int(i), int(j), float(b0)))
    x = shake(s.x, [mols[k] for k in sorted(mols)], 1.0 / s.mass[s.iac])
    molecules = [np.arange(s.nat_solute)] + [s.nat_solute + s.solv_atom * w + np.arange(s.solv_atom)
                                             for w in range(s.nwat)]
    x, _ = put_back_in_box(x, g["boxlength"], molecules, s.mass[s.iac], 1, s.nat_solute,
                           put_solute=False, put_solvent=True)
    return x


# the box run's cut-offs (run_test.sh:173-176: q_atom 24, lrf 24; solute and
# solvent cut-offs at their defaults of 10 A)
PBC_CUT = dict(Rcq=24.0, RcLRF=24.0, Rcpp=10.0, Rcpw=10.0, Rcww=10.0)


def lig_w_pbc_eq1_inputs(s):
    """eq1.inp with run_test.sh's box settings (tests/basic_tests/run_test.sh:
    172-176): [PBC] put_solvent_back_in_box on, put_solute_back_in_box off;
    q_atom 24, lrf 24; otherwise as the sphere run (stepsize 0.1 fs,
    temperature 0.1 K, bath_coupling 1 fs, separate scaling, non_bond 25); no
    solvent restraints in a box.  Returns (MdSetup, topology terms, evaluated
    bonded terms)."""
    from q6_gb300.md import MdSetup
    top = lig_w_topology_terms(s)
    setup = MdSetup(stepsize=0.1, temp0=0.1, tau_t=1.0, separate_scaling=True, nbcycle=25, cut=PBC_CUT)
    return setup, top, lig_w_bonded(s)
