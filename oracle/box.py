"""Oracle (test infrastructure only): the periodic-box pair lists and
energies of qdyn (use_PBC), restated in numpy.  The product computes these on
the GPU (k_build_box_*, k_box_*); nothing in the package imports this file.

Q6 sources restated (paths within the Q6 tree):
  lattice shift   boxlength * q_nint(shift * inv_boxl), src/math.f90:566-574
                  (Fortran nint: halves away from zero)
  lists           nbpplist_box, src/nonbondene.f90:1643-1775; nbpwlist_box,
                  2730-2841; nbwwlist_box, 4174-4273; nbqplist_box, 3747-3860;
                  nbqwlist_box, 3949-4026
  energies        nonbond_pp_box 4763-4853, nonbond_pw_box 4920-5009,
                  nonbond_ww_spc_box / nonbond_ww_box 5979-6077 / 5576-5654,
                  nonbond_qp_box 5234-5335, nonbond_qw_spc_box / nonbond_qw_box
                  5771-5881 / 5422-5505; pair kernels nbe_b, nbe_spcb, nbe_qx,
                  nbe_qspc (src/nonbonded.f90)
Every pair takes its partner at x_j + shift, shift from the two units'
reference atoms (switch atoms, first solvent atoms, qswitch).  nonbond_qp_box
as written takes the group shift with the opposite sign (x_a - x_qswitch
against x_i - x_j) and reads a group index nbqplist_box never sets; the
restatement uses the minimum image of the group's first atom inside Rcq, the
shift nonbond_qw_spc_box uses for waters.  With any-atom group tests
(nbpplis2_box, nbpwlis2_box) the reference shifts a group pair by its first
atom pair inside the cut-off; the restatement keeps the switch atoms (the
same shift unless a group spans half a box).
"""
from __future__ import annotations

import numpy as np

from oracle.pairsets import PairValues, _combine


def nint(v):
    return np.sign(v) * np.floor(np.abs(v) + 0.5)


def shift_of(L, xa, xb):
    return L * nint((xa - xb) / L)


def d2_min_image(L, xa, xb):
    d = xa - xb
    t = L * nint(d / L) - d
    return (t * t).sum(-1)


def _groups(s):
    return [np.asarray(s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1], np.int64) for g in range(s.ncgp_solute)]


def box_lists(s, x, L, qswitch, cut):
    """The box lists: pp atom pairs (i, j), pw (solute atom, water), ww (iw, jw),
    qp solute atoms, qw waters."""
    L = np.asarray(L, np.float64)
    pv = PairValues(s)
    groups = _groups(s)
    sw = np.asarray(s.cgp_iswitch[:s.ncgp_solute], np.int64)
    nonq = np.asarray(pv.iqatom) < 0
    ns, sa, W = s.nat_solute, s.solv_atom, s.nwat
    first = ns + sa * np.arange(W)
    pp = []
    G = len(groups)
    any_atom = int(s.iuse_switch_atom) == 0   # nbpplis2_box / nbpwlis2_box: any atom pair
    for g1 in range(G):
        for g2 in range(g1, G):
            if g1 != g2:
                if any_atom:
                    d2 = d2_min_image(L, x[groups[g1]][:, None, :], x[groups[g2]][None, :, :])
                    if (d2 > cut["Rcpp"] ** 2).all():
                        continue
                elif d2_min_image(L, x[sw[g1]], x[sw[g2]]) > cut["Rcpp"] ** 2:
                    continue
            for i in groups[g1]:
                if not nonq[i]:
                    continue
                for j in groups[g2]:
                    if not nonq[j] or (g1 == g2 and i >= j):
                        continue
                    ok, _ = pv.pp(int(i), int(j))
                    if ok:
                        pp.append((int(i), int(j)))
    pw = []
    if W:
        for g in range(G):
            if any_atom:
                d2 = d2_min_image(L, x[groups[g]][:, None, :], x[first][None, :, :])
                inside = np.nonzero((d2 <= cut["Rcpw"] ** 2).any(0))[0]
            else:
                inside = np.nonzero(d2_min_image(L, x[sw[g]][None, :], x[first]) <= cut["Rcpw"] ** 2)[0]
            for i in groups[g]:
                if nonq[i]:
                    pw.extend((int(i), int(w)) for w in inside)
    ww = []
    if W:
        d2 = d2_min_image(L, x[first][:, None, :], x[first][None, :, :])
        iw, jw = np.nonzero(np.triu(d2 <= cut["Rcww"] ** 2, 1))
        ww = list(zip(iw.tolist(), jw.tolist()))
    qp, qw = [], []
    if s.nqat:
        rq2 = cut["Rcq"] ** 2
        for g in range(G):
            if (d2_min_image(L, x[groups[g]], x[qswitch][None, :]) <= rq2).any():
                qp.extend(int(i) for i in groups[g] if not pv.qnear[i])
        if W:
            qw = np.nonzero(d2_min_image(L, x[first], x[qswitch][None, :]) <= rq2)[0].tolist()
    return dict(pp=pp, pw=pw, ww=ww, qp=qp, qw=qw)


def _qw_values(s, iq, a, st):
    """precompute_set_values_qw (src/simprep.f90:3517-3558)."""
    ns = s.nat_solute
    tw = int(s.iac[ns + a])
    i = int(s.iqseq[iq])
    vdw = int(s.ljcod[tw, s.iac[i]])
    qvdw = 1 if vdw == 2 else vdw
    if s.qvdw_flag:
        qt = int(s.qiac[iq, st])
        qa, qb = s.qavdw[qt, qvdw - 1], s.qbvdw[qt, qvdw - 1]
    else:
        qa, qb = s.avdw[s.iac[i], vdw - 1], s.bvdw[s.iac[i], vdw - 1]
    A, B = _combine(s.ivdw_rule, qa, s.avdw[tw, vdw - 1], qb, s.bvdw[tw, vdw - 1])
    el = s.crg[i] * s.crg[ns + a] if s.qq_use_library_charges else s.qcrg[iq, st] * s.crg[ns + a]
    return float(A), float(B), float(el), float(s.sc_lookup[iq, tw, st])


def _lj_pair(s, ti, tj, code):
    return _combine(s.ivdw_rule, s.avdw[ti, code - 1], s.avdw[tj, code - 1], s.bvdw[ti, code - 1],
                    s.bvdw[tj, code - 1])


def box_energies(s, x, lam, L, qswitch, cut, lists=None):
    """(d, E, EQ) of the box routines: gradient [natom][3], classical
    energies {pp,pw,ww}_{el,vdw}, EQ [nstates][6] with the Q-P and Q-W
    columns (the static Q-Q energies are nonbond_qq's, unchanged by a box)."""
    x = np.asarray(x, np.float64)
    L = np.asarray(L, np.float64)
    lam = np.asarray(lam, np.float64)
    lists = lists or box_lists(s, x, L, qswitch, cut)
    pv = PairValues(s)
    ns, sa = s.nat_solute, s.solv_atom
    S, nq = s.nstates, s.nqat
    d = np.zeros_like(x)
    E = dict(pp_el=0.0, pp_vdw=0.0, pw_el=0.0, pw_vdw=0.0, ww_el=0.0, ww_vdw=0.0)
    EQ = np.zeros((S, 6))
    iwhich = np.zeros(s.natom, np.int64)
    for g, atoms in enumerate(_groups(s)):
        iwhich[atoms] = g
    sw = np.asarray(s.cgp_iswitch, np.int64)
    spc = s.ivdw_rule == 1 and s.solvent_type == 0

    def pair(i, j, sh, A, B, el, lj=True):
        vec = sh - (x[i] - x[j])
        r2 = 1.0 / float(vec @ vec)
        r = np.sqrt(r2)
        vel = el * r
        if lj:
            r6 = r2 * r2 * r2
            va, vb = A * r6 * r6, B * r6
            dv = r2 * (-vel - 12.0 * va + 6.0 * vb)
            vdw = va - vb
        else:
            dv, vdw = r2 * (-vel), 0.0
        d[i] -= vec * dv
        d[j] += vec * dv
        return vel, vdw

    for i, j in lists["pp"]:
        _, (A, B, el, _, _) = pv.pp(i, j)
        sh = shift_of(L, x[sw[iwhich[i]]], x[sw[iwhich[j]]])
        v = pair(i, j, sh, A, B, el)
        E["pp_el"] += v[0]
        E["pp_vdw"] += v[1]
    wt = [int(s.iac[ns + a]) for a in range(sa)]
    for i, w in lists["pw"]:
        j0 = ns + sa * w
        sh = shift_of(L, x[sw[iwhich[i]]], x[j0])
        for a in range(sa):
            code = int(s.ljcod[s.iac[i], wt[a]])
            A, B = _lj_pair(s, int(s.iac[i]), wt[a], code)
            v = pair(i, j0 + a, sh, A, B, s.crg[i] * s.crg[j0 + a])
            E["pw_el"] += v[0]
            E["pw_vdw"] += v[1]
    for iw, jw in lists["ww"]:
        i0, j0 = ns + sa * iw, ns + sa * jw
        sh = shift_of(L, x[i0], x[j0])
        for la in range(sa):
            for ka in range(sa):
                lj = (not spc) or (la == 0 and ka == 0)
                code = int(s.ljcod[wt[la], wt[ka]])
                A, B = _lj_pair(s, wt[la], wt[ka], code)
                v = pair(i0 + la, j0 + ka, sh, A, B, s.crg[i0 + la] * s.crg[j0 + ka], lj)
                E["ww_el"] += v[0]
                E["ww_vdw"] += v[1]

    def qpair(i, j, sh, pars, lj):
        vec = sh - (x[i] - x[j])
        r2 = 1.0 / float(vec @ vec)
        r = np.sqrt(r2)
        r6hc = 1.0 / (r2 * r2 * r2)
        dvs = 0.0
        out = []
        for st, (A, B, el, sc) in enumerate(pars):
            vel = el * r
            if lj:
                r6 = 1.0 / (r6hc + sc)
                va, vb = A * r6 * r6, B * r6
                dvs += r2 * (-vel - (12.0 * va - 6.0 * vb) * r6 * r6hc) * lam[st]
                out.append((vel, va - vb))
            else:
                dvs += -r2 * vel * lam[st]
                out.append((vel, 0.0))
        d[i] -= vec * dvs
        d[j] += vec * dvs
        return out

    rq2 = cut["Rcq"] ** 2
    groups = _groups(s)
    for j in lists["qp"]:
        g = iwhich[j]
        ref = next((int(a) for a in groups[g] if d2_min_image(L, x[a], x[qswitch]) <= rq2), int(groups[g][0]))
        sh = shift_of(L, x[qswitch], x[ref])
        for iq in range(nq):
            pars = [pv.q_with_p(iq, j, st)[1][:4] for st in range(S)]
            for st, (vel, vdw) in enumerate(qpair(int(s.iqseq[iq]), j, sh, pars, True)):
                EQ[st, 2] += vel
                EQ[st, 3] += vdw
    for w in lists["qw"]:
        j0 = ns + sa * w
        sh = shift_of(L, x[qswitch], x[j0])
        for iq in range(nq):
            for a in range(sa):
                pars = [_qw_values(s, iq, a, st) for st in range(S)]
                lj = (not spc) or a == 0
                for st, (vel, vdw) in enumerate(qpair(int(s.iqseq[iq]), j0 + a, sh, pars, lj)):
                    EQ[st, 4] += vel
                    EQ[st, 5] += vdw
    return d, E, EQ


def put_back_in_box(x, L, molecules, mass, nmol_solute, nat_solute, put_solute=True, put_solvent=True,
                    boxcentre=None):
    """put_back_in_box (src/simprep.f90:4177-4352): returns (x, centre)."""
    x = np.array(x, dtype=np.float64)
    L = np.asarray(L, np.float64)
    if boxcentre is None:
        n = nat_solute if nat_solute > 0 else len(x)
        c = x[:n].mean(0)
    else:
        c = np.asarray(boxcentre, np.float64)
    lo, hi = c - L / 2.0, c + L / 2.0
    first = 0 if put_solute else nmol_solute
    last = len(molecules) if put_solvent else nmol_solute
    for mol in molecules[first:last]:
        mol = np.asarray(mol)
        cm = (x[mol] * mass[mol][:, None]).sum(0) * (1.0 / mass[mol].sum())
        for k in range(3):
            if cm[k] > hi[k]:
                x[mol, k] -= L[k]
            elif cm[k] < lo[k]:
                x[mol, k] += L[k]
    return x, c
