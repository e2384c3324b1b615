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


def _pairs_within_box(L, p, rc):
    """(i, j), i < j, with minimum-image d2 <= rc^2 in FP64: a periodic k-d
    tree proposes the pairs within rc + 0.01 A of the wrapped positions, the
    d2 above decides (scipy; the all-pairs matrix when it is absent)."""
    try:
        from scipy.spatial import cKDTree
    except ImportError:
        cKDTree = None
    if cKDTree is None or len(p) < 2:
        d2 = d2_min_image(L, p[:, None, :], p[None, :, :])
        return np.nonzero(np.triu(d2 <= rc * rc, 1))
    w = np.mod(p, L)
    w = np.where(w >= L, 0.0, w)   # mod may round up to L itself
    cand = cKDTree(w, boxsize=L).query_pairs(rc + 0.01, output_type="ndarray")
    if len(cand) == 0:
        return np.zeros(0, np.int64), np.zeros(0, np.int64)
    i, j = np.minimum(cand[:, 0], cand[:, 1]), np.maximum(cand[:, 0], cand[:, 1])
    keep = d2_min_image(L, p[i], p[j]) <= rc * rc
    o = np.lexsort((j[keep], i[keep]))
    return i[keep][o], j[keep][o]


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
        iw, jw = _pairs_within_box(L, x[first], cut["Rcww"])
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

    def pairs(i, j, sh, A, B, el, lj=True):
        """pair() over arrays of pairs; returns the summed (el, vdw)."""
        vec = sh - (x[i] - x[j])
        r2 = 1.0 / (vec * vec).sum(1)
        r = np.sqrt(r2)
        vel = el * r
        if lj:
            r6 = r2 * r2 * r2
            va, vb = A * r6 * r6, B * r6
            dv = r2 * (-vel - 12.0 * va + 6.0 * vb)
            vdw = float((va - vb).sum())
        else:
            dv, vdw = r2 * (-vel), 0.0
        np.add.at(d, i, -vec * dv[:, None])
        np.add.at(d, j, vec * dv[:, None])
        return float(vel.sum()), vdw

    if len(lists["pw"]):
        P = np.asarray(lists["pw"], np.int64).reshape(-1, 2)
        i, j0 = P[:, 0], ns + sa * P[:, 1]
        sh = shift_of(L, x[sw[iwhich[i]]], x[j0])
        ti = np.asarray(s.iac, np.int64)[i]
        for a in range(sa):
            code = np.asarray(s.ljcod, np.int64)[ti, wt[a]]
            A = np.zeros(len(i))
            B = np.zeros(len(i))
            for t in np.unique(ti):
                for c in np.unique(code[ti == t]):
                    m = (ti == t) & (code == c)
                    A[m], B[m] = _lj_pair(s, int(t), wt[a], int(c))
            v = pairs(i, j0 + a, sh, A, B, s.crg[i] * s.crg[j0 + a])
            E["pw_el"] += v[0]
            E["pw_vdw"] += v[1]
    if len(lists["ww"]):
        P = np.asarray(lists["ww"], np.int64).reshape(-1, 2)
        i0, j0 = ns + sa * P[:, 0], ns + sa * P[:, 1]
        sh = shift_of(L, x[i0], x[j0])
        for la in range(sa):
            for ka in range(sa):
                lj = (not spc) or (la == 0 and ka == 0)
                code = int(s.ljcod[wt[la], wt[ka]])
                A, B = _lj_pair(s, wt[la], wt[ka], code)
                v = pairs(i0 + la, j0 + ka, sh, A, B, s.crg[i0 + la] * s.crg[j0 + ka], lj)
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
    if len(lists["qw"]):
        j0 = ns + sa * np.asarray(lists["qw"], np.int64)
        sh = shift_of(L, x[qswitch], x[j0])
        for iq in range(nq):
            i = int(s.iqseq[iq])
            for a in range(sa):
                lj = (not spc) or a == 0
                vec = sh - (x[i] - x[j0 + a])
                r2 = 1.0 / (vec * vec).sum(1)
                r = np.sqrt(r2)
                r6hc = 1.0 / (r2 * r2 * r2)
                dvs = np.zeros(len(j0))
                for st in range(S):
                    A, B, el, sc = _qw_values(s, iq, a, st)
                    vel = el * r
                    if lj:
                        r6 = 1.0 / (r6hc + sc)
                        va, vb = A * r6 * r6, B * r6
                        dvs += r2 * (-vel - (12.0 * va - 6.0 * vb) * r6 * r6hc) * lam[st]
                        EQ[st, 5] += float((va - vb).sum())
                    else:
                        dvs += -r2 * vel * lam[st]
                    EQ[st, 4] += float(vel.sum())
                d[i] -= (vec * dvs[:, None]).sum(0)
                np.add.at(d, j0 + a, vec * dvs[:, None])
    return d, E, EQ


def _all_groups(s):
    return [np.asarray(s.cgpatom[s.cgp_first[g]:s.cgp_last[g] + 1], np.int64) for g in range(s.ncgp)]


def _unit_min_d2(L, x, tests):
    """[G][G] minimum-image d2 minimised over the atom pairs of two units'
    test atoms (tests[g]: the atoms unit g is tested by)."""
    T = np.concatenate(tests)
    starts = np.cumsum([0] + [len(t) for t in tests[:-1]])
    D = d2_min_image(L, x[T][:, None, :], x[T][None, :, :])
    D = np.minimum.reduceat(D, starts, axis=0)
    return np.minimum.reduceat(D, starts, axis=1)


def box_lrf(s, x, L, cut, batch=64):
    """LRF records of the box lists (cgp_centers, then the LRF branch of
    nbpplist_box_lrf 1910-2055, nbpwlist_box_lrf 2957-3085, nbwwlist_box_lrf
    4397-4515 with lrf_update 628-725): every unit pair (solute group, water)
    whose minimum-image switch-atom distance r2 satisfies Rc^2 < r2 <=
    RcLRF^2 (Rc of the pair's kind) adds the non-Q atoms of each unit to the
    other's Taylor moments about its group centre, the source shifted by
    boxlength * nint((x_switch(source) - centre(target)) / boxlength).
    With the topology's switch-atom flag off (nbpplis2_box_lrf 1220-1367,
    nbpwlis2_box_lrf 2359-2491) a pair with a solute group is LRF when no
    atom pair of the two units (a water by its first atom) lies within Rc
    and some atom pair within RcLRF; water pairs keep the first-atom test,
    and lrf_update still shifts by the source's switch atom.
    Excluded atoms take part (the box lists do not test excl).  Returns
    [ncgp][43]: centre(3), phi0, phi1(3), phi2(3x3 row-major), phi3(9x3)."""
    x = np.asarray(x, np.float64)
    L = np.asarray(L, np.float64)
    groups = _all_groups(s)
    G, Gs, ns, sa = s.ncgp, s.ncgp_solute, s.nat_solute, s.solv_atom
    cent = np.array([x[a].mean(0) for a in groups])
    sw = np.array([int(s.cgp_iswitch[g]) if g < Gs else int(groups[g][0]) for g in range(G)], np.int64)
    if int(s.iuse_switch_atom) == 0:   # any-atom unit tests
        dmin = _unit_min_d2(L, x, [groups[g] if g < Gs else np.array([ns + sa * (g - Gs)]) for g in range(G)])
    else:
        dmin = None
    isq = np.zeros(s.natom, bool)
    isq[np.asarray(s.iqseq, np.int64)] = True
    gof = np.zeros(s.natom, np.int64)
    for g, a in enumerate(groups):
        gof[a] = g
    src = np.nonzero(~isq)[0]                 # LRF source atoms
    sgrp = gof[src]
    q = np.asarray(s.crg, np.float64)[src]
    solute = np.arange(G) < Gs
    rl2 = cut["RcLRF"] ** 2
    out = np.zeros((G, 43))
    out[:, :3] = cent
    for b0 in range(0, G, batch):
        tg = np.arange(b0, min(G, b0 + batch))
        if dmin is None:
            d2 = d2_min_image(L, x[sw][None, :, :], x[sw[tg]][:, None, :])      # [target][source group]
        else:
            d2 = dmin[tg]
        both = solute[tg][:, None] & solute[None, :]
        none = ~solute[tg][:, None] & ~solute[None, :]
        rc2 = np.where(both, cut["Rcpp"] ** 2, np.where(none, cut["Rcww"] ** 2, cut["Rcpw"] ** 2))
        use = (d2 > rc2) & (d2 <= rl2)
        use[np.arange(len(tg)), tg] = False
        sh = L * nint((x[sw][None, :, :] - cent[tg][:, None, :]) / L)             # [target][source group][3]
        dr = x[src][None, :, :] - cent[tg][:, None, :] - sh[:, sgrp, :]           # [target][atom][3]
        w = use[:, sgrp]
        r2 = (dr * dr).sum(2)
        r2 = np.where(w, r2, 1.0)
        f0 = np.where(w, q[None, :] / (r2 * np.sqrt(r2)), 0.0)
        f1 = 3.0 * f0 / r2
        f2 = -f1 / r2
        out[tg, 3] = (f0 * r2).sum(1)
        out[tg, 4:7] = -(dr * f0[:, :, None]).sum(1)
        drT = dr.transpose(0, 2, 1)                                                # [t][3][a]
        phi2 = (drT * f1[:, None, :]) @ dr                                         # sum_a f1 dr_k dr_l
        phi2 -= f0.sum(1)[:, None, None] * np.eye(3)[None]
        out[tg, 7:16] = phi2.reshape(len(tg), 9)
        # phi3(n, j, c) = 5 f2 dr_n dr_j dr_c - f2 r2 (d_nj dr_c + d_nc dr_j + d_jc dr_n)
        nj = (drT[:, :, None, :] * drT[:, None, :, :]).reshape(len(tg), 9, -1)   # [t][(n, j)][a]
        phi3 = ((nj * (5.0 * f2)[:, None, :]) @ dr).reshape(len(tg), 3, 3, 3)
        gs = ((f2 * r2)[:, :, None] * dr).sum(1)                                   # [t][3]
        I = np.eye(3)
        phi3 -= (I[None, :, :, None] * gs[:, None, None, :] + I[None, :, None, :] * gs[:, None, :, None]
                 + I[None, None, :, :] * gs[:, :, None, None])
        out[tg, 16:43] = phi3.reshape(len(tg), 27)
    return out


def box_lrf_taylor(s, x, lrf):
    """lrf_taylor (src/nonbondene.f90:507-571) with use_PBC: every non-Q atom
    (excluded atoms included) takes the Taylor potential and field of its own
    group's record.  Returns (E_LRF, gradient)."""
    x = np.asarray(x, np.float64)
    groups = _all_groups(s)
    isq = np.zeros(s.natom, bool)
    isq[np.asarray(s.iqseq, np.int64)] = True
    gof = np.zeros(s.natom, np.int64)
    for g, a in enumerate(groups):
        gof[a] = g
    i = np.nonzero(~isq)[0]
    R = lrf[gof[i]]
    dr = R[:, :3] - x[i]
    phi0, phi1 = R[:, 3], R[:, 4:7]
    phi2 = R[:, 7:16].reshape(-1, 3, 3)
    phi3 = R[:, 16:43].reshape(-1, 9, 3)
    t2 = np.einsum("akl,al->ak", phi2, dr)                   # tmp_k = dr . phi2(k)
    V = phi0 + (dr * phi1).sum(1) + 0.5 * (dr * t2).sum(1)
    q = np.asarray(s.crg, np.float64)[i]
    E = float((0.5 * q * V).sum())
    t3 = np.einsum("amc,ac->am", phi3, dr).reshape(-1, 3, 3)   # [atom][k][j] = dr . phi3(3k + j)
    df = phi1 + t2 + 0.5 * np.einsum("akj,aj->ak", t3, dr)
    d = np.zeros_like(x)
    d[i] -= df * q[:, None]
    return E, d


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
