"""Oracle (test infrastructure only): monitor-group energies and the excluded
interactions of group contributions, restated from Q6 in plain Python/numpy.
The product computes these on the GPU (k_pair_sets); nothing in the package
imports this file.

Q6 sources restated (paths within the Q6 tree):
  pair values    src/simprep.f90:3321-3351 (precompute_set_values_pp),
                 3390-3438 (_qp), 3442-3512 (_qq), 3112-3148 (qp_int_comp),
                 3152-3260 (qq_int_comp: Q-Q pairs, then the Q-bonded-P
                 pairs of atoms bonded or angled to a Q atom)
  pair energy    src/nonbonded.f90:111-150 (nbe_qq), 200-222 (nbe_qx)
  monitors       src/nonbondene.f90:4517-4680 (nbmonitorlist, nonbond_monitor)
  exclusions     src/simprep.f90:2879-2945 (exc_assign),
                 src/nonbondene.f90:6825-6920 (calculate_exc)
Two index slips of nbmonitorlist (pp_map indexed by the loop counters,
qp_precomp with its arguments swapped) and the fill of exc_assign (which
covers only the Q-Q pairs whose higher Q index is in the group, and checks
qp_precomp(iq,iq) for the plain Q-P pairs) are not restated: the pairs are
the ones the reference's counting loops name, each with its own values.
"""
from __future__ import annotations

import numpy as np

QREAL_EPS = 1e-10


def _combine(rule, ai, aj, bi, bj, arith_soft=False):
    if rule == 1:
        return ai * aj, bi * bj
    if arith_soft:
        return ai * aj, bi * bj
    a = (ai + aj) ** 2
    a = a * a * a
    b = bi * bj
    return a * a * b, 2.0 * a * b


def _set(A, B, el):
    return abs(A) > QREAL_EPS or abs(B) > QREAL_EPS or abs(el) > QREAL_EPS


class PairValues:
    """The precomputed pair values of one system (qq, Q-P, P-P)."""

    def __init__(self, s):
        self.s = s
        ns, nq, S = s.nat_solute, s.nqat, s.nstates
        self.iqatom = np.full(s.natom, -1, np.int64)
        self.iqatom[np.asarray(s.iqseq)] = np.arange(nq)
        qconn = np.asarray(s.qconn)               # [S][ns][nq]
        self.qconn = qconn
        self.qnear = np.zeros(s.natom, bool)
        if nq:
            self.qnear[:ns] = (qconn <= 3).any(axis=(0, 2))
        self.nt = np.asarray(s.avdw).shape[0]
        sp = {}
        for a, b in np.asarray(s.pairs14).reshape(-1, 2):
            sp[(min(a, b), max(a, b))] = 3
        for a, b in np.asarray(s.excl_pairs).reshape(-1, 2):
            sp[(min(a, b), max(a, b))] = 1        # exclusion wins
        self.special = sp

    # precompute_set_values_qp (Q index iq, solute atom j, state, code)
    def qp(self, iq, j, st, vdw):
        s = self.s
        i = int(s.iqseq[iq])
        qvdw = 1 if vdw == 2 else vdw
        tj = int(s.iac[j])
        if s.qvdw_flag:
            qt = int(s.qiac[iq, st])
            qa, qb = s.qavdw[qt, qvdw - 1], s.qbvdw[qt, qvdw - 1]
        else:
            qa, qb = s.avdw[s.iac[i], vdw - 1], s.bvdw[s.iac[i], vdw - 1]
        A, B = _combine(s.ivdw_rule, qa, s.avdw[tj, vdw - 1], qb, s.bvdw[tj, vdw - 1])
        el = s.crg[i] * s.crg[j] if s.qq_use_library_charges else s.qcrg[iq, st] * s.crg[j]
        ok = _set(A, B, el)
        sc = s.sc_lookup[iq, tj, st]
        if vdw == 3:
            el = el * s.el14_scale
        return ok, (float(A), float(B), float(el), float(sc), 0)

    # qq_int_comp + precompute_set_values_qq (iq < jq)
    def qq(self, iq, jq, st):
        s = self.s
        ia, ja = int(s.iqseq[iq]), int(s.iqseq[jq])
        if self.qconn[st, ja, iq] < 4:
            return False, None
        els = 1.0
        for e, (k, l) in enumerate(np.asarray(s.el_scale_pairs).reshape(-1, 2)):
            if (iq == k and jq == l) or (iq == l and jq == k):
                els = s.el_scale[e, st]
                break
        if self.qconn[st, ja, iq] == 4:
            vdw = 3
        elif not s.qvdw_flag:
            vdw = int(s.ljcod[s.iac[ia], s.iac[ja]])
        else:
            vdw = 1
            for a, b in np.asarray(s.qexpnb_pairs).reshape(-1, 2):
                if (iq == a and jq == b) or (jq == a and iq == b):
                    vdw = 2
                    break
        k = vdw - 1
        if s.qvdw_flag:
            ti, tj = int(s.qiac[iq, st]), int(s.qiac[jq, st])
            ai, aj, bi, bj = s.qavdw[ti, k], s.qavdw[tj, k], s.qbvdw[ti, k], s.qbvdw[tj, k]
        else:
            ai, aj = s.avdw[s.iac[ia], k], s.avdw[s.iac[ja], k]
            bi, bj = s.bvdw[s.iac[ia], k], s.bvdw[s.iac[ja], k]
        A, B = _combine(s.ivdw_rule, ai, aj, bi, bj, arith_soft=(vdw == 2 and s.qvdw_flag))
        el = s.crg[ia] * s.crg[ja] if s.qq_use_library_charges else s.qcrg[iq, st] * s.qcrg[jq, st]
        el = el * els
        sc = s.sc_lookup[iq, self.nt + jq, st]
        ok = _set(A, B, el)
        if vdw == 3:
            el = el * s.el14_scale
        return ok, (float(A), float(B), float(el), float(sc), 1 if (vdw == 2 and s.qvdw_flag) else 0)

    # a Q atom with a non-Q solute atom: Q-bonded-P values (qq_int_comp's
    # second loop) or qp_int_comp's
    def q_with_p(self, iq, j, st):
        s = self.s
        ia = int(s.iqseq[iq])
        qc = self.qconn[st, j, iq]
        if self.qnear[j]:
            if qc < 4:
                return False, None
            if qc == 4:
                vdw = 3
            elif s.qvdw_flag:
                vdw = 1
            else:
                vdw = int(s.ljcod[s.iac[ia], s.iac[j]])
            return self.qp(iq, j, st, vdw)
        # qp_int_comp carries vdw = 3 over to the later states once a state
        # has qconn 4
        vdw = int(s.ljcod[s.iac[j], s.iac[ia]])
        for st2 in range(st + 1):
            if self.qconn[st2, j, iq] == 4:
                vdw = 3
        return self.qp(iq, j, st, vdw)

    # precompute_set_values_pp
    def pp(self, a, b):
        s = self.s
        i, j = min(a, b), max(a, b)
        code = self.special.get((i, j), int(s.ljcod[s.iac[i], s.iac[j]]))
        if code == 1 and (i, j) in self.special:
            return False, None
        ti, tj = int(s.iac[i]), int(s.iac[j])
        A, B = _combine(s.ivdw_rule, s.avdw[ti, code - 1], s.avdw[tj, code - 1], s.bvdw[ti, code - 1],
                        s.bvdw[tj, code - 1])
        el = s.crg[i] * s.crg[j]
        ok = _set(A, B, el)
        if code == 3:
            el = el * s.el14_scale
        return ok, (float(A), float(B), float(el), 0.0, 0)


def nbe(x, i, j, par):
    """nbe_qq's Vel and V_a - V_b (the soft branch for soft Q-Q pairs)."""
    A, B, el, sc, soft = par
    d = np.asarray(x[j], np.float64) - np.asarray(x[i], np.float64)
    r2 = 1.0 / float(d @ d)
    r = np.sqrt(r2)
    vel = el * r
    if soft:
        return vel, A * np.exp(-B / r)
    r6 = 1.0 / (1.0 / (r2 * r2 * r2) + sc)
    return vel, A * r6 * r6 - B * r6


def monitor_energies(s, x, groups, pairs):
    """[npairs][nstates][2] = Vel, Vlj of nonbond_monitor."""
    pv = PairValues(s)
    S = s.nstates
    out = np.zeros((len(pairs), S, 2))
    for p, (gi, gj) in enumerate(pairs):
        for a in groups[gi]:
            for b in groups[gj]:
                a, b = int(a), int(b)
                if a == b:
                    raise ValueError("two paired monitor atom groups contain the same atom")
                qa, qb = pv.iqatom[a], pv.iqatom[b]
                for st in range(S):
                    if qa >= 0 and qb >= 0:
                        ok, par = pv.qq(min(qa, qb), max(qa, qb), st)
                        i, j = int(s.iqseq[min(qa, qb)]), int(s.iqseq[max(qa, qb)])
                    elif qa >= 0 or qb >= 0:
                        iq, j = (qa, b) if qa >= 0 else (qb, a)
                        ok, par = pv.q_with_p(int(iq), j, st)
                        i = int(s.iqseq[iq])
                    else:
                        ok, par = pv.pp(a, b)
                        i, j = min(a, b), max(a, b)
                    if ok:
                        out[p, st] += nbe(x, i, j, par)
    return out


def group_exclusions(s, x, masks):
    """[ngroups][nstates][4] = qq el, qq vdw, qp el, qp vdw of the
    interactions calculate_exc subtracts for each group."""
    pv = PairValues(s)
    S, nq = s.nstates, s.nqat
    out = np.zeros((len(masks), S, 4))
    for g, mk in enumerate(masks):
        mk = np.asarray(mk).astype(bool)
        for st in range(S):
            for iq in range(nq):
                for jq in range(iq + 1, nq):
                    ia, ja = int(s.iqseq[iq]), int(s.iqseq[jq])
                    if not (mk[ia] or mk[ja]):
                        continue
                    ok, par = pv.qq(iq, jq, st)
                    if ok:
                        out[g, st, 0:2] += nbe(x, ia, ja, par)
            for j in np.nonzero(mk)[0]:
                j = int(j)
                if pv.iqatom[j] >= 0:
                    continue
                for iq in range(nq):
                    ok, par = pv.q_with_p(iq, j, st)
                    if ok:
                        out[g, st, 2:4] += nbe(x, int(s.iqseq[iq]), j, par)
    return out
