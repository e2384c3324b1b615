"""TEST INFRASTRUCTURE ONLY: FP64 reference of the Q-atom energies and their
parameter gradient, written in numpy independently of the C oracle.

For every FEP state s, E_s is the state's unweighted Q-atom nonbonded energy
(EQ(s)%qq + %qp + %qw, Q6 src/potene.f90:224-230): the dynamic Q-solute and
Q-water lists (nbqplist, nbqwlist with the spherical Rcq test about xpcent,
src/nonbondene.f90:3647-3742, 3862-3944), the static Q-Q and Q-bonded-solute
lists (qq_int_comp + nbqqlist, src/simprep.f90:3152-3268,
src/nonbondene.f90:3231-3282) with the pair values of
precompute_set_values_qp/qq/qw (src/simprep.f90:3390-3558, including the
sticky 1-4 code of qp_int_comp, 3134-3137), and the pair energies of nbe_qx,
nbe_qspc and nbe_qq (src/nonbonded.f90:111-150, 200-243):
    E = el / r + A u^2 - B u,   u = 1 / (r^6 + alpha).

The parameters are, per Q atom and state, the scaled charge qcrg and the Q
atom's code-1 LJ factors a, b (qavdw/qbvdw of its Q type with Q types on, else
the factors of its own atom type).  ``evaluate`` returns E_s and dE_s/dq,
dE_s/da, dE_s/db, the latter analytically for either combination rule
(geometric A = a_i a_j, B = b_i b_j; arithmetic A = (a_i + a_j)^12 b_i b_j,
B = 2 (a_i + a_j)^6 b_i b_j, src/simprep.f90:3326-3341), for given parameter
arrays, so that central differences of E_s can be taken too.  The
exponential soft pairs are not parameterised by a, b and raise here.
"""
from __future__ import annotations

import numpy as np


class QEnergyReference:
    def __init__(self, s, Rcq: float = 99.0):
        if len(np.asarray(s.qexpnb_pairs).reshape(-1, 2)) and s.qvdw_flag:
            raise NotImplementedError("exponential soft pairs")
        self.s = s
        self.S, self.nq = int(s.nstates), int(s.nqat)
        self.arith = int(s.ivdw_rule) == 2
        self.Rcq2 = Rcq * Rcq
        nt = int(s.natyps)
        iac = np.asarray(s.iac)
        self.iqseq = np.asarray(s.iqseq)
        qatom = np.full(s.natom, -1)
        qatom[self.iqseq] = np.arange(self.nq)
        qconn = np.asarray(s.qconn)               # [S, nat_solute, nq]
        near = (qconn <= 3).any(axis=(0, 2)) if s.nat_solute else np.zeros(0, bool)
        ljcod = np.asarray(s.ljcod).reshape(nt, nt)
        el14 = float(s.el14_scale)
        terms = []        # (iq, j_atom, state, Q-side code column, elec factor, alpha, env a, env b)
        ns = int(s.nat_solute)
        sc = np.asarray(s.sc_lookup)              # [nq, natyps + nq, S]

        def q_factors(iq, st, k):
            if s.qvdw_flag:
                t = int(s.qiac[iq, st])
                return float(s.qavdw[t, k]), float(s.qbvdw[t, k])
            ti = int(iac[self.iqseq[iq]])
            return float(s.avdw[ti, k]), float(s.bvdw[ti, k])

        self.q_factors = q_factors
        # dynamic Q-solute list: every non-near solute atom of a non-excluded
        # group whose switch atom is inside Rcq of xpcent (nbqplist)
        qp_atoms = []
        xp = np.asarray(s.xpcent, float)
        for g in range(int(s.ncgp_solute)):
            sw = int(s.cgp_iswitch[g])
            if s.excl[sw]:
                continue
            if float(((np.asarray(s.x)[sw] - xp) ** 2).sum()) > self.Rcq2:
                continue
            for a in np.asarray(s.cgpatom)[s.cgp_first[g]:s.cgp_last[g] + 1]:
                if not near[a]:
                    qp_atoms.append(int(a))
        for j in qp_atoms:
            for iq in range(self.nq):
                vdw = int(ljcod[iac[j], iac[self.iqseq[iq]]])
                for st in range(self.S):
                    if qconn[st, j, iq] == 4:
                        vdw = 3                    # kept for later states (qp_int_comp)
                    terms.append(self._env_term("qp", iq, j, st, vdw, el14, sc, nt))
        # static Q-bonded solute atoms (nbqqlist's Q-P part)
        for j in range(ns):
            if qatom[j] >= 0 or not near[j]:
                continue
            for iq in range(self.nq):
                for st in range(self.S):
                    qc = int(qconn[st, j, iq])
                    if qc < 4:
                        continue
                    vdw = 3 if qc == 4 else (1 if s.qvdw_flag else int(ljcod[iac[self.iqseq[iq]], iac[j]]))
                    t = self._env_term("qqp", iq, j, st, vdw, el14, sc, nt)
                    if t is not None:
                        terms.append(t)
        self.terms_env = terms
        # Q-Q pairs (qq_int_comp)
        qq = []
        elp = np.asarray(s.el_scale_pairs).reshape(-1, 2)
        elv = np.asarray(s.el_scale).reshape(-1, self.S)
        for iq in range(self.nq - 1):
            ia = int(self.iqseq[iq])
            for jq in range(iq + 1, self.nq):
                ja = int(self.iqseq[jq])
                for st in range(self.S):
                    qc = int(qconn[st, ja, iq])
                    if qc < 4:
                        continue
                    els = 1.0
                    for e, (k_, l_) in enumerate(elp):
                        if (iq, jq) in ((k_, l_), (l_, k_)):
                            els = float(elv[e, st])
                            break
                    vdw = 3 if qc == 4 else (int(ljcod[iac[ia], iac[ja]]) if not s.qvdw_flag else 1)
                    qq.append((iq, jq, st, vdw - 1, els * (el14 if vdw == 3 else 1.0),
                               float(sc[iq, nt + jq, st])))
        self.terms_qq = qq
        # dynamic Q-water list: waters whose first atom is inside Rcq of xpcent
        self.qw_waters = []
        for w in range(int(s.nwat)):
            o = ns + s.solv_atom * w
            if s.excl[o]:
                continue
            if float(((np.asarray(s.x)[o] - xp) ** 2).sum()) <= self.Rcq2:
                self.qw_waters.append(o)
        qw = []
        for iq in range(self.nq):
            for a in range(s.solv_atom):
                tw = int(iac[ns + a])
                vdw = int(ljcod[tw, iac[self.iqseq[iq]]])
                lj = not (s.solvent_type == 0 and a > 0)   # nbe_qspc: SPC hydrogens Coulomb only
                for st in range(self.S):
                    qk = 0 if (vdw == 2 and s.qvdw_flag) else vdw - 1
                    qw.append((iq, a, st, qk, float(s.crg[ns + a]), float(sc[iq, tw, st]),
                               float(s.avdw[tw, vdw - 1]), float(s.bvdw[tw, vdw - 1]), lj))
        self.terms_qw = qw
        self._compile()

    def _env_term(self, kind, iq, j, st, vdw, el14, sc, nt):
        s = self.s
        qk = 0 if (vdw == 2 and s.qvdw_flag) else vdw - 1   # Q types read code 1 for type-2 pairs
        tj = int(s.iac[j])
        aj, bj = float(s.avdw[tj, vdw - 1]), float(s.bvdw[tj, vdw - 1])
        elfac = float(s.crg[j]) * (el14 if vdw == 3 else 1.0)
        qa, qb = self.q_factors(iq, st, qk)
        A, B = self._combine(qa, aj, qb, bj)
        el = float(s.qcrg[iq, st]) * float(s.crg[j])
        if kind == "qqp" and not (abs(A) > 1e-10 or abs(B) > 1e-10 or abs(el) > 1e-10):
            return None                              # not set: not listed (nbqqlist)
        return (iq, j, st, qk, elfac, float(sc[iq, tj, st]), aj, bj)

    def _combine(self, ai, aj, bi, bj):
        if not self.arith:
            return ai * aj, bi * bj
        t = (ai + aj) ** 6
        return t * t * bi * bj, 2.0 * t * bi * bj

    def _compile(self):
        e = self.terms_env
        self.e_iq = np.array([t[0] for t in e], int)
        self.e_j = np.array([t[1] for t in e], int)
        self.e_s = np.array([t[2] for t in e], int)
        self.e_qk = np.array([t[3] for t in e], int)
        self.e_el = np.array([t[4] for t in e], float)
        self.e_sc = np.array([t[5] for t in e], float)
        self.e_a = np.array([t[6] for t in e], float)
        self.e_b = np.array([t[7] for t in e], float)
        q = self.terms_qq
        self.q_i = np.array([t[0] for t in q], int)
        self.q_j = np.array([t[1] for t in q], int)
        self.q_s = np.array([t[2] for t in q], int)
        self.q_k = np.array([t[3] for t in q], int)
        self.q_f = np.array([t[4] for t in q], float)
        self.q_sc = np.array([t[5] for t in q], float)
        w = self.terms_qw
        self.w_iq = np.array([t[0] for t in w], int)
        self.w_a = np.array([t[1] for t in w], int)
        self.w_s = np.array([t[2] for t in w], int)
        self.w_qk = np.array([t[3] for t in w], int)
        self.w_el = np.array([t[4] for t in w], float)
        self.w_sc = np.array([t[5] for t in w], float)
        self.w_ea = np.array([t[6] for t in w], float)
        self.w_eb = np.array([t[7] for t in w], float)
        self.w_lj = np.array([t[8] for t in w], bool)

    def parameters(self):
        """(q, a, b), each [nq, S]: the charges (scaled) and code-1 factors."""
        s = self.s
        q = np.array(s.qcrg, float).reshape(self.nq, self.S).copy()
        a = np.zeros((self.nq, self.S))
        b = np.zeros((self.nq, self.S))
        for iq in range(self.nq):
            for st in range(self.S):
                a[iq, st], b[iq, st] = self.q_factors(iq, st, 0)
        return q, a, b

    def _q_side(self, iq, st, qk, a, b):
        """Factors of the Q side: the parameters for code 1, the fixed type
        values for codes 2 and 3."""
        fa = np.empty(len(iq))
        fb = np.empty(len(iq))
        for n in range(len(iq)):
            if qk[n] == 0:
                fa[n], fb[n] = a[iq[n], st[n]], b[iq[n], st[n]]
            else:
                fa[n], fb[n] = self.q_factors(int(iq[n]), int(st[n]), int(qk[n]))
        return fa, fb

    def _lj(self, ai, aj, bi, bj, u):
        """Energy and d/d(ai), d/d(bi) of A u^2 - B u."""
        if not self.arith:
            A, B = ai * aj, bi * bj
            return A * u * u - B * u, aj * u * u, -bj * u
        S = ai + aj
        t6 = S ** 6
        tB = bi * bj
        A, B = t6 * t6 * tB, 2.0 * t6 * tB
        dA_da, dB_da = 12.0 * t6 * S ** 5 * tB, 12.0 * S ** 5 * tB
        dA_db, dB_db = t6 * t6 * bj, 2.0 * t6 * bj
        return A * u * u - B * u, dA_da * u * u - dB_da * u, dA_db * u * u - dB_db * u

    def _geometry(self, x, i, j):
        d = x[j] - x[i]
        r2 = (d * d).sum(-1)
        return 1.0 / np.sqrt(r2), r2 ** 3

    def _env_geometry(self, x):
        """Per env term and per qw term (per water): 1/r and r^6."""
        out = []
        if len(self.e_iq):
            out.append(self._geometry(x, self.iqseq[self.e_iq], self.e_j))
        else:
            out.append((np.zeros(0), np.zeros(0)))
        ow = np.array(self.qw_waters, int)
        if len(ow) and len(self.w_iq):
            i = np.repeat(self.iqseq[self.w_iq], len(ow))
            j = (ow[None, :] + self.w_a[:, None]).ravel()
            ri, r6 = self._geometry(x, i, j)
            out.append((ri.reshape(len(self.w_iq), len(ow)), r6.reshape(len(self.w_iq), len(ow))))
        else:
            out.append((np.zeros((len(self.w_iq), 0)), np.zeros((len(self.w_iq), 0))))
        if len(self.q_i):
            out.append(self._geometry(x, self.iqseq[self.q_i], self.iqseq[self.q_j]))
        else:
            out.append((np.zeros(0), np.zeros(0)))
        return out

    def _terms(self, geo, q, a, b, side_j=None):
        """Energies of every term: (env [n_env], qw [n_qw], qq [n_qq]).  For
        the Q-Q terms the j side's parameters come from side_j = (q, a, b)
        when given (else the same arrays)."""
        (e_ri, e_r6), (w_ri, w_r6), (q_ri, q_r6) = geo
        E_env = np.zeros(len(self.e_iq))
        if len(self.e_iq):
            u = 1.0 / (e_r6 + self.e_sc)
            fa, fb = self._q_side(self.e_iq, self.e_s, self.e_qk, a, b)
            lj, _, _ = self._lj(fa, self.e_a, fb, self.e_b, u)
            E_env = q[self.e_iq, self.e_s] * self.e_el * e_ri + lj
        E_qw = np.zeros(len(self.w_iq))
        for n in range(len(self.w_iq)):
            iq, st, qk = self.w_iq[n], self.w_s[n], self.w_qk[n]
            e = q[iq, st] * self.w_el[n] * w_ri[n]
            if self.w_lj[n]:
                u = 1.0 / (w_r6[n] + self.w_sc[n])
                qa, qb = (a[iq, st], b[iq, st]) if qk == 0 else self.q_factors(int(iq), int(st), int(qk))
                e = e + self._lj(qa, self.w_ea[n], qb, self.w_eb[n], u)[0]
            E_qw[n] = e.sum()
        E_qq = np.zeros(len(self.q_i))
        if len(self.q_i):
            qj_, aj_, bj_ = side_j if side_j is not None else (q, a, b)
            u = 1.0 / (q_r6 + self.q_sc)
            fai, fbi = self._q_side(self.q_i, self.q_s, self.q_k, a, b)
            faj, fbj = self._q_side(self.q_j, self.q_s, self.q_k, aj_, bj_)
            E_qq = q[self.q_i, self.q_s] * qj_[self.q_j, self.q_s] * self.q_f * q_ri + \
                self._lj(fai, faj, fbi, fbj, u)[0]
        return E_env, E_qw, E_qq

    def _state_sums(self, E_env, E_qw, E_qq):
        E = np.zeros(self.S)
        np.add.at(E, self.e_s, E_env)
        np.add.at(E, self.w_s, E_qw)
        np.add.at(E, self.q_s, E_qq)
        return E

    def energies(self, x, q=None, a=None, b=None):
        """E_s [S] at x for the given parameters (default: the system's)."""
        p = self.parameters()
        q = p[0] if q is None else q
        a = p[1] if a is None else a
        b = p[2] if b is None else b
        return self._state_sums(*self._terms(self._env_geometry(np.asarray(x, float)), q, a, b))

    def finite_differences(self, x, h=1e-5):
        """Central differences dE_s/dp, p = (q, a, b) [nq, S] each, step
        h * max(1, |p|).  Every Q-environment term holds one parameter, so all
        of them are stepped at once and each term's difference is credited to
        its own parameter; a Q-Q term holds one per side, stepped one side at
        a time.  The result is the central difference of E_s in each parameter
        alone, since no other term depends on it."""
        geo = self._env_geometry(np.asarray(x, float))
        base = list(self.parameters())
        out = []
        for kind in range(3):
            p = base[kind]
            step = h * np.maximum(1.0, np.abs(p))
            g = np.zeros_like(p)
            plus, minus = [v.copy() for v in base], [v.copy() for v in base]
            plus[kind] = p + step
            minus[kind] = p - step
            Ep = self._terms(geo, *plus, side_j=base)
            Em = self._terms(geo, *minus, side_j=base)
            np.add.at(g, (self.e_iq, self.e_s), Ep[0] - Em[0])
            np.add.at(g, (self.w_iq, self.w_s), Ep[1] - Em[1])
            np.add.at(g, (self.q_i, self.q_s), Ep[2] - Em[2])
            Ep = self._terms(geo, *base, side_j=plus)
            Em = self._terms(geo, *base, side_j=minus)
            np.add.at(g, (self.q_j, self.q_s), Ep[2] - Em[2])
            out.append(g / (2.0 * step))
        return tuple(out)

    def evaluate(self, x, q=None, a=None, b=None):
        """(E [S], dE/dq [nq, S], dE/da [nq, S], dE/db [nq, S]) at x."""
        x = np.asarray(x, float)
        p = self.parameters()
        q = p[0] if q is None else q
        a = p[1] if a is None else a
        b = p[2] if b is None else b
        S, nq = self.S, self.nq
        E = np.zeros(S)
        gq, ga, gb = np.zeros((nq, S)), np.zeros((nq, S)), np.zeros((nq, S))
        (e_ri, e_r6), (w_ri, w_r6), (q_ri, q_r6) = self._env_geometry(x)
        # Q-environment solute pairs
        if len(self.e_iq):
            u = 1.0 / (e_r6 + self.e_sc)
            fa, fb = self._q_side(self.e_iq, self.e_s, self.e_qk, a, b)
            qv = q[self.e_iq, self.e_s]
            lj, dla, dlb = self._lj(fa, self.e_a, fb, self.e_b, u)
            np.add.at(E, self.e_s, qv * self.e_el * e_ri + lj)
            np.add.at(gq, (self.e_iq, self.e_s), self.e_el * e_ri)
            c1 = self.e_qk == 0
            np.add.at(ga, (self.e_iq[c1], self.e_s[c1]), dla[c1])
            np.add.at(gb, (self.e_iq[c1], self.e_s[c1]), dlb[c1])
        # Q-water pairs
        for n in range(len(self.w_iq)):
            iq, st, qk = self.w_iq[n], self.w_s[n], self.w_qk[n]
            e = q[iq, st] * self.w_el[n] * w_ri[n]
            gq[iq, st] += (self.w_el[n] * w_ri[n]).sum()
            if self.w_lj[n]:
                u = 1.0 / (w_r6[n] + self.w_sc[n])
                qa, qb = (a[iq, st], b[iq, st]) if qk == 0 else self.q_factors(int(iq), int(st), int(qk))
                lj, dla, dlb = self._lj(qa, self.w_ea[n], qb, self.w_eb[n], u)
                e = e + lj
                if qk == 0:
                    ga[iq, st] += dla.sum()
                    gb[iq, st] += dlb.sum()
            E[st] += e.sum()
        # Q-Q pairs
        if len(self.q_i):
            u = 1.0 / (q_r6 + self.q_sc)
            qi, qj = q[self.q_i, self.q_s], q[self.q_j, self.q_s]
            fai, fbi = self._q_side(self.q_i, self.q_s, self.q_k, a, b)
            faj, fbj = self._q_side(self.q_j, self.q_s, self.q_k, a, b)
            lj, dlai, dlbi = self._lj(fai, faj, fbi, fbj, u)
            _, dlaj, dlbj = self._lj(faj, fai, fbj, fbi, u)
            np.add.at(E, self.q_s, qi * qj * self.q_f * q_ri + lj)
            np.add.at(gq, (self.q_i, self.q_s), qj * self.q_f * q_ri)
            np.add.at(gq, (self.q_j, self.q_s), qi * self.q_f * q_ri)
            c1 = self.q_k == 0
            np.add.at(ga, (self.q_i[c1], self.q_s[c1]), dlai[c1])
            np.add.at(gb, (self.q_i[c1], self.q_s[c1]), dlbi[c1])
            np.add.at(ga, (self.q_j[c1], self.q_s[c1]), dlaj[c1])
            np.add.at(gb, (self.q_j[c1], self.q_s[c1]), dlbj[c1])
        return E, gq, ga, gb
