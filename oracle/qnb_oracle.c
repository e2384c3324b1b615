/*
 * qnb_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU FP64 restatement of Q6 qdyn's nonbonded path (spherical boundary,
 * switch-atom charge-group cut-offs) used as the parity checker for the CUDA
 * engine.  Only the test suite, the smoke check and the benchmark's CPU
 * baseline may load it; the product library never does.
 *
 * It follows the reference's serial (non-OpenMP) semantics and loop order:
 * same list order, same summation order, strict IEEE double arithmetic (the
 * build uses -ffp-contract=off and no fast-math).  Every routine cites the Q6
 * source lines it restates (paths relative to the Q6 tree).
 *
 * Parity pinning: the step-0 energies of the reference's own regression test
 * (tests/basic_tests, lig_w.top) are reproduced by tests/test_golden.py.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/qnb.h"

#define QREAL_EPS 1.0e-10 /* src/sizes.f90:50 (QDOUBLE) */
#define NLRF 43

typedef struct { double x, y, z; } v3;

static inline v3 vsub(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline v3 vadd(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static inline v3 vscale(v3 a, double s) { v3 r = {a.x * s, a.y * s, a.z * s}; return r; }
/* qvec_square, src/math.f90:206-212 */
static inline double vsq(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline double vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

typedef struct { int i, j; double A, B, el; } nb_t;            /* NB_TYPE */
typedef struct { int i, j; double A, B, el, sc; int soft; } nbq_t; /* NBQ(P)_TYPE */
typedef struct { double A, B, el, sc; int set; int soft; } pre_t; /* PRECOMPUTE_INT */

typedef struct {
    void* p; long n, cap; size_t sz;
} vec_t;

static void* vpush(vec_t* v) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 1024;
        v->p = realloc(v->p, v->cap * v->sz);
    }
    return (char*)v->p + (v->n++) * v->sz;
}

typedef struct orc {
    /* topology copies */
    int natom, nat_solute, nwat, solv_atom, solvent_type, natyps, ivdw_rule;
    double el14;
    double *crg; int *iac; uint8_t *excl, *heavy;
    double *avdw, *bvdw; uint8_t* ljcod;
    int ncgp, ncgp_solute; int *cfirst, *clast, *csw, *cgpatom; int *iwhich;
    long nex, n14; int64_t *exkeys, *k14;     /* sorted keys i*natom+j, i<j */
    int nqat, S, nqlib, qvdw_flag, qq_lib; int* iqseq; int* iqatom;
    double *qcrg, *qavdw, *qbvdw, *sc; int* qiac; int8_t* qconn;
    int nel; int* elp; double* elv; int nqexp; int* qexp;
    double xpcent[3], xwcent[3], rexcl_o;
    int use_lrf;
    int any_atom;
    /* nonbnd_solv_int: intra-molecular solvent pairs (offsets in a molecule) */
    int nsi; int *si_i, *si_j; double *si_A, *si_B, *si_el;       /* iuse_switch_atom == 0: the *lis2* group tests   */
    /* solvent (first molecule) parameters: chg_solv, aLJ_solv, bLJ_solv */
    double chg_solv[16], aLJ[16][3], bLJ[16][3];
    pre_t ww_pre[16][16];
    pre_t* pw_pre;      /* [nat_solute][solv_atom]                  */
    pre_t* qp_pre;      /* [nat_solute][nqat][S]                    */
    pre_t* qw_pre;      /* [nqat][solv_atom][S]                     */
    double lambda[64];
    /* lists */
    vec_t nbpp, nbpp14, nbpw, nbww, nbqp, nbqw; /* nbpp14: flag per nbpp entry */
    vec_t* nbqq;  vec_t* nbqqp;                 /* per state                   */
    int qp_done, qw_done;
    double* lrf; /* [ncgp][43] */
    /* solvent boundary */
    qnb_solvent_params sp; int have_sp;
    double *theta, *theta0, *tdum; int *list_sh, *nsort; int n_insh[16];
    double avtheta[16], avn_insh[16], theta_corr[16];
} orc;

static int cmp64(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return x < y ? -1 : x > y;
}
static int has_key(const int64_t* k, long n, int64_t key) {
    long lo = 0, hi = n - 1;
    while (lo <= hi) {
        long m = (lo + hi) / 2;
        if (k[m] == key) return 1;
        if (k[m] < key) lo = m + 1; else hi = m - 1;
    }
    return 0;
}
static int64_t* make_keys(const int32_t* pairs, long n, int natom) {
    int64_t* k = (int64_t*)malloc(sizeof(int64_t) * (n ? n : 1));
    for (long p = 0; p < n; ++p) {
        int a = pairs[2 * p], b = pairs[2 * p + 1];
        if (a > b) { int t = a; a = b; b = t; }
        k[p] = (int64_t)a * natom + b;
    }
    qsort(k, n, sizeof(int64_t), cmp64);
    return k;
}
static inline int is_excl(const orc* o, int i, int j) {
    if (i > j) { int t = i; i = j; j = t; }
    return has_key(o->exkeys, o->nex, (int64_t)i * o->natom + j);
}
static inline int is_14(const orc* o, int i, int j) {
    if (i > j) { int t = i; i = j; j = t; }
    return has_key(o->k14, o->n14, (int64_t)i * o->natom + j);
}
static inline int QCONN(const orc* o, int s, int i, int iq) {
    return o->qconn[s + o->S * (i + o->nat_solute * iq)];
}
static inline int any_qconn_le3(const orc* o, int i) {
    for (int iq = 0; iq < o->nqat; ++iq)
        for (int s = 0; s < o->S; ++s)
            if (QCONN(o, s, i, iq) <= 3) return 1;
    return 0;
}
#define QCRG(o, iq, s) ((o)->qcrg[(iq) + (o)->nqat * (s)])
#define QIAC(o, iq, s) ((o)->qiac[(iq) + (o)->nqat * (s)])
#define SCL(o, iq, t, s) ((o)->sc[(iq) + (o)->nqat * ((t) + ((o)->natyps + (o)->nqat) * (s))])
#define AV(o, t, k) ((o)->avdw[(t) * 3 + (k)])
#define BV(o, t, k) ((o)->bvdw[(t) * 3 + (k)])
#define QAV(o, t, k) ((o)->qavdw[(t) * 3 + (k)])
#define QBV(o, t, k) ((o)->qbvdw[(t) * 3 + (k)])

/* combination rules, src/simprep.f90:3326-3341 (vdw is the 1-based code) */
static void combine(int rule, double ai, double aj, double bi, double bj, double* A, double* B) {
    if (rule == 1) {
        *A = ai * aj;
        *B = bi * bj;
    } else {
        double tA = ai + aj;
        tA = tA * tA;
        tA = tA * tA * tA;
        double tB = bi * bj;
        *A = (tA * tA) * tB;
        *B = 2.0 * tA * tB;
    }
}
static int nonzero3(double A, double B, double el) {
    return fabs(A - 0.0) > QREAL_EPS || fabs(B - 0.0) > QREAL_EPS || fabs(el - 0.0) > QREAL_EPS;
}

/* precompute_set_values_pp, src/simprep.f90:3321-3350 */
static pre_t pp_values(const orc* o, int i, int j, int vdw) {
    pre_t p = {0};
    int k = vdw - 1, ti = o->iac[i], tj = o->iac[j];
    combine(o->ivdw_rule, AV(o, ti, k), AV(o, tj, k), BV(o, ti, k), BV(o, tj, k), &p.A, &p.B);
    p.el = o->crg[i] * o->crg[j];
    p.set = nonzero3(p.A, p.B, p.el);
    if (vdw == 3) p.el = p.el * o->el14;
    return p;
}

/* pp_int_comp's classification of one oriented pair, src/simprep.f90:2992-3053:
   returns 0 excluded, 3 for 1-4, else ljcod(iac(i),iac(j)) */
static int pp_code(const orc* o, int i, int j) {
    if (is_excl(o, i, j)) return 0;
    if (is_14(o, i, j)) return 3;
    return o->ljcod[o->iac[i] * o->natyps + o->iac[j]];
}

/* precompute_set_values_qp, src/simprep.f90:3390-3438 */
static pre_t qp_values(const orc* o, int iq, int j, int s, int vdw) {
    pre_t p = {0};
    int i = o->iqseq[iq];
    int qvdw = (vdw == 2) ? 1 : vdw;
    int k = vdw - 1, qk = qvdw - 1;
    int tj = o->iac[j];
    if (o->ivdw_rule == 1) {
        if (o->qvdw_flag) {
            p.A = QAV(o, QIAC(o, iq, s), qk) * AV(o, tj, k);
            p.B = QBV(o, QIAC(o, iq, s), qk) * BV(o, tj, k);
        } else {
            p.A = AV(o, o->iac[i], k) * AV(o, tj, k);
            p.B = BV(o, o->iac[i], k) * BV(o, tj, k);
        }
    } else {
        double tA, tB;
        if (o->qvdw_flag) {
            tA = QAV(o, QIAC(o, iq, s), qk) + AV(o, tj, k);
            tB = QBV(o, QIAC(o, iq, s), qk) * BV(o, tj, k);
        } else {
            tA = AV(o, o->iac[i], k) + AV(o, tj, k);
            tB = BV(o, o->iac[i], k) * BV(o, tj, k);
        }
        tA = tA * tA;
        tA = tA * tA * tA;
        p.A = (tA * tA) * tB;
        p.B = 2.0 * tA * tB;
    }
    p.el = o->qq_lib ? o->crg[i] * o->crg[j] : QCRG(o, iq, s) * o->crg[j];
    p.set = nonzero3(p.A, p.B, p.el);
    p.sc = SCL(o, iq, tj, s);
    if (vdw == 3) p.el = p.el * o->el14;
    return p;
}

/* precompute_set_values_qq, src/simprep.f90:3442-3512 */
static pre_t qq_values(const orc* o, int iq, int jq, int s, int vdw, double elscale) {
    pre_t p = {0};
    int i = o->iqseq[iq], j = o->iqseq[jq], k = vdw - 1;
    int ti = QIAC(o, iq, s), tj = QIAC(o, jq, s);
    if (o->ivdw_rule == 1) {
        if (o->qvdw_flag) {
            p.A = QAV(o, ti, k) * QAV(o, tj, k);
            p.B = QBV(o, ti, k) * QBV(o, tj, k);
        } else {
            p.A = AV(o, o->iac[i], k) * AV(o, o->iac[j], k);
            p.B = BV(o, o->iac[i], k) * BV(o, o->iac[j], k);
        }
    } else {
        double tA, tB;
        if (o->qvdw_flag) {
            tA = (vdw == 2) ? QAV(o, ti, k) * QAV(o, tj, k) : QAV(o, ti, k) + QAV(o, tj, k);
            tB = QBV(o, ti, k) * QBV(o, tj, k);
        } else {
            tA = AV(o, o->iac[i], k) + AV(o, o->iac[j], k);
            tB = BV(o, o->iac[i], k) * BV(o, o->iac[j], k);
        }
        if (vdw == 2 && o->qvdw_flag) {
            p.A = tA;
            p.B = tB;
        } else {
            tA = tA * tA;
            tA = tA * tA * tA;
            p.A = (tA * tA) * tB;
            p.B = 2.0 * tA * tB;
        }
    }
    p.el = o->qq_lib ? o->crg[i] * o->crg[j] : QCRG(o, iq, s) * QCRG(o, jq, s);
    p.el = p.el * elscale;
    p.sc = SCL(o, iq, o->natyps + jq, s);
    p.set = nonzero3(p.A, p.B, p.el);
    if (vdw == 3) p.el = p.el * o->el14;
    p.soft = (vdw == 2 && o->qvdw_flag);
    return p;
}

/* generic solvent-pair precompute with given per-side factors */
static pre_t solv_values(const orc* o, double ai, double aj, double bi, double bj, double el) {
    pre_t p = {0};
    combine(o->ivdw_rule, ai, aj, bi, bj, &p.A, &p.B);
    p.el = el;
    p.set = 1;
    return p;
}

static double* dup_d(const double* s, long n) {
    double* d = (double*)malloc(sizeof(double) * (n ? n : 1));
    if (n) memcpy(d, s, sizeof(double) * n);
    return d;
}
static int* dup_i(const int32_t* s, long n) {
    int* d = (int*)malloc(sizeof(int) * (n ? n : 1));
    for (long k = 0; k < n; ++k) d[k] = s[k];
    return d;
}
static uint8_t* dup_u8(const uint8_t* s, long n) {
    uint8_t* d = (uint8_t*)malloc(n ? n : 1);
    if (n) memcpy(d, s, n);
    return d;
}

/* ---- set-up: precompute_interactions (src/simprep.f90:2860-2870) ---------- */
orc* orc_create(const qnb_topology* t, int use_lrf) {
    orc* o = (orc*)calloc(1, sizeof(orc));
    o->natom = t->natom; o->nat_solute = t->nat_solute; o->nwat = t->nwat;
    o->solv_atom = t->solv_atom; o->solvent_type = t->solvent_type;
    o->natyps = t->natyps; o->ivdw_rule = t->ivdw_rule; o->el14 = t->el14_scale;
    o->crg = dup_d(t->crg, t->natom); o->iac = dup_i(t->iac, t->natom);
    o->excl = dup_u8(t->excl, t->natom); o->heavy = dup_u8(t->heavy, t->natom);
    o->avdw = dup_d(t->avdw, 3L * t->natyps); o->bvdw = dup_d(t->bvdw, 3L * t->natyps);
    o->ljcod = dup_u8(t->ljcod, (long)t->natyps * t->natyps);
    o->ncgp = t->ncgp; o->ncgp_solute = t->ncgp_solute;
    o->cfirst = dup_i(t->cgp_first, t->ncgp); o->clast = dup_i(t->cgp_last, t->ncgp);
    o->csw = dup_i(t->cgp_iswitch, t->ncgp);
    long ncgpatom = t->ncgp ? t->cgp_last[t->ncgp - 1] + 1 : 0;
    o->cgpatom = dup_i(t->cgpatom, ncgpatom);
    o->iwhich = (int*)calloc(t->natom, sizeof(int));
    for (int g = 0; g < o->ncgp; ++g)                 /* src/simprep.f90:3658-3667 */
        for (int a = o->cfirst[g]; a <= o->clast[g]; ++a) o->iwhich[o->cgpatom[a]] = g;
    o->nex = t->nexcl_pairs; o->exkeys = make_keys(t->excl_pairs, o->nex, o->natom);
    o->n14 = t->n14_pairs; o->k14 = make_keys(t->pairs14, o->n14, o->natom);
    o->nqat = t->nqat; o->S = t->nstates; o->nqlib = t->nqlib;
    o->qvdw_flag = t->qvdw_flag; o->qq_lib = t->qq_use_library_charges;
    o->iqseq = dup_i(t->iqseq, t->nqat);
    o->iqatom = (int*)calloc(t->natom, sizeof(int));
    for (int iq = 0; iq < o->nqat; ++iq) o->iqatom[o->iqseq[iq]] = iq + 1;
    o->qcrg = dup_d(t->qcrg, (long)o->nqat * o->S);
    o->qiac = dup_i(t->qiac, (long)o->nqat * o->S);
    o->qavdw = dup_d(t->qavdw, 3L * t->nqlib); o->qbvdw = dup_d(t->qbvdw, 3L * t->nqlib);
    o->sc = dup_d(t->sc_lookup, (long)o->nqat * (o->natyps + o->nqat) * o->S);
    long nqc = (long)o->S * o->nat_solute * o->nqat;
    o->qconn = (int8_t*)malloc(nqc ? nqc : 1);
    if (nqc) memcpy(o->qconn, t->qconn, nqc);
    o->nel = t->nel_scale; o->elp = dup_i(t->el_scale_pairs, 2L * o->nel);
    o->elv = dup_d(t->el_scale, (long)o->nel * o->S);
    o->nqexp = t->nqexpnb; o->qexp = dup_i(t->qexpnb_pairs, 2L * o->nqexp);
    for (int k = 0; k < 3; ++k) { o->xpcent[k] = t->xpcent[k]; o->xwcent[k] = t->xwcent[k]; }
    o->rexcl_o = t->rexcl_o;
    o->use_lrf = use_lrf;
    o->any_atom = t->iuse_switch_atom == 0;
    for (int s = 0; s < o->S; ++s) o->lambda[s] = 1.0;

    /* solvent parameters from the first solvent molecule, src/simprep.f90:3616-3621 */
    if (o->nwat > 0) {
        for (int a = 0; a < o->solv_atom; ++a) {
            int ia = o->nat_solute + a;
            o->chg_solv[a] = o->crg[ia];
            for (int k = 0; k < 3; ++k) { o->aLJ[a][k] = AV(o, o->iac[ia], k); o->bLJ[a][k] = BV(o, o->iac[ia], k); }
        }
        /* ww_int_comp, src/simprep.f90:3296-3317 */
        for (int a = 0; a < o->solv_atom; ++a)
            for (int b = 0; b < o->solv_atom; ++b) {
                int vdw = o->ljcod[o->iac[o->nat_solute + a] * o->natyps + o->iac[o->nat_solute + b]];
                o->ww_pre[a][b] = solv_values(o, o->aLJ[a][vdw - 1], o->aLJ[b][vdw - 1],
                                              o->bLJ[a][vdw - 1], o->bLJ[b][vdw - 1],
                                              o->chg_solv[a] * o->chg_solv[b]);
            }
        /* pw_int_comp, src/simprep.f90:3069-3108 (+ precompute_set_values_pw) */
        o->pw_pre = (pre_t*)calloc((size_t)(o->nat_solute ? o->nat_solute : 1) * o->solv_atom, sizeof(pre_t));
        for (int i = 0; i < o->nat_solute; ++i)
            for (int a = 0; a < o->solv_atom; ++a) {
                int vdw = o->ljcod[o->iac[i] * o->natyps + o->iac[o->nat_solute + a]];
                int k = vdw - 1;
                pre_t p = solv_values(o, AV(o, o->iac[i], k), o->aLJ[a][k], BV(o, o->iac[i], k),
                                      o->bLJ[a][k], o->crg[i] * o->chg_solv[a]);
                o->pw_pre[i * o->solv_atom + a] = p;
            }
    }
    /* qp_int_comp, src/simprep.f90:3112-3148, then the Q-bonded part of
       qq_int_comp, src/simprep.f90:3237-3267 */
    if (o->nqat > 0 && o->nat_solute > 0) {
        o->qp_pre = (pre_t*)calloc((size_t)o->nat_solute * o->nqat * o->S, sizeof(pre_t));
        for (int ig = 0; ig < o->nat_solute; ++ig) {
            if (any_qconn_le3(o, ig)) continue;
            for (int jq = 0; jq < o->nqat; ++jq) {
                int vdw = o->ljcod[o->iac[ig] * o->natyps + o->iac[o->iqseq[jq]]];
                for (int s = 0; s < o->S; ++s) {
                    if (QCONN(o, s, ig, jq) == 4) vdw = 3; /* sticky across states */
                    o->qp_pre[((long)ig * o->nqat + jq) * o->S + s] = qp_values(o, jq, ig, s, vdw);
                }
            }
        }
        for (int ja = 0; ja < o->nat_solute; ++ja) {
            if (o->iqatom[ja] != 0) continue;
            if (!any_qconn_le3(o, ja)) continue;
            for (int iq = 0; iq < o->nqat; ++iq) {
                int ia = o->iqseq[iq];
                for (int s = 0; s < o->S; ++s) {
                    int qc = QCONN(o, s, ja, iq);
                    if (qc >= 4) {
                        int vdw;
                        if (qc == 4) vdw = 3;
                        else if (o->qvdw_flag) vdw = 1;
                        else vdw = o->ljcod[o->iac[ia] * o->natyps + o->iac[ja]];
                        o->qp_pre[((long)ja * o->nqat + iq) * o->S + s] = qp_values(o, iq, ja, s, vdw);
                    }
                }
            }
        }
    }
    /* qw_int_comp, src/simprep.f90:3272-3292 (+ precompute_set_values_qw 3517-3558) */
    if (o->nqat > 0 && o->nwat > 0) {
        o->qw_pre = (pre_t*)calloc((size_t)o->nqat * o->solv_atom * o->S, sizeof(pre_t));
        for (int iq = 0; iq < o->nqat; ++iq)
            for (int a = 0; a < o->solv_atom; ++a) {
                int tw = o->iac[o->nat_solute + a];
                int vdw = o->ljcod[tw * o->natyps + o->iac[o->iqseq[iq]]];
                int qvdw = (vdw == 2) ? 1 : vdw;
                int i = o->iqseq[iq];
                for (int s = 0; s < o->S; ++s) {
                    pre_t p = {0};
                    double qa = o->qvdw_flag ? QAV(o, QIAC(o, iq, s), qvdw - 1) : AV(o, o->iac[i], vdw - 1);
                    double qb = o->qvdw_flag ? QBV(o, QIAC(o, iq, s), qvdw - 1) : BV(o, o->iac[i], vdw - 1);
                    combine(o->ivdw_rule, qa, o->aLJ[a][vdw - 1], qb, o->bLJ[a][vdw - 1], &p.A, &p.B);
                    p.el = o->qq_lib ? o->crg[i] * o->chg_solv[a] : QCRG(o, iq, s) * o->chg_solv[a];
                    p.sc = SCL(o, iq, tw, s);
                    p.set = 1;
                    o->qw_pre[((long)iq * o->solv_atom + a) * o->S + s] = p;
                }
            }
    }
    /* static Q lists: qq_int_comp (src/simprep.f90:3152-3236) + nbqqlist
       (src/nonbondene.f90:3231-3282) */
    o->nbqq = (vec_t*)calloc(o->S ? o->S : 1, sizeof(vec_t));
    o->nbqqp = (vec_t*)calloc(o->S ? o->S : 1, sizeof(vec_t));
    for (int s = 0; s < o->S; ++s) { o->nbqq[s].sz = sizeof(nbq_t); o->nbqqp[s].sz = sizeof(nbq_t); }
    for (int iq = 0; iq + 1 < o->nqat; ++iq) {
        int ia = o->iqseq[iq];
        for (int jq = iq + 1; jq < o->nqat; ++jq) {
            int ja = o->iqseq[jq];
            for (int s = 0; s < o->S; ++s) {
                int qc = QCONN(o, s, ja, iq);
                if (qc < 4) continue;
                double els = 1.0;
                for (int e = 0; e < o->nel; ++e) {
                    int k = o->elp[2 * e], l = o->elp[2 * e + 1];
                    if ((iq == k && jq == l) || (iq == l && jq == k)) { els = o->elv[e * o->S + s]; break; }
                }
                int vdw;
                if (qc == 4) vdw = 3;
                else if (!o->qvdw_flag) vdw = o->ljcod[o->iac[ia] * o->natyps + o->iac[ja]];
                else {
                    vdw = 1;
                    for (int e = 0; e < o->nqexp; ++e) {
                        int a = o->qexp[2 * e], b = o->qexp[2 * e + 1];
                        if ((iq == a && jq == b) || (jq == a && iq == b)) { vdw = 2; break; }
                    }
                }
                pre_t p = qq_values(o, iq, jq, s, vdw, els);
                if (!p.set) continue;
                nbq_t* e = (nbq_t*)vpush(&o->nbqq[s]);
                e->i = iq; e->j = jq; e->A = p.A; e->B = p.B; e->el = p.el; e->sc = p.sc; e->soft = p.soft;
            }
        }
    }
    for (int ja = 0; ja < o->nat_solute; ++ja) {
        if (o->iqatom[ja] != 0) continue;
        if (!any_qconn_le3(o, ja)) continue;
        for (int iq = 0; iq < o->nqat; ++iq)
            for (int s = 0; s < o->S; ++s) {
                pre_t p = o->qp_pre[((long)ja * o->nqat + iq) * o->S + s];
                if (!p.set) continue;
                nbq_t* e = (nbq_t*)vpush(&o->nbqqp[s]);
                e->i = iq; e->j = ja; e->A = p.A; e->B = p.B; e->el = p.el; e->sc = p.sc; e->soft = 0;
            }
    }
    o->nbpp.sz = sizeof(nb_t); o->nbpp14.sz = 1; o->nbpw.sz = sizeof(nb_t);
    o->nbww.sz = sizeof(nb_t); o->nbqp.sz = sizeof(nb_t); o->nbqw.sz = sizeof(nb_t);
    o->lrf = (double*)calloc((size_t)(o->ncgp ? o->ncgp : 1) * NLRF, sizeof(double));
    int nw = o->nwat ? o->nwat : 1;
    o->theta = (double*)calloc(nw, sizeof(double)); o->theta0 = (double*)calloc(nw, sizeof(double));
    o->tdum = (double*)calloc(nw, sizeof(double));
    o->list_sh = (int*)calloc((size_t)nw * 16, sizeof(int)); o->nsort = (int*)calloc((size_t)nw * 16, sizeof(int));
    return o;
}

void orc_destroy(orc* o) {
    if (!o) return;
    free(o->crg); free(o->iac); free(o->excl); free(o->heavy); free(o->avdw); free(o->bvdw);
    free(o->ljcod); free(o->cfirst); free(o->clast); free(o->csw); free(o->cgpatom); free(o->iwhich);
    free(o->si_i); free(o->si_j); free(o->si_A); free(o->si_B); free(o->si_el);
    free(o->exkeys); free(o->k14); free(o->iqseq); free(o->iqatom); free(o->qcrg); free(o->qiac);
    free(o->qavdw); free(o->qbvdw); free(o->sc); free(o->qconn); free(o->elp); free(o->elv); free(o->qexp);
    free(o->pw_pre); free(o->qp_pre); free(o->qw_pre);
    free(o->nbpp.p); free(o->nbpp14.p); free(o->nbpw.p); free(o->nbww.p); free(o->nbqp.p); free(o->nbqw.p);
    for (int s = 0; s < o->S; ++s) { free(o->nbqq[s].p); free(o->nbqqp[s].p); }
    free(o->nbqq); free(o->nbqqp); free(o->lrf);
    free(o->theta); free(o->theta0); free(o->tdum); free(o->list_sh); free(o->nsort);
    free(o);
}

void orc_set_lambda(orc* o, const double* lam) {
    for (int s = 0; s < o->S; ++s) o->lambda[s] = lam[s];
}

static inline v3 X(const double* x, int i) { v3 r = {x[3 * i], x[3 * i + 1], x[3 * i + 2]}; return r; }
/* q_dist4, src/math.f90:255-262 */
static inline double qdist4(v3 a, v3 b) { return vsq(vsub(b, a)); }
static inline double* LRF(orc* o, int g) { return o->lrf + (size_t)g * NLRF; }
/* LRF record: 0-2 cent, 3 phi0, 4-6 phi1, 7-15 phi2(3 vectors), 16-42 phi3(9 vectors) */

/* cgp_centers, src/nonbondene.f90:43-78 */
static void cgp_centers(orc* o, const double* x) {
    for (int g = 0; g < o->ncgp; ++g) {
        double* L = LRF(o, g);
        memset(L, 0, sizeof(double) * NLRF);
        v3 c = {0, 0, 0};
        for (int a = o->cfirst[g]; a <= o->clast[g]; ++a) c = vadd(c, X(x, o->cgpatom[a]));
        double n = (double)(o->clast[g] - o->cfirst[g] + 1);
        L[0] = c.x / n; L[1] = c.y / n; L[2] = c.z / n;
    }
}

/* lrf_update(group1, group2), src/nonbondene.f90:628-725 (sphere: shift 0) */
static void lrf_update(orc* o, const double* x, int g1, int g2) {
    double* L = LRF(o, g2);
    v3 cent = {L[0], L[1], L[2]};
    for (int ia = o->cfirst[g1]; ia <= o->clast[g1]; ++ia) {
        int i = o->cgpatom[ia];
        if (o->iqatom[i] != 0) continue;
        v3 dr = vsub(X(x, i), cent);
        double r2 = vsq(dr);
        double f0 = o->crg[i] / (r2 * sqrt(r2));
        double f1 = 3.0 * f0 / r2;
        double f2 = -f1 / r2;
        L[3] = L[3] + f0 * r2;
        L[4] = L[4] - dr.x * f0; L[5] = L[5] - dr.y * f0; L[6] = L[6] - dr.z * f0;
        v3 t1 = vscale(dr, f1);
        double tt[3] = {t1.x, t1.y, t1.z};
        for (int a = 0; a < 3; ++a) {
            L[7 + 3 * a + 0] = L[7 + 3 * a + 0] + dr.x * tt[a];
            L[7 + 3 * a + 1] = L[7 + 3 * a + 1] + dr.y * tt[a];
            L[7 + 3 * a + 2] = L[7 + 3 * a + 2] + dr.z * tt[a];
        }
        L[7 + 0] -= f0; L[7 + 4] -= f0; L[7 + 8] -= f0;
        double d[3] = {dr.x, dr.y, dr.z};
        for (int n = 0; n < 3; ++n)
            for (int j = 0; j < 3; ++j) {
                int m = j + 3 * n;            /* phi3(m), 0-based */
                double tk = d[n] * d[j];
                for (int c = 0; c < 3; ++c) {
                    double tl = tk * d[c];
                    tl = tl * 5.0;
                    tl = tl * f2;
                    L[16 + 3 * m + c] = L[16 + 3 * m + c] + tl;
                }
            }
        double u[3] = {dr.x * r2, dr.y * r2, dr.z * r2};
        double* P = L + 16; /* P[3*m + c] = phi3(m+1)%(x,y,z)[c] */
        P[0] -= f2 * (3.0 * u[0]); P[1] -= f2 * u[1]; P[2] -= f2 * u[2];     /* phi3(1) */
        P[3] -= f2 * u[1]; P[4] -= f2 * u[0];                               /* phi3(2) x,y */
        P[6] -= f2 * u[2];                                                  /* phi3(3) x */
        P[8] -= f2 * u[0];                                                  /* phi3(3) z */
        P[9] -= f2 * u[1]; P[10] -= f2 * u[0];                              /* phi3(4) x,y */
        P[12] -= f2 * u[0]; P[13] -= f2 * (3.0 * u[1]); P[14] -= f2 * u[2]; /* phi3(5) */
        P[16] -= f2 * u[2]; P[17] -= f2 * u[1];                             /* phi3(6) y,z */
        P[18] -= f2 * u[2];                                                 /* phi3(7) x */
        P[20] -= f2 * u[0];                                                 /* phi3(7) z */
        P[22] -= f2 * u[2]; P[23] -= f2 * u[1];                             /* phi3(8) y,z */
        P[24] -= f2 * u[0]; P[25] -= f2 * u[1]; P[26] -= f2 * (3.0 * u[2]); /* phi3(9) */
    }
}

static inline int parity_skip(int a, int b) {
    return (a > b && ((a + b) % 2) == 0) || (a < b && ((a + b) % 2) == 1);
}

/* Group-pair cut-off test.  Switch-atom mode (nbpplist_lrf,
   src/nonbondene.f90:1861): r2 of the two switch atoms.  Any-atom mode
   (nbpplis2_lrf, src/nonbondene.f90:1451-1468): inside as soon as one atom
   pair (all atoms, Q and excluded ones too) is within the cut-off; r2 is then
   the last pair examined, which for an outside pair is (last atom of ig, last
   atom of jg) -- the value the reference's LRF test reads. */
static int pp_inside(const orc* o, const double* x, int ig, int jg, double rcut2, double* r2) {
    if (!o->any_atom) {
        *r2 = qdist4(X(x, o->csw[ig]), X(x, o->csw[jg]));
        return *r2 <= rcut2;
    }
    *r2 = 1.0;
    for (int ia = o->cfirst[ig]; ia <= o->clast[ig]; ++ia)
        for (int jb = o->cfirst[jg]; jb <= o->clast[jg]; ++jb) {
            *r2 = qdist4(X(x, o->cgpatom[ia]), X(x, o->cgpatom[jb]));
            if (*r2 <= rcut2) return 1;
        }
    return 0;
}

/* Solute group to water (first atom ja) test: switch atom (nbpwlist_lrf,
   src/nonbondene.f90:2915) or any atom of the group (nbpwlis2_lrf,
   src/nonbondene.f90:2565-2577, r2 of the last atom when outside). */
static int pw_inside(const orc* o, const double* x, int ig, int ja, double rcut2, double* r2) {
    if (!o->any_atom) {
        *r2 = qdist4(X(x, o->csw[ig]), X(x, ja));
        return *r2 <= rcut2;
    }
    *r2 = 1.0;
    for (int ia = o->cfirst[ig]; ia <= o->clast[ig]; ++ia) {
        *r2 = qdist4(X(x, o->cgpatom[ia]), X(x, ja));
        if (*r2 <= rcut2) return 1;
    }
    return 0;
}

/* nbpplist(_lrf), src/nonbondene.f90:1520-1639, 1777-1908; nbpplis2(_lrf) 950-1086, 1369-1516 */
static void nbpplist(orc* o, const double* x, double rcut2, double rlrf2) {
    o->nbpp.n = 0; o->nbpp14.n = 0;
    for (int ig = 0; ig < o->ncgp_solute; ++ig) {
        int is = o->csw[ig];
        if (o->excl[is]) continue;
        for (int jg = 0; jg < o->ncgp_solute; ++jg) {
            if (parity_skip(ig, jg)) continue;
            int ja = o->csw[jg];
            if (o->excl[ja]) continue;
            double r2;
            if (pp_inside(o, x, ig, jg, rcut2, &r2)) {
                for (int ia = o->cfirst[ig]; ia <= o->clast[ig]; ++ia) {
                    int i = o->cgpatom[ia];
                    if (o->iqatom[i] != 0) continue;
                    for (int jb = o->cfirst[jg]; jb <= o->clast[jg]; ++jb) {
                        int j = o->cgpatom[jb];
                        if (o->iqatom[j] != 0) continue;
                        if (ig == jg && i >= j) continue;
                        int code = pp_code(o, i, j);
                        if (code == 0) continue;
                        pre_t p = pp_values(o, i, j, code);
                        if (!p.set) continue;
                        nb_t* e = (nb_t*)vpush(&o->nbpp);
                        e->i = i; e->j = j; e->A = p.A; e->B = p.B; e->el = p.el;
                        *(char*)vpush(&o->nbpp14) = (code == 3);
                    }
                }
            } else if (o->use_lrf && r2 <= rlrf2) {
                lrf_update(o, x, ig, jg);
                lrf_update(o, x, jg, ig);
            }
        }
    }
}

/* nbpwlist(_lrf), src/nonbondene.f90:2622-2725, 2842-2955; nbpwlis2(_lrf) 2137-2242, 2493-2618 */
static void nbpwlist(orc* o, const double* x, double rcut2, double rlrf2) {
    o->nbpw.n = 0;
    for (int ig = 0; ig < o->ncgp_solute; ++ig) {
        int is = o->csw[ig];
        if (o->excl[is]) continue;
        for (int jw = 0; jw < o->nwat; ++jw) {
            int ja = o->nat_solute + o->solv_atom * jw;
            int jg = o->iwhich[ja];
            if (o->excl[ja]) continue;
            double r2;
            if (pw_inside(o, x, ig, ja, rcut2, &r2)) {
                for (int ia = o->cfirst[ig]; ia <= o->clast[ig]; ++ia) {
                    int i = o->cgpatom[ia];
                    if (o->iqatom[i] != 0) continue;
                    for (int a = 0; a < o->solv_atom; ++a) {
                        nb_t* e = (nb_t*)vpush(&o->nbpw);
                        pre_t p = o->pw_pre[i * o->solv_atom + a];
                        e->i = i; e->j = ja + a; e->A = p.A; e->B = p.B; e->el = p.el;
                    }
                }
            } else if (o->use_lrf && r2 <= rlrf2) {
                lrf_update(o, x, ig, jg);
                lrf_update(o, x, jg, ig);
            }
        }
    }
}

/* nbwwlist(_lrf), src/nonbondene.f90:4079-4172, 4274-4395 */
static void nbwwlist(orc* o, const double* x, double rcut2, double rlrf2) {
    o->nbww.n = 0;
    int sa = o->solv_atom;
    for (int iw = 0; iw < o->nwat; ++iw) {
        int is = o->nat_solute + sa * iw;
        if (o->excl[is]) continue;
        int ig = o->iwhich[is];
        for (int jw = 0; jw < o->nwat; ++jw) {
            int ja = o->nat_solute + sa * jw;
            if (o->excl[ja]) continue;
            int jg = o->iwhich[ja];
            /* parity rule on 1-based indices == parity on 0-based (shift by 2) */
            if (parity_skip(iw, jw) || iw == jw) continue;
            double r2 = qdist4(X(x, is), X(x, ja));
            if (r2 <= rcut2) {
                for (int la = 0; la < sa; ++la)
                    for (int ka = 0; ka < sa; ++ka) {
                        nb_t* e = (nb_t*)vpush(&o->nbww);
                        e->i = is + la; e->j = ja + ka;
                        e->A = o->ww_pre[la][ka].A; e->B = o->ww_pre[la][ka].B; e->el = o->ww_pre[la][ka].el;
                    }
            } else if (o->use_lrf && r2 <= rlrf2) {
                lrf_update(o, x, ig, jg);
                lrf_update(o, x, jg, ig);
            }
        }
    }
}

/* nbqplist, src/nonbondene.f90:3647-3742; nbqplis2 3408-3519 */
static void nbqplist(orc* o, const double* x, double rcq2) {
    if (o->qp_done && rcq2 > o->rexcl_o * o->rexcl_o) return;
    if (o->nqat == 0) return;
    o->nbqp.n = 0;
    v3 xp = {o->xpcent[0], o->xpcent[1], o->xpcent[2]};
    for (int ig = 0; ig < o->ncgp_solute; ++ig) {
        int ia = o->csw[ig];
        if (o->excl[ia]) continue;
        int inside = 0;
        if (o->any_atom) {   /* nbqplis2, src/nonbondene.f90:3477-3487 */
            for (int a = o->cfirst[ig]; a <= o->clast[ig] && !inside; ++a)
                inside = qdist4(X(x, o->cgpatom[a]), xp) <= rcq2;
        } else {
            inside = qdist4(X(x, ia), xp) <= rcq2;
        }
        if (!inside) continue;
        for (int a = o->cfirst[ig]; a <= o->clast[ig]; ++a) {
            int i = o->cgpatom[a];
            if (any_qconn_le3(o, i)) continue;
            for (int iq = 0; iq < o->nqat; ++iq) {
                nb_t* e = (nb_t*)vpush(&o->nbqp);
                e->i = iq; e->j = i;
            }
        }
    }
    o->qp_done = 1;
}

/* nbqwlist, src/nonbondene.f90:3862-3944 */
static void nbqwlist(orc* o, const double* x, double rcq2) {
    if (o->qw_done && rcq2 > o->rexcl_o * o->rexcl_o) return;
    if (o->nqat == 0) return;
    o->nbqw.n = 0;
    v3 xp = {o->xpcent[0], o->xpcent[1], o->xpcent[2]};
    for (int iw = 0; iw < o->nwat; ++iw) {
        int ia = o->nat_solute + o->solv_atom * iw;
        if (o->excl[ia]) continue;
        double r2 = qdist4(X(x, ia), xp);
        if (r2 <= rcq2)
            for (int iq = 0; iq < o->nqat; ++iq)
                for (int a = 0; a < o->solv_atom; ++a) {
                    nb_t* e = (nb_t*)vpush(&o->nbqw);
                    e->i = iq; e->j = ia + a;
                }
    }
    o->qw_done = 1;
}

/* make_pair_lists, spherical branch, src/nonbondene.f90:749-837 */
int orc_make_pair_lists(orc* o, const double* x, double Rq, double Rcq2, double RcLRF2,
                        double Rcpp2, double Rcpw2, double Rcww2) {
    (void)Rq;
    if (o->use_lrf) cgp_centers(o, x);
    nbpplist(o, x, Rcpp2, RcLRF2);
    nbpwlist(o, x, Rcpw2, RcLRF2);
    nbqplist(o, x, Rcq2);
    nbwwlist(o, x, Rcww2, RcLRF2);
    nbqwlist(o, x, Rcq2);
    return 0;
}

/* ---- pair kernels, src/nonbonded.f90 --------------------------------------- */
typedef struct { double Vel, Va, Vb, dv; v3 vec; } eret;

/* nbe, src/nonbonded.f90:45-75 (with q_dist2, src/math.f90:226-238) */
static eret nbe(const double* x, int i, int j, double A, double B, double el) {
    eret r;
    v3 t = vsub(X(x, j), X(x, i));
    double r2 = 1.0 / vsq(t);
    double rr = sqrt(r2);
    double r6 = r2 * r2 * r2;
    double r12 = r6 * r6;
    r.Vel = el * rr;
    r.Va = A * r12;
    r.Vb = B * r6;
    r.dv = r2 * (-r.Vel - 12.0 * r.Va + 6.0 * r.Vb);
    r.vec = t;
    return r;
}
/* nonbond_solvent_internal, src/nonbondene.f90:6082-6154: the listed pairs
   inside every solvent molecule (q_dist2), with the reference's grouping of
   dv = r2*(-Vel) + r2*(-12 Va + 6 Vb) */
static void nonbond_solvent_internal(const orc* o, const double* x, double* d, double* el, double* vdw) {
    for (int iw = 0; iw < o->nwat; ++iw) {
        int is = o->nat_solute + o->solv_atom * iw;
        for (int ip = 0; ip < o->nsi; ++ip) {
            int ia = is + o->si_i[ip], ib = is + o->si_j[ip];
            v3 t = vsub(X(x, ib), X(x, ia));
            double r2 = 1.0 / vsq(t);
            double r = sqrt(r2);
            double r6 = r2 * r2 * r2;
            double r12 = r6 * r6;
            double Vel = o->si_el[ip] * r, Va = o->si_A[ip] * r12, Vb = o->si_B[ip] * r6;
            double dv = r2 * (-Vel) + r2 * (-12.0 * Va + 6.0 * Vb);
            *el += Vel;
            *vdw += Va - Vb;
            d[3 * ia] -= t.x * dv; d[3 * ia + 1] -= t.y * dv; d[3 * ia + 2] -= t.z * dv;
            d[3 * ib] += t.x * dv; d[3 * ib + 1] += t.y * dv; d[3 * ib + 2] += t.z * dv;
        }
    }
}

void orc_set_solvent_internal(orc* o, int n, const int32_t* ij, const double* A, const double* B,
                              const double* el) {
    free(o->si_i); free(o->si_j); free(o->si_A); free(o->si_B); free(o->si_el);
    o->nsi = n;
    o->si_i = (int*)calloc(n ? n : 1, sizeof(int)); o->si_j = (int*)calloc(n ? n : 1, sizeof(int));
    o->si_A = dup_d(A, n); o->si_B = dup_d(B, n); o->si_el = dup_d(el, n);
    for (int k = 0; k < n; ++k) { o->si_i[k] = ij[2 * k]; o->si_j[k] = ij[2 * k + 1]; }
}

/* nbe_spc, src/nonbonded.f90:247-267 (q_dist, src/math.f90:214-224) */
static eret nbe_spc(const double* x, int i, int j, double el) {
    eret r;
    v3 t = vsub(X(x, j), X(x, i));
    double r2 = 1.0 / vsq(t);
    double rr = sqrt(r2);
    r.vec = t;
    r.Vel = el * rr;
    r.dv = r2 * (-r.Vel);
    r.Va = r.Vb = 0.0;
    return r;
}
typedef struct { double r2, r, r6; v3 vec; } dist3;
/* q_dist3, src/math.f90:240-253 */
static dist3 qdist3(const double* x, int i, int j) {
    dist3 d;
    d.vec = vsub(X(x, j), X(x, i));
    d.r2 = 1.0 / vsq(d.vec);
    d.r = sqrt(d.r2);
    d.r6 = d.r2 * d.r2 * d.r2;
    return d;
}
/* nbe_qx, src/nonbonded.f90:200-222 */
static eret nbe_qx(double A, double B, double el, double sc, double lambda, dist3 d) {
    eret r;
    double r6_hc = 1.0 / d.r6;
    double r6 = r6_hc + sc;
    r6 = 1.0 / r6;
    double r12 = r6 * r6;
    r.Vel = el * d.r;
    r.Va = A * r12;
    r.Vb = B * r6;
    r.dv = d.r2 * (-r.Vel - (12.0 * r.Va - 6.0 * r.Vb) * r6 * r6_hc) * lambda;
    r.vec = d.vec;
    return r;
}
/* nbe_qspc, src/nonbonded.f90:226-243 */
static eret nbe_qspc(double el, double lambda, double r2, double rr) {
    eret r;
    r.Vel = el * rr;
    r.dv = -r2 * r.Vel * lambda;
    r.Va = r.Vb = 0.0;
    return r;
}
/* nbe_qq, src/nonbonded.f90:111-150 */
static eret nbe_qq(const orc* o, const double* x, const nbq_t* nb, double lambda) {
    eret r;
    dist3 d = qdist3(x, o->iqseq[nb->i], o->iqseq[nb->j]);
    double r6_hc = 1.0 / d.r6;
    double rr = d.r;
    double r6 = r6_hc + nb->sc;
    r6 = 1.0 / r6;
    double r12 = r6 * r6;
    r.Vel = nb->el * rr;
    r.vec = d.vec;
    if (nb->soft) {
        r.Vb = 0.0;
        r.Va = nb->A * exp(-nb->B / rr);
        r.dv = d.r2 * (-r.Vel - nb->B * r.Va / rr) * lambda;
    } else {
        r.Va = nb->A * r12;
        r.Vb = nb->B * r6;
        r.dv = d.r2 * (-r.Vel - (12.0 * r.Va - 6.0 * r.Vb) * r6 * r6_hc) * lambda;
    }
    return r;
}

static inline void dsub(double* d, int i, v3 v, double dv) {
    d[3 * i] = d[3 * i] - v.x * dv; d[3 * i + 1] = d[3 * i + 1] - v.y * dv; d[3 * i + 2] = d[3 * i + 2] - v.z * dv;
}
static inline void dadd(double* d, int i, v3 v, double dv) {
    d[3 * i] = d[3 * i] + v.x * dv; d[3 * i + 1] = d[3 * i + 1] + v.y * dv; d[3 * i + 2] = d[3 * i + 2] + v.z * dv;
}

/* nonbond_pp / nonbond_pw / nonbond_ww, src/nonbondene.f90:4694-4760, 4856-4916, 5509-5573 */
static void nonbond_list(const vec_t* L, const double* x, double* d, double* el, double* vdw) {
    const nb_t* e = (const nb_t*)L->p;
    for (long p = 0; p < L->n; ++p) {
        eret r = nbe(x, e[p].i, e[p].j, e[p].A, e[p].B, e[p].el);
        dsub(d, e[p].i, r.vec, r.dv);
        dadd(d, e[p].j, r.vec, r.dv);
        *el = *el + r.Vel;
        *vdw = *vdw + r.Va - r.Vb;
    }
}

/* nonbond_ww_spc, src/nonbondene.f90:5886-5975 */
static void nonbond_ww_spc(const orc* o, const double* x, double* d, double* el, double* vdw) {
    const nb_t* e = (const nb_t*)o->nbww.p;
    int blk = o->solv_atom * o->solv_atom;
    for (long iw = 0; iw < o->nbww.n; iw += blk) {
        eret r = nbe(x, e[iw].i, e[iw].j, e[iw].A, e[iw].B, e[iw].el);
        *vdw = *vdw + r.Va - r.Vb;
        *el = *el + r.Vel;
        dsub(d, e[iw].i, r.vec, r.dv);
        dadd(d, e[iw].j, r.vec, r.dv);
        for (int jw = 1; jw < blk; ++jw) {
            const nb_t* q = &e[iw + jw];
            eret s = nbe_spc(x, q->i, q->j, q->el);
            *el = *el + s.Vel;
            dsub(d, q->i, s.vec, s.dv);
            dadd(d, q->j, s.vec, s.dv);
        }
    }
}

/* nonbond_qp, src/nonbondene.f90:5157-5230 */
static void nonbond_qp(const orc* o, const double* x, double* d, qnb_qenergies* EQ) {
    const nb_t* e = (const nb_t*)o->nbqp.p;
    for (long ip = 0; ip < o->nbqp.n; ++ip) {
        int iq = e[ip].i, i = o->iqseq[iq], j = e[ip].j;
        dist3 ds = qdist3(x, i, j);
        for (int s = 0; s < o->S; ++s) {
            pre_t p = o->qp_pre[((long)j * o->nqat + iq) * o->S + s];
            eret r = nbe_qx(p.A, p.B, p.el, p.sc, o->lambda[s], ds);
            dsub(d, i, ds.vec, r.dv);
            dadd(d, j, ds.vec, r.dv);
            EQ[s].qp_el = EQ[s].qp_el + r.Vel;
            EQ[s].qp_vdw = EQ[s].qp_vdw + r.Va - r.Vb;
        }
    }
}

/* nonbond_qw_spc, src/nonbondene.f90:5658-5767 */
static void nonbond_qw_spc(const orc* o, const double* x, double* d, qnb_qenergies* EQ) {
    const nb_t* e = (const nb_t*)o->nbqw.p;
    int sa = o->solv_atom;
    for (long iw = 0; iw < o->nbqw.n; iw += sa) {
        int iq = e[iw].i, i = o->iqseq[iq], j = e[iw].j;
        dist3 ds = qdist3(x, i, j);
        double dv = 0.0;
        for (int s = 0; s < o->S; ++s) {
            pre_t p = o->qw_pre[((long)iq * sa + 0) * o->S + s];
            eret r = nbe_qx(p.A, p.B, p.el, p.sc, o->lambda[s], ds);
            dv = dv + r.dv;
            EQ[s].qw_el = EQ[s].qw_el + r.Vel;
            EQ[s].qw_vdw = EQ[s].qw_vdw + r.Va - r.Vb;
        }
        dsub(d, i, ds.vec, dv);
        dadd(d, j, ds.vec, dv);
        for (int ip = 1; ip < sa; ++ip) {
            int ja = j + ip;
            v3 t = vsub(X(x, ja), X(x, i));
            double r2 = 1.0 / vsq(t), rr = sqrt(r2);
            dv = 0.0;
            for (int s = 0; s < o->S; ++s) {
                pre_t p = o->qw_pre[((long)iq * sa + ip) * o->S + s];
                eret r = nbe_qspc(p.el, o->lambda[s], r2, rr);
                EQ[s].qw_el = EQ[s].qw_el + r.Vel;
                dv = dv + r.dv;
            }
            dsub(d, i, t, dv);
            dadd(d, ja, t, dv);
        }
    }
}

/* nonbond_qw (general solvent), src/nonbondene.f90:5339-5418 */
static void nonbond_qw(const orc* o, const double* x, double* d, qnb_qenergies* EQ) {
    const nb_t* e = (const nb_t*)o->nbqw.p;
    int sa = o->solv_atom;
    for (long iw = 0; iw < o->nbqw.n; iw += sa) {
        int iq = e[iw].i, i = o->iqseq[iq];
        for (int jw = 0; jw < sa; ++jw) {
            int j = e[iw + jw].j;
            dist3 ds = qdist3(x, i, j);
            for (int s = 0; s < o->S; ++s) {
                pre_t p = o->qw_pre[((long)iq * sa + jw) * o->S + s];
                eret r = nbe_qx(p.A, p.B, p.el, p.sc, o->lambda[s], ds);
                dsub(d, i, ds.vec, r.dv);
                dadd(d, j, ds.vec, r.dv);
                EQ[s].qw_el = EQ[s].qw_el + r.Vel;
                EQ[s].qw_vdw = EQ[s].qw_vdw + r.Va - r.Vb;
            }
        }
    }
}

/* lrf_taylor, src/nonbondene.f90:507-571 */
static void lrf_taylor(orc* o, const double* x, double* d, double* elrf) {
    for (int i = 0; i < o->natom; ++i) {
        if (o->excl[i] || o->iqatom[i] != 0) continue;
        int ic = o->iwhich[i];
        double* L = LRF(o, ic);
        v3 c = {L[0], L[1], L[2]};
        v3 dr = vsub(c, X(x, i));
        v3 p1 = {L[4], L[5], L[6]};
        v3 p2[3], p3[9];
        for (int a = 0; a < 3; ++a) { p2[a].x = L[7 + 3 * a]; p2[a].y = L[8 + 3 * a]; p2[a].z = L[9 + 3 * a]; }
        for (int m = 0; m < 9; ++m) { p3[m].x = L[16 + 3 * m]; p3[m].y = L[17 + 3 * m]; p3[m].z = L[18 + 3 * m]; }
        v3 tmp = {vdot(dr, p2[0]), vdot(dr, p2[1]), vdot(dr, p2[2])};
        double Vij = L[3] + vdot(dr, p1) + 0.5 * vdot(dr, tmp);
        *elrf = *elrf + 0.5 * o->crg[i] * Vij;
        v3 df;
        tmp.x = vdot(dr, p3[0]); tmp.y = vdot(dr, p3[1]); tmp.z = vdot(dr, p3[2]);
        df.x = p1.x + vdot(dr, p2[0]) + 0.5 * vdot(dr, tmp);
        tmp.x = vdot(dr, p3[3]); tmp.y = vdot(dr, p3[4]); tmp.z = vdot(dr, p3[5]);
        df.y = p1.y + vdot(dr, p2[1]) + 0.5 * vdot(dr, tmp);
        tmp.x = vdot(dr, p3[6]); tmp.y = vdot(dr, p3[7]); tmp.z = vdot(dr, p3[8]);
        df.z = p1.z + vdot(dr, p2[2]) + 0.5 * vdot(dr, tmp);
        d[3 * i] = d[3 * i] - df.x * o->crg[i];
        d[3 * i + 1] = d[3 * i + 1] - df.y * o->crg[i];
        d[3 * i + 2] = d[3 * i + 2] - df.z * o->crg[i];
    }
}

/* pot_energy_nonbonds, spherical branch, src/potene.f90:320-380 */
int orc_pot_energy_nonbonds(orc* o, const double* x, double* d, qnb_energies* E, qnb_qenergies* EQ, int md) {
    if (o->natom > o->nat_solute) {
        if (o->ivdw_rule == 1 && o->solvent_type == 0) {
            if (md) nonbond_ww_spc(o, x, d, &E->ww_el, &E->ww_vdw);
            nonbond_qw_spc(o, x, d, EQ);
        } else {
            nonbond_qw(o, x, d, EQ);
            if (md) nonbond_list(&o->nbww, x, d, &E->ww_el, &E->ww_vdw);
        }
        /* src/potene.f90:361-366: only when the solvent has torsions */
        if (md && o->nsi > 0) nonbond_solvent_internal(o, x, d, &E->ww_el, &E->ww_vdw);
        if (md) nonbond_list(&o->nbpw, x, d, &E->pw_el, &E->pw_vdw);
    }
    if (md) nonbond_list(&o->nbpp, x, d, &E->pp_el, &E->pp_vdw);
    nonbond_qp(o, x, d, EQ);
    if (o->use_lrf && md) lrf_taylor(o, x, d, &E->lrf);
    return 0;
}

/* nonbond_qq + nonbond_qqp, src/nonbondene.f90:5013-5153 */
int orc_nonbond_qq(orc* o, const double* x, double* d, qnb_qenergies* EQ) {
    for (int s = 0; s < o->S; ++s) {
        const nbq_t* e = (const nbq_t*)o->nbqq[s].p;
        for (long p = 0; p < o->nbqq[s].n; ++p) {
            int i = o->iqseq[e[p].i], j = o->iqseq[e[p].j];
            eret r = nbe_qq(o, x, &e[p], o->lambda[s]);
            dsub(d, i, r.vec, r.dv);
            dadd(d, j, r.vec, r.dv);
            EQ[s].qq_el = EQ[s].qq_el + r.Vel;
            EQ[s].qq_vdw = EQ[s].qq_vdw + r.Va - r.Vb;
        }
    }
    for (int s = 0; s < o->S; ++s) {
        const nbq_t* e = (const nbq_t*)o->nbqqp[s].p;
        for (long p = 0; p < o->nbqqp[s].n; ++p) {
            int i = o->iqseq[e[p].i], j = e[p].j;
            dist3 ds = qdist3(x, i, j);
            eret r = nbe_qx(e[p].A, e[p].B, e[p].el, e[p].sc, o->lambda[s], ds);
            dsub(d, i, ds.vec, r.dv);
            dadd(d, j, ds.vec, r.dv);
            EQ[s].qp_el = EQ[s].qp_el + r.Vel;
            EQ[s].qp_vdw = EQ[s].qp_vdw + r.Va - r.Vb;
        }
    }
    return 0;
}

/* ---- solvent boundary ------------------------------------------------------ */
void orc_set_solvent_params(orc* o, const qnb_solvent_params* p) {
    o->sp = *p;
    o->have_sp = 1;
    for (int s = 0; s < 16; ++s) { o->theta_corr[s] = p->theta_corr[s]; o->avtheta[s] = 0; o->avn_insh[s] = 0; }
}

/* restrain_solvent, src/nonbondene.f90:6466-6544 */
int orc_restrain_solvent(orc* o, const double* x, double* d, double Tfree, double* Erad) {
    const qnb_solvent_params* p = &o->sp;
    double shift = (p->fk_wsphere != 0.0) ? sqrt(p->boltz * Tfree / p->fk_wsphere) : 0.0;
    v3 wc = {o->xwcent[0], o->xwcent[1], o->xwcent[2]};
    for (int iw = o->ncgp_solute; iw < o->ncgp; ++iw) {
        int i0 = o->csw[iw];
        if (o->excl[i0]) continue;
        int jsolv = iw - o->ncgp_solute;
        for (int isolv = 0; isolv < o->solv_atom; ++isolv) {
            int i, ifirst;
            if (o->solv_atom == 3) {
                if (isolv > 0) break;
                i = ifirst = i0;
            } else {
                /* the distance is that of the molecule's first atom; the
                   force goes to heavy atom isolv (src/nonbondene.f90:6513-6537) */
                if (!o->heavy[o->nat_solute + isolv]) continue;
                ifirst = o->nat_solute + o->solv_atom * jsolv;
                i = ifirst + isolv;
            }
            v3 vec = vsub(X(x, ifirst), wc);   /* q_dist5(xwcent, x): x - xwcent */
            double b = sqrt(vsq(vec));
            double db = b - (p->rwat - shift);
            double erst, dv;
            if (db > 0.0) {
                erst = 0.5 * p->fk_wsphere * (db * db) - p->Dwmz;
                dv = p->fk_wsphere * db / b;
            } else if (b > 0.0) {
                double fexp = exp(p->awmz * db);
                erst = p->Dwmz * (fexp * fexp - 2.0 * fexp);
                dv = -2.0 * p->Dwmz * p->awmz * (fexp - fexp * fexp) / b;
            } else {
                dv = 0.0;
                erst = 0.0;
            }
            dadd(d, i, vec, dv);
            *Erad = *Erad + erst;
        }
    }
    return 0;
}

/* watpol, src/nonbondene.f90:6548-6746 (solv_atom == 3 branch and general) */
int orc_watpol(orc* o, const double* x, double* d, int istep, int md, double* Epol) {
    const qnb_solvent_params* p = &o->sp;
    int nsh = p->nwpolr_shell, sa = o->solv_atom;
    v3 wc = {o->xwcent[0], o->xwcent[1], o->xwcent[2]};
    const double pi = 4.0 * atan(1.0);
    int nw = o->nwat;
    if (md) {
        for (int s = 0; s < nsh; ++s) o->n_insh[s] = 0;
        for (int iw = 0; iw < nw; ++iw) {
            o->theta[iw] = 0.0;
            o->theta0[iw] = 0.0;
            int i = o->nat_solute + sa * iw;
            if (o->excl[i]) continue;
            v3 rmu = {0, 0, 0}, rmc = {0, 0, 0}, rcu;
            if (sa == 3) {
                for (int k = 1; k < sa; ++k) rmu = vadd(rmu, X(x, i + k));
                rmu = vsub(rmu, vscale(X(x, i), 2.0));
            } else {
                for (int k = 0; k < sa; ++k) {
                    rmc = vadd(rmc, X(x, i + k));
                    rmu = vadd(rmu, vscale(X(x, i + k), o->chg_solv[k]));
                }
                rmc = vscale(rmc, 1.0 / (double)sa);
            }
            double rm = sqrt(vsq(rmu));
            rmu = vscale(rmu, 1.0 / rm);
            rcu = (sa == 3) ? vsub(X(x, i), wc) : vsub(rmc, wc);
            double rc = sqrt(vsq(rcu));
            rcu = vscale(rcu, 1.0 / rc);
            double scp = vdot(rmu, rcu);
            if (scp > 1.0) scp = 1.0;
            if (scp < -1.0) scp = -1.0;
            o->theta[iw] = acos(scp);
            o->tdum[iw] = o->theta[iw];
            if (rc > p->shell_rout[nsh - 1] - p->shell_dr[nsh - 1]) {
                int is;
                for (is = nsh - 1; is >= 1; --is)
                    if (rc <= p->shell_rout[is]) break;
                if (is < 0) is = 0;
                o->list_sh[(long)is * nw + o->n_insh[is]] = iw;
                o->n_insh[is]++;
            }
        }
        /* per-shell selection sort by theta; earliest list entry wins ties */
        int jmin = 0;
        for (int is = 0; is < nsh; ++is) {
            int imin = 0;
            for (int il = 0; il < o->n_insh[is]; ++il) {
                double tmin = 2.0 * pi;
                for (int jl = 0; jl < o->n_insh[is]; ++jl) {
                    int jw = o->list_sh[(long)is * nw + jl];
                    if (o->tdum[jw] < tmin) { jmin = jw; tmin = o->theta[jw]; }
                }
                o->nsort[(long)is * nw + imin] = jmin;
                imin++;
                o->tdum[jmin] = 99999.0;
            }
        }
    }
    if (istep > 0 && (istep % (int)llround(p->itdis)) == 0 && md) {
        for (int is = 0; is < nsh; ++is) {
            o->avtheta[is] = o->avtheta[is] / p->itdis;
            o->avn_insh[is] = o->avn_insh[is] / p->itdis;
            o->theta_corr[is] = o->theta_corr[is] + o->avtheta[is] - acos(p->shell_cstb[is]);
            o->avtheta[is] = 0.0;
            o->avn_insh[is] = 0.0;
        }
    }
    for (int is = 0; is < nsh; ++is) {
        int n = o->n_insh[is];
        if (n == 0) continue;
        double avtdum = 0.0;
        for (int il = 0; il < n; ++il) {
            int iw = o->nsort[(long)is * nw + il];
            double arg = 1.0 + (1.0 - 2.0 * (double)(il + 1)) / (double)n;
            double t0 = acos(arg);
            t0 = t0 - 3.0 * sin(t0) * p->shell_cstb[is] / 2.0;
            if (t0 < 0.0) t0 = 0.0;
            if (t0 > pi) t0 = pi;
            o->theta0[il] = t0;
            avtdum = avtdum + o->theta[iw];
            double dtheta = o->theta[iw] - t0 + o->theta_corr[is];
            *Epol = *Epol + 0.5 * p->fkwpol * dtheta * dtheta;
            double dv = p->fkwpol * dtheta;
            int i = o->nat_solute + sa * iw;
            v3 rmu = {0, 0, 0}, rmc = {0, 0, 0}, rcu;
            if (sa == 3) {
                for (int k = 1; k < sa; ++k) rmu = vadd(rmu, X(x, i + k));
                rmu = vsub(rmu, vscale(X(x, i), 2.0));
            } else {
                for (int k = 0; k < sa; ++k) {
                    rmc = vadd(rmc, X(x, i + k));
                    rmu = vadd(rmu, vscale(X(x, i + k), o->chg_solv[k]));
                }
                rmc = vscale(rmc, 1.0 / (double)sa);
            }
            double rm = sqrt(vsq(rmu));
            rmu = vscale(rmu, 1.0 / rm);
            rcu = (sa == 3) ? vsub(X(x, i), wc) : vsub(rmc, wc);
            double rc = sqrt(vsq(rcu));
            rcu = vscale(rcu, 1.0 / rc);
            double scp = vdot(rmu, rcu);
            if (scp > 1.0) scp = 1.0;
            if (scp < -1.0) scp = -1.0;
            double f0 = sin(acos(scp));
            if (fabs(f0) < QREAL_EPS) f0 = QREAL_EPS;
            f0 = -1.0 / f0;
            f0 = dv * f0;
            v3 f1 = vscale(vscale(vsub(rcu, vscale(rmu, scp)), -2.0), 1.0 / rm);
            v3 f3 = vscale(vsub(rcu, vscale(rmu, scp)), 1.0 / rm);
            v3 f2 = vscale(vsub(rmu, vscale(rcu, scp)), 1.0 / rc);
            v3 fi = vscale(vadd(f1, f2), f0);
            d[3 * i] += fi.x; d[3 * i + 1] += fi.y; d[3 * i + 2] += fi.z;
            for (int k = 1; k < sa; ++k) {
                v3 fk = vscale(f3, f0);
                d[3 * (i + k)] += fk.x; d[3 * (i + k) + 1] += fk.y; d[3 * (i + k) + 2] += fk.z;
            }
        }
        if (md) {
            o->avtheta[is] = o->avtheta[is] + avtdum / (double)n;
            o->avn_insh[is] = o->avn_insh[is] + n;
        }
    }
    return 0;
}

void orc_get_watpol_state(const orc* o, double* theta_corr, double* avtheta, double* avn) {
    for (int s = 0; s < 16; ++s) { theta_corr[s] = o->theta_corr[s]; avtheta[s] = o->avtheta[s]; avn[s] = o->avn_insh[s]; }
}

/* ---- inspection ----------------------------------------------------------- */
long orc_list_size(const orc* o, int kind) {
    switch (kind) {
    case QNB_LIST_PP: return o->nbpp.n;
    case QNB_LIST_PW: return o->nbpw.n;
    case QNB_LIST_WW: return o->nbww.n;
    case QNB_LIST_QP: return o->nbqp.n;
    case QNB_LIST_QW: return o->nbqw.n;
    case QNB_LIST_PP14: {
        long n = 0;
        for (long k = 0; k < o->nbpp14.n; ++k) n += ((char*)o->nbpp14.p)[k];
        return n;
    }
    }
    return -1;
}

long orc_export_pairs(const orc* o, int kind, int32_t* i, int32_t* j) {
    const vec_t* L = NULL;
    switch (kind) {
    case QNB_LIST_PP: case QNB_LIST_PP14: L = &o->nbpp; break;
    case QNB_LIST_PW: L = &o->nbpw; break;
    case QNB_LIST_WW: L = &o->nbww; break;
    case QNB_LIST_QP: L = &o->nbqp; break;
    case QNB_LIST_QW: L = &o->nbqw; break;
    default: return -1;
    }
    const nb_t* e = (const nb_t*)L->p;
    long n = 0;
    for (long k = 0; k < L->n; ++k) {
        if (kind == QNB_LIST_PP14 && !((char*)o->nbpp14.p)[k]) continue;
        i[n] = e[k].i; j[n] = e[k].j; ++n;
    }
    return n;
}

void orc_get_lrf(const orc* o, double* out) {
    memcpy(out, o->lrf, sizeof(double) * (size_t)o->ncgp * NLRF);
}

long orc_static_qq_size(const orc* o, int s, int which) {
    return which == 0 ? o->nbqq[s].n : o->nbqqp[s].n;
}

/* shake(xx, x), src/bondene.f90:1069-1150: constraints grouped per molecule
   (mol_start[m] .. mol_start[m+1]-1), x corrected toward dist2 using the
   reference geometry xx; returns the total iteration count or -1 on failure.
   CONST_TOL 1e-4 and CONST_MAX_ITER 1000 (src/globals.f90:519-520). */
long orc_shake(double* x, const double* xx, int nmol, const int32_t* mol_start, const int32_t* ci,
               const int32_t* cj, const double* dist2, const double* winv) {
    long total = 0;
    char* ready = NULL;
    for (int m = 0; m < nmol; ++m) {
        int c0 = mol_start[m], c1 = mol_start[m + 1];
        int nc = c1 - c0;
        ready = (char*)realloc(ready, nc ? nc : 1);
        memset(ready, 0, nc ? nc : 1);
        int nits = 0;
        for (;;) {
            for (int ic = 0; ic < nc; ++ic) {
                if (ready[ic]) continue;
                int i = ci[c0 + ic], j = cj[c0 + ic];
                v3 xij = vsub(X(x, i), X(x, j));
                double r2 = vsq(xij);
                double diff = dist2[c0 + ic] - r2;
                if (fabs(diff) < 0.0001 * dist2[c0 + ic]) ready[ic] = 1;
                v3 xxij = vsub(X(xx, i), X(xx, j));
                double scp = vdot(xij, xxij);
                double corr = diff / (2.0 * scp * (winv[i] + winv[j]));
                v3 ci_ = vscale(vscale(xxij, corr), winv[i]);
                v3 cj_ = vscale(vscale(vscale(xxij, -1.0), corr), winv[j]);
                x[3 * i] += ci_.x; x[3 * i + 1] += ci_.y; x[3 * i + 2] += ci_.z;
                x[3 * j] += cj_.x; x[3 * j + 1] += cj_.y; x[3 * j + 2] += cj_.z;
            }
            nits++;
            int all = 1;
            for (int ic = 0; ic < nc; ++ic) all &= ready[ic];
            if (all) break;
            if (nits >= 1000) { free(ready); return -1; }
        }
        total += nits;
    }
    free(ready);
    return total;
}

/* ---- MD step pieces (strict FP64, the reference's evaluation order) ------
   newvel_ber src/md.f90:1451-1466; v = (x - xx)/dt src/md.f90:1787-1789;
   temperature src/md.f90:1379-1447; stop_cm_translation
   src/simprep.f90:4496-4518.  SHAKE is orc_shake above. */
static int md_group(int i, int ntg, const int32_t* first, const int32_t* last) {
    for (int g = 0; g < ntg; ++g)
        if (i >= first[g] && i <= last[g]) return g;
    return -1;
}

void orc_md_newvel(int natom, double* x, double* xx, double* v, const double* d, const double* winv, double dt,
                   int ntg, const int32_t* first, const int32_t* last, const double* sfact) {
    for (int g = 0; g < ntg; ++g)
        for (int i = first[g]; i <= last[g]; ++i)
            for (int c = 0; c < 3; ++c) {
                int k = 3 * i + c;
                v[k] = (v[k] - d[k] * winv[i] * dt) * sfact[g];
                xx[k] = x[k];
                x[k] = x[k] + v[k] * dt;
            }
    (void)natom;
}

/* newvel_ber / newvel_nos with the force step `step` (dt, or dt/2 for
   velocity Verlet, which repeats the force half-step after the move),
   src/md.f90:1451-1466, 1505-1521; sfact 1 for Nose-Hoover */
void orc_md_newvel2(int natom, double* x, double* xx, double* v, const double* d, const double* winv, double dt,
                    double step, int vv, int ntg, const int32_t* first, const int32_t* last, const double* sfact) {
    for (int g = 0; g < ntg; ++g)
        for (int i = first[g]; i <= last[g]; ++i)
            for (int c = 0; c < 3; ++c) {
                int k = 3 * i + c;
                double vk = (v[k] - d[k] * winv[i] * step) * sfact[g];
                xx[k] = x[k];
                x[k] = x[k] + vk * dt;
                if (vv) vk = (vk - d[k] * winv[i] * step) * sfact[g];
                v[k] = vk;
            }
    (void)natom;
}

/* newvel_lan, src/md.f90:1468-1503, with the uniform random forces drawn
   from SplitMix64 keyed by (seed, window, step, component) as the device
   does (qdyn's own randm stream is sequential) */
static uint64_t orc_splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
void orc_md_newvel_lan(int natom, double* x, double* xx, double* v, const double* d, const double* winv, double dt,
                       double step, int vv, double friction, double gkT, uint64_t seed, int window, int istep) {
    const double lf = 1.0 - friction * step;
    for (int i = 0; i < natom; ++i) {
        const double rs = sqrt(gkT / winv[i]);
        for (int c = 0; c < 3; ++c) {
            int k = 3 * i + c;
            uint64_t z = orc_splitmix64(orc_splitmix64(orc_splitmix64(seed + (uint64_t)window) + (uint64_t)(uint32_t)istep) +
                                        (uint64_t)k);
            double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
            double re = rs * (u - 0.5);
            double fd = (d[k] - re) * winv[i] * step;
            double vk = v[k] * lf - fd;
            xx[k] = x[k];
            x[k] = x[k] + vk * dt;
            if (vv) vk = vk * lf - fd;
            v[k] = vk;
        }
    }
}

void orc_md_velocity(int natom, const double* x, const double* xx, double* v, double dt) {
    for (int k = 0; k < 3 * natom; ++k) v[k] = (x[k] - xx[k]) / dt;
}

void orc_md_stop_cm(int natom, double* v, const double* mass) {
    double tot = 0.0, vcm[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < natom; ++i) {
        tot = tot + mass[i];
        for (int c = 0; c < 3; ++c) vcm[c] = vcm[c] + v[3 * i + c] * mass[i];
    }
    for (int c = 0; c < 3; ++c) vcm[c] = vcm[c] / tot;
    for (int i = 0; i < natom; ++i)
        for (int c = 0; c < 3; ++c) v[3 * i + c] = v[3 * i + c] - vcm[c];
}

/* out: ekin, temp, tfree, then per group temp, tfree, texcl; sfact updated */
void orc_md_temperature(int natom, const double* v, const double* mass, const uint8_t* excl, int ntg,
                        const int32_t* first, const int32_t* last, const double* tg_ndegf,
                        const double* tg_ndegfree, double ndegf, double ndegfree, double temp0, double dt,
                        double tau, double boltz, double* sfact, double* out) {
    double gt[8] = {0}, gf[8] = {0}, gx[8] = {0};
    for (int g = 0; g < ntg; ++g)
        for (int i = first[g]; i <= last[g]; ++i) {
            double sq = v[3 * i] * v[3 * i] + v[3 * i + 1] * v[3 * i + 1] + v[3 * i + 2] * v[3 * i + 2];
            double ek = 0.5 * mass[i] * sq;
            gt[g] = gt[g] + ek;
            if (!excl[i]) gf[g] = gf[g] + ek;
            else gx[g] = gx[g] + ek;
        }
    double tfree = 0.0, temp = 0.0;
    for (int g = 0; g < ntg; ++g) tfree = tfree + gf[g];
    for (int g = 0; g < ntg; ++g) temp = temp + gt[g];
    out[0] = temp;
    out[1] = 2.0 * temp / boltz / ndegf;
    out[2] = 2.0 * tfree / boltz / ndegfree;
    for (int g = 0; g < ntg; ++g) {
        double tt = 2.0 * gt[g] / boltz / tg_ndegf[g];
        double tf = 2.0 * gf[g] / boltz / tg_ndegfree[g];
        double tx = tg_ndegf[g] != tg_ndegfree[g] ? 2.0 * gx[g] / boltz / (tg_ndegf[g] - tg_ndegfree[g]) : gx[g];
        out[3 + 3 * g] = tt;
        out[4 + 3 * g] = tf;
        out[5 + 3 * g] = tx;
        if (tf != 0.0) sfact[g] = temp0 / tf - 1.0;
        sfact[g] = sqrt(1.0 + dt / tau * sfact[g]);
    }
    (void)natom;
}

/* ---- bonded terms (strict FP64) ------------------------------------------
   bond_calc / angle_calc / torsion_calc / improper_calc src/bonded.f90:53-320;
   bond, angle, urey_bradley, torsion, improper, improper2
   src/bondene.f90:41-385, 689-762; qbond, qangle, qurey_bradley, qtorsion,
   qimproper src/bondene.f90:387-688 (no Morse couplings). */
static v3 vneg(v3 a) { v3 r = {-a.x, -a.y, -a.z}; return r; }
static v3 vcrs(v3 a, v3 b) {
    v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    return r;
}
static v3 vdivs(v3 a, double s) { v3 r = {a.x / s, a.y / s, a.z / s}; return r; }
static void gadd(double* d, int i, v3 g) { d[3 * i] += g.x; d[3 * i + 1] += g.y; d[3 * i + 2] += g.z; }
#define QEPS 1e-10

typedef struct { double angl; v3 a, b, c; } angval;
static angval angle_calc(v3 a, v3 b, v3 c) {
    v3 ab = vsub(a, b), bc = vsub(c, b);
    double ab2 = vsq(ab); ab2 = 1.0 / ab2;
    double bc2 = vsq(bc); bc2 = 1.0 / bc2;
    double abd = sqrt(ab2), bcd = sqrt(bc2);
    double scalar = vdot(ab, bc);
    scalar = scalar * abd * bcd;
    if (scalar > 1.0) scalar = 1.0;
    if (scalar < -1.0) scalar = -1.0;
    angval r;
    r.angl = acos(scalar);
    double inv = sin(r.angl);
    if (fabs(inv) < QEPS) inv = QEPS;
    inv = -1.0 / inv;
    v3 af = vscale(vsub(vscale(vscale(bc, abd), bcd), vscale(ab, ab2 * scalar)), inv);
    v3 cf = vscale(vsub(vscale(vscale(ab, abd), bcd), vscale(bc, bc2 * scalar)), inv);
    r.a = af; r.b = vadd(af, cf); r.c = cf;
    return r;
}

typedef struct { double angl; v3 a, b, c, d; } torval;
static torval torsion_calc(v3 a, v3 b, v3 c, v3 d) {
    v3 ab = vsub(a, b), bc = vsub(c, b), cd = vsub(d, c);
    v3 cabc = vcrs(ab, bc), cbcd = vcrs(vneg(bc), cd);
    double a2abc = vsq(cabc), a2bcd = vsq(cbcd);
    double aabc = sqrt(a2abc), abcd = sqrt(a2bcd);
    double scalar = vdot(cabc, cbcd);
    scalar = scalar / (aabc * abcd);
    if (scalar > 1.0) scalar = 1.0;
    if (scalar < -1.0) scalar = -1.0;
    torval r;
    r.angl = acos(scalar);
    v3 dc = vcrs(cabc, cbcd);
    if (vdot(bc, dc) < 0.0) r.angl = -r.angl;
    double inv = sin(r.angl);
    if (fabs(inv) < QEPS) inv = QEPS;
    inv = -1.0 / inv;
    v3 v1 = vscale(vsub(vdivs(cbcd, aabc * abcd), vscale(vdivs(cabc, a2abc), scalar)), inv);
    v3 v2 = vscale(vsub(vdivs(cabc, aabc * abcd), vscale(vdivs(cbcd, a2bcd), scalar)), inv);
    v3 ca = vsub(ab, bc), db = vsub(vneg(bc), cd);
    r.a = vcrs(bc, v1);
    r.b = vadd(vcrs(ca, v1), vcrs(cd, v2));
    r.c = vsub(vcrs(db, v2), vcrs(ab, v1));
    r.d = vcrs(bc, v2);
    return r;
}

/* Eb[8]: p bond angle torsion improper, w bond angle torsion improper (added);
   EQb[4*S]: per state q bond angle torsion improper (added); d added. */
void orc_bonded(const double* x, double* d, const qnb_bonded* b, int S, const double* lambda, double* Eb,
                double* EQb) {
    const double two_pi = 2.0 * (4.0 * atan(1.0));
    for (int k = 0; k < b->nbonds; ++k) {
        const int32_t* e = b->bonds + 3 * k;
        if (e[2] < 0) continue;
        double fk = b->bondlib[2 * e[2]], b0 = b->bondlib[2 * e[2] + 1];
        v3 av = vsub(X(x, e[1]), X(x, e[0]));
        double dist = sqrt(vsq(av));
        double db = dist - b0;
        Eb[k < b->nbonds_solute ? 0 : 4] += 0.5 * fk * db * db;
        double dv = fk * db / dist;
        gadd(d, e[0], vscale(av, -dv));
        gadd(d, e[1], vscale(av, dv));
    }
    for (int k = 0; k < b->nangles; ++k) {
        const int32_t* e = b->angles + 4 * k;
        if (e[3] < 0) continue;
        const double* L = b->anglib + 4 * e[3];
        angval c = angle_calc(X(x, e[0]), X(x, e[1]), X(x, e[2]));
        double da = c.angl - L[1];
        int slot = k < b->nangles_solute ? 1 : 5;
        Eb[slot] += 0.5 * L[0] * da * da;
        double dv = L[0] * da;
        gadd(d, e[0], vscale(c.a, dv));
        gadd(d, e[1], vscale(c.b, -dv));
        gadd(d, e[2], vscale(c.c, dv));
        if (b->urey_bradley && L[2] > 0.0) {   /* urey_bradley: the reference's gradient signs */
            v3 av = vsub(X(x, e[2]), X(x, e[0]));
            double dist = sqrt(vsq(av));
            double ru = dist - L[3];
            Eb[slot] += L[2] * ru * ru;
            double du = 2.0 * L[2] * ru / dist;
            gadd(d, e[2], vscale(av, -du));
            gadd(d, e[0], vscale(av, du));
        }
    }
    for (int k = b->ntors - 1; k >= 0; --k) {
        const int32_t* e = b->torsions + 5 * k;
        if (e[4] < 0) continue;
        const double* L = b->torlib + 4 * e[4];
        torval c = torsion_calc(X(x, e[0]), X(x, e[1]), X(x, e[2]), X(x, e[3]));
        double arg = L[1] * c.angl - L[2];
        Eb[k < b->ntors_solute ? 2 : 6] += L[0] * (1.0 + cos(arg)) * L[3];
        double dv = -L[1] * L[0] * sin(arg) * L[3];
        gadd(d, e[0], vscale(c.a, dv)); gadd(d, e[1], vscale(c.b, dv));
        gadd(d, e[2], vscale(c.c, dv)); gadd(d, e[3], vscale(c.d, dv));
    }
    for (int k = b->nimps - 1; k >= 0; --k) {
        const int32_t* e = b->impropers + 5 * k;
        if (e[4] < 0) continue;
        const double* L = b->implib + 2 * e[4];
        torval c = torsion_calc(X(x, e[0]), X(x, e[1]), X(x, e[2]), X(x, e[3]));
        double ei, dv;
        if (b->imp_type == 2) {
            double arg = 2.0 * c.angl - L[1];
            ei = L[0] * (1.0 + cos(arg));
            dv = -2.0 * L[0] * sin(arg);
        } else {
            double arg = c.angl - L[1];
            arg = arg - two_pi * round(arg / two_pi);
            dv = L[0] * arg;
            ei = 0.5 * dv * arg;
        }
        Eb[k < b->nimps_solute ? 3 : 7] += ei;
        gadd(d, e[0], vscale(c.a, dv)); gadd(d, e[1], vscale(c.b, dv));
        gadd(d, e[2], vscale(c.c, dv)); gadd(d, e[3], vscale(c.d, dv));
    }
    /* EMorseD / dMorse of every Q bond in the current state (qbond,
       src/bondene.f90:530-548); gamma 1 and no gradient for a bond absent in
       the state or shorter than r0 */
    double* emd = (double*)calloc((size_t)(b->nqbonds > 0 ? b->nqbonds : 1), sizeof(double));
    v3* dmi = (v3*)calloc((size_t)(b->nqbonds > 0 ? b->nqbonds : 1), sizeof(v3));
    for (int st = 0; st < S; ++st) {
        const double lam = lambda[st];
        for (int k = 0; k < b->nqbonds; ++k) {
            int code = b->qbond_code[k * S + st];
            emd[k] = 1.0;
            dmi[k] = vscale(dmi[k], 0.0);
            if (code < 0) continue;
            const double* L = b->qbondlib + 4 * code;
            int i = b->qbonds[2 * k], j = b->qbonds[2 * k + 1];
            v3 av = vsub(X(x, j), X(x, i));
            double dist = sqrt(vsq(av));
            double db = dist - L[2];
            double fexp = exp(-L[1] * db);
            if (db > 0.0) {
                emd[k] = -(fexp * fexp - 2.0 * fexp);
                dmi[k] = vscale(av, 2.0 * L[1] * (fexp - fexp * fexp) * lam / dist);
            }
        }
/* the coupling of term q in table (n, tab): sets gamma, returns the bond or -1 */
#define COUPLING(n, tab, q, gamma)                                                  \
    ({                                                                             \
        int ib_ = -1;                                                              \
        gamma = 1.0;                                                               \
        for (int m_ = 0; m_ < (n); ++m_)                                           \
            if ((tab)[3 * m_] == (q)) {                                            \
                ib_ = (tab)[3 * m_ + 1];                                           \
                gamma = emd[ib_];                                                  \
                if ((tab)[3 * m_ + 2] == 1) gamma = 1.0 - gamma;                   \
                break;                                                             \
            }                                                                      \
        ib_;                                                                       \
    })
#define COUPLED_GRAD(ib, e)                                                         \
    if ((ib) >= 0) {                                                               \
        gadd(d, b->qbonds[2 * (ib)], vscale(dmi[ib], (e)));                        \
        gadd(d, b->qbonds[2 * (ib) + 1], vscale(dmi[ib], -(e)));                   \
    }
        for (int k = 0; k < b->nqbonds; ++k) {
            int code = b->qbond_code[k * S + st];
            if (code < 0) continue;
            const double* L = b->qbondlib + 4 * code;   /* Dmz amz r0 fk */
            int i = b->qbonds[2 * k], j = b->qbonds[2 * k + 1];
            v3 av = vsub(X(x, j), X(x, i));
            double dist = sqrt(vsq(av));
            double db = dist - L[2];
            double fexp = exp(-L[1] * db);
            EQb[4 * st] += L[0] * (fexp * fexp - 2.0 * fexp) + 0.5 * L[3] * db * db;
            double dv = (2.0 * L[0] * L[1] * (fexp - fexp * fexp) + L[3] * db) * lam / dist;
            gadd(d, i, vscale(av, -dv));
            gadd(d, j, vscale(av, dv));
        }
        for (int k = 0; k < b->nqangles; ++k) {
            int code = b->qangle_code[k * S + st];
            if (code < 0) continue;
            const double* L = b->qanglib + 4 * code;
            const int32_t* e = b->qangles + 3 * k;
            double gamma;
            int ib = COUPLING(b->nang_coupl, b->ang_coupl, k, gamma);
            angval c = angle_calc(X(x, e[0]), X(x, e[1]), X(x, e[2]));
            double da = c.angl - L[1];
            double ae = 0.5 * L[0] * da * da;
            EQb[4 * st + 1] += ae * gamma;
            double dv = gamma * L[0] * da * lam;
            gadd(d, e[0], vscale(c.a, dv));
            gadd(d, e[1], vscale(c.b, -dv));
            gadd(d, e[2], vscale(c.c, dv));
            COUPLED_GRAD(ib, ae)
        }
        if (b->urey_bradley)
            for (int k = 0; k < b->nqangles; ++k) {
                int code = b->qangle_code[k * S + st];
                if (code < 0 || b->qanglib[4 * code + 2] == 0.0) continue;
                const double* L = b->qanglib + 4 * code;
                const int32_t* e = b->qangles + 3 * k;
                double gamma;
                int ib = COUPLING(b->nang_coupl, b->ang_coupl, k, gamma);
                v3 av = vsub(X(x, e[2]), X(x, e[0]));
                double dist = sqrt(vsq(av));
                double ru = dist - L[3];
                double eu = L[2] * ru * ru;
                EQb[4 * st + 1] += eu * gamma;
                double du = gamma * 2.0 * (L[2] * ru / dist) * lam;
                gadd(d, e[0], vscale(av, -du));
                gadd(d, e[2], vscale(av, du));
                COUPLED_GRAD(ib, eu)
            }
        for (int k = 0; k < b->nqtors; ++k) {
            int code = b->qtorsion_code[k * S + st];
            if (code < 0) continue;
            const double* L = b->qtorlib + 3 * code;
            const int32_t* e = b->qtorsions + 4 * k;
            double gamma;
            int ib = COUPLING(b->ntor_coupl, b->tor_coupl, k, gamma);
            torval c = torsion_calc(X(x, e[0]), X(x, e[1]), X(x, e[2]), X(x, e[3]));
            double arg = L[1] * c.angl - L[2];
            double pe = L[0] * (1.0 + cos(arg));
            EQb[4 * st + 2] += pe * gamma;
            double dv = -L[1] * L[0] * sin(arg) * gamma * lam;
            gadd(d, e[0], vscale(c.a, dv)); gadd(d, e[1], vscale(c.b, dv));
            gadd(d, e[2], vscale(c.c, dv)); gadd(d, e[3], vscale(c.d, dv));
            COUPLED_GRAD(ib, pe)
        }
        for (int k = 0; k < b->nqimps; ++k) {
            int code = b->qimproper_code[k * S + st];
            if (code < 0) continue;
            const double* L = b->qimplib + 2 * code;
            const int32_t* e = b->qimpropers + 4 * k;
            torval c = torsion_calc(X(x, e[0]), X(x, e[1]), X(x, e[2]), X(x, e[3]));
            double gamma;
            int ib = COUPLING(b->nimp_coupl, b->imp_coupl, k, gamma);
            double arg = c.angl - L[1];
            arg = arg - two_pi * round(arg / two_pi);
            double dv = L[0] * arg;
            double pe = 0.5 * dv * arg;
            EQb[4 * st + 3] += pe * gamma;
            dv = dv * gamma * lam;
            gadd(d, e[0], vscale(c.a, dv)); gadd(d, e[1], vscale(c.b, dv));
            gadd(d, e[2], vscale(c.c, dv)); gadd(d, e[3], vscale(c.d, dv));
            COUPLED_GRAD(ib, pe)
        }
    }
#undef COUPLING
#undef COUPLED_GRAD
    free(emd);
    free(dmi);
}

/* fix_shell, src/potene.f90:386-423: E[0] += fix, E[1] += shell */
void orc_fix_shell(int natom, const double* x, double* d, const double* xtop, const uint8_t* excl,
                   const uint8_t* shell, double fk_fix, double fk_pshell, double* E) {
    for (int i = 0; i < natom; ++i) {
        if (!excl[i] && !shell[i]) continue;
        double fk = excl[i] ? fk_fix : fk_pshell;
        v3 vec = vsub(X(x, i), X(xtop, i));
        double r2 = vsq(vec);
        double erst = 0.5 * fk * r2;
        if (excl[i]) E[0] += erst;
        if (shell[i]) E[1] += erst;
        gadd(d, i, vscale(vec, fk));
    }
}

/* p_restrain, src/bondene.f90:764-1020 (no PBC, no freeze).  Eprot[0] +=
   E%restraint%protein; EQr[s] += EQ(s)%restraint; xtop natom x 3; heavy and
   mass per atom; xwcent the solvent centre.  States as qnb_restraints (-1:
   every state). */
static void rstate(int S, int st, double e, double* Eprot, double* EQr) {
    if (st >= 0) EQr[st] += e;
    else if (S == 0) Eprot[0] += e;
    else for (int k = 0; k < S; ++k) EQr[k] += e;
}
void orc_p_restrain(const double* x, double* d, const qnb_restraints* r, const double* xtop, const uint8_t* heavy,
                    const double* mass, const double* xwcent, int S, const double* lambda, double* Eprot,
                    double* EQr) {
    for (int k = 0; k < r->nseq; ++k) {
        int a = r->seq_ij[2 * k], b = r->seq_ij[2 * k + 1], ih = r->seq_ih[k], mode = r->seq_mode[k];
        double fk = r->seq_fk[k];
        if (mode == 1 || mode == 2) {
            v3 dr = {0.0, 0.0, 0.0};
            double tot = 0.0;
            for (int i = a; i <= b; ++i) {
                if (!(heavy[i] || ih == 1)) continue;
                double w = mode == 2 ? mass[i] : 1.0;
                dr = vadd(dr, vscale(vsub(X(x, i), X(xtop, i)), w));
                tot += w;
            }
            if (tot > 0.0) {
                dr = vscale(dr, 1.0 / tot);
                Eprot[0] += 0.5 * fk * vsq(dr);
                for (int i = a; i <= b; ++i) {
                    if (!(heavy[i] || ih == 1)) continue;
                    gadd(d, i, vscale(dr, mode == 2 ? fk : fk * mass[i] / 12.010));
                }
            }
        } else {
            for (int i = a; i <= b; ++i) {
                if (!(heavy[i] || ih == 1)) continue;
                v3 dr = vsub(X(x, i), X(xtop, i));
                Eprot[0] += 0.5 * fk * vsq(dr);
                gadd(d, i, vscale(dr, fk));
            }
        }
    }
    for (int k = 0; k < r->npos; ++k) {
        int i = r->pos_i[k], st = r->pos_state[k];
        v3 x0 = {r->pos_x[3 * k], r->pos_x[3 * k + 1], r->pos_x[3 * k + 2]};
        v3 fk = {r->pos_fk[3 * k], r->pos_fk[3 * k + 1], r->pos_fk[3 * k + 2]};
        v3 dr = vsub(X(x, i), x0);
        double wgt = st >= 0 ? lambda[st] : 1.0;
        rstate(S, st, 0.5 * (fk.x * dr.x * dr.x + fk.y * dr.y * dr.y + fk.z * dr.z * dr.z), Eprot, EQr);
        v3 g = {fk.x * dr.x * wgt, fk.y * dr.y * wgt, fk.z * dr.z * wgt};
        gadd(d, i, g);
    }
    for (int k = 0; k < r->ndist; ++k) {
        int i = r->dist_ij[2 * k], j = r->dist_ij[2 * k + 1], st = r->dist_state[k];
        v3 av = vsub(X(x, j), X(x, i));
        double dist = sqrt(vsq(av)), db;
        if (dist < r->dist_d[2 * k]) db = dist - r->dist_d[2 * k];
        else if (dist > r->dist_d[2 * k + 1]) db = dist - r->dist_d[2 * k + 1];
        else continue;
        double wgt = st >= 0 ? lambda[st] : 1.0;
        rstate(S, st, 0.5 * r->dist_fk[k] * db * db, Eprot, EQr);
        double dv = wgt * r->dist_fk[k] * db / dist;
        gadd(d, i, vscale(av, -dv));
        gadd(d, j, vscale(av, dv));
    }
    const double deg2rad = (4.0 * atan(1.0)) / 180.0;
    for (int k = 0; k < r->nang; ++k) {
        int i = r->ang_ijk[3 * k], j = r->ang_ijk[3 * k + 1], l = r->ang_ijk[3 * k + 2], st = r->ang_state[k];
        angval c = angle_calc(X(x, i), X(x, j), X(x, l));
        double db = c.angl - r->ang_theta[k] * deg2rad;
        double wgt = st >= 0 ? lambda[st] : 1.0;
        rstate(S, st, 0.5 * r->ang_fk[k] * db * db, Eprot, EQr);
        double dv = wgt * r->ang_fk[k] * db;
        gadd(d, i, vscale(c.a, dv));
        gadd(d, j, vscale(c.b, -dv));
        gadd(d, l, vscale(c.c, dv));
    }
    v3 xw = {xwcent[0], xwcent[1], xwcent[2]};
    for (int k = 0; k < r->nwall; ++k) {
        int a = r->wall_ij[2 * k], b = r->wall_ij[2 * k + 1], ih = r->wall_ih[k];
        double fk = r->wall_fk[k], d0 = r->wall_d[k], aM = r->wall_aMorse[k], dM = r->wall_dMorse[k];
        for (int i = a; i <= b; ++i) {
            if (!(heavy[i] || ih == 1)) continue;
            v3 av = vsub(X(x, i), xw);
            double dist = sqrt(vsq(av));
            double db = dist - d0, erst, dv;
            if (db > 0.0) {
                erst = 0.5 * fk * db * db - dM;
                dv = fk * db / dist;
            } else {
                double fexp = exp(aM * db);
                erst = dM * (fexp * fexp - 2.0 * fexp);
                dv = -2.0 * dM * aM * (fexp - fexp * fexp) / dist;
            }
            Eprot[0] += erst;
            gadd(d, i, vscale(av, dv));
        }
    }
}
