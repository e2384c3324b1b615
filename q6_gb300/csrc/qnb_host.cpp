// Host layer of the qdyn nonbonded engine: the C ABI of include/qnb.h.
//
// qnb_create restates Q6's interaction precompute (src/simprep.f90:2860-3587)
// as compact tables the kernels index by atom type and LJ code instead of the
// reference's per-pair arrays, builds the static Q-Q / Q-bonded lists
// (src/nonbondene.f90:3231-3282), and uploads everything once.  The other
// entry points stage coordinates and gradients and launch the kernels of
// qnb_kernels.cu on the context's stream.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "qnb_internal.h"

using namespace qnb;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CU(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(QNB_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                        __FILE__, __LINE__);                                                      \
    } while (0)

constexpr double kQrealEps = 1.0e-10;   // src/sizes.f90:50

// combination rules, src/simprep.f90:3326-3341
void combine(int rule, double ai, double aj, double bi, double bj, double* A, double* B) {
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

}  // namespace

struct qnb_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    int mixed = 0;
    int use_lrf = 1;
    // host copies of the model pieces the host logic needs
    int natom = 0, nat_solute = 0, nwat = 0, sa = 0, ncgp = 0, ncgp_solute = 0, nqat = 0, S = 0;
    double rexcl_o2 = 0.0;
    DevModel m{};
    DevState s{};
    int* d_iwhich = nullptr;
    uint8_t* d_qnear = nullptr;
    int* d_wsw = nullptr;
    uint8_t* d_heavy_solv = nullptr;
    double* d_shell_tsum = nullptr;
    std::vector<void*> allocs;
    bool lists_built = false, qp_done = false, qw_done = false;
    int counts[C_NUM] = {0};
    SolventDev solv{};
    bool have_solv = false;
    int64_t launches = 0;
    double* h_stage = nullptr;   // pinned staging for x / d (natom*3)
    double* h_e = nullptr;       // pinned energies (kNumE doubles + kNumE fixed)

    template <typename T>
    int alloc(T** p, size_t n) {
        if (n == 0) n = 1;
        cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
        if (e != cudaSuccess) return fail(QNB_ERR_NOMEM, "cudaMalloc(%zu bytes): %s", n * sizeof(T), cudaGetErrorString(e));
        allocs.push_back((void*)*p);
        return QNB_OK;
    }
    template <typename T>
    int upload(T** p, const std::vector<T>& v) {
        int rc = alloc(p, v.size());
        if (rc) return rc;
        if (!v.empty()) CU(cudaMemcpy(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
        return QNB_OK;
    }
    void release(void* p) {
        if (!p) return;
        auto it = std::find(allocs.begin(), allocs.end(), p);
        if (it != allocs.end()) allocs.erase(it);
        cudaFree(p);
    }
};

namespace {

#define TRY(x)                 \
    do {                       \
        int rc_ = (x);         \
        if (rc_) return rc_;   \
    } while (0)

int check_launch() {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(QNB_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e));
    return QNB_OK;
}

// capacity of a list; grows on overflow
template <typename T>
int ensure_cap(qnb_context* c, T** buf, int64_t* cap, int64_t need) {
    if (need <= *cap && *buf) return QNB_OK;
    int64_t n = std::max<int64_t>(need, 1024);
    c->release(*buf);
    *buf = nullptr;
    TRY(c->alloc(buf, (size_t)n));
    *cap = n;
    return QNB_OK;
}

int build_model(qnb_context* c, const qnb_topology* t) {
    const int natom = t->natom, ns = t->nat_solute, nt = t->natyps, nq = t->nqat, S = t->nstates;
    const int sa = t->solv_atom;
    DevModel& m = c->m;
    m.natom = natom;
    m.nat_solute = ns;
    m.nwat = t->nwat;
    m.sa = sa;
    m.ncgp = t->ncgp;
    m.ncgp_solute = t->ncgp_solute;
    m.natyps = nt;
    m.nqat = nq;
    m.S = S;
    m.el14 = t->el14_scale;
    m.use_lrf = c->use_lrf;
    m.spc = (t->ivdw_rule == 1 && t->solvent_type == 0) ? 1 : 0;   // src/potene.f90:347-349
    for (int k = 0; k < 3; ++k) {
        m.xpcent[k] = t->xpcent[k];
        m.xwcent[k] = t->xwcent[k];
    }
    m.rexcl_o2 = t->rexcl_o * t->rexcl_o;
    c->rexcl_o2 = m.rexcl_o2;

    // per-atom arrays
    std::vector<int> iac(t->iac, t->iac + natom);
    std::vector<double> crg(t->crg, t->crg + natom);
    std::vector<uint8_t> excl(t->excl, t->excl + natom);
    std::vector<int> iqatom(natom, -1);
    for (int iq = 0; iq < nq; ++iq) {
        if (t->iqseq[iq] < 0 || t->iqseq[iq] >= ns) return fail(QNB_ERR_ARG, "Q atom %d is not a solute atom", iq);
        iqatom[t->iqseq[iq]] = iq;
    }
    TRY(c->upload((int**)&m.iac, iac));
    TRY(c->upload((double**)&m.crg, crg));
    TRY(c->upload((uint8_t**)&m.excl, excl));
    TRY(c->upload((int**)&m.iqatom, iqatom));
    std::vector<int> iqseq(t->iqseq, t->iqseq + nq);
    TRY(c->upload((int**)&m.iqseq, iqseq));

    // charge groups: slot ranges must be consecutive (as the topology stores them)
    std::vector<int> gslot(t->ncgp + 1), gsw(t->ncgp), iwhich(natom, 0);
    for (int g = 0; g < t->ncgp; ++g) {
        if (t->cgp_first[g] != (g ? t->cgp_last[g - 1] + 1 : 0))
            return fail(QNB_ERR_ARG, "charge group %d: slots not consecutive", g);
        gslot[g] = t->cgp_first[g];
    }
    gslot[t->ncgp] = t->ncgp ? t->cgp_last[t->ncgp - 1] + 1 : 0;
    std::vector<int> gatom(t->cgpatom, t->cgpatom + gslot[t->ncgp]);
    for (int g = 0; g < t->ncgp; ++g) {
        if (gslot[g + 1] <= gslot[g]) return fail(QNB_ERR_ARG, "charge group %d is empty", g);
        int lim = g < t->ncgp_solute ? ns : natom;
        for (int a = gslot[g]; a < gslot[g + 1]; ++a)
            if (gatom[a] < 0 || gatom[a] >= lim) return fail(QNB_ERR_ARG, "charge group %d member out of range", g);
        if (t->cgp_iswitch[g] < 0 || t->cgp_iswitch[g] >= natom) return fail(QNB_ERR_ARG, "switch atom of group %d", g);
    }
    if (t->nwat == 0 && t->ncgp != t->ncgp_solute) return fail(QNB_ERR_ARG, "solvent groups without solvent");
    for (int i = 0; i < natom; ++i)
        if (t->iac[i] < 0 || t->iac[i] >= nt) return fail(QNB_ERR_ARG, "iac of atom %d out of range", i);
    for (int iq = 0; iq < nq; ++iq) {
        if (t->iqseq[iq] < 0 || t->iqseq[iq] >= ns) return fail(QNB_ERR_ARG, "Q atom %d is not a solute atom", iq);
        for (int s = 0; s < S; ++s)
            if (t->qvdw_flag && (t->qiac[iq + nq * s] < 0 || t->qiac[iq + nq * s] >= t->nqlib))
                return fail(QNB_ERR_ARG, "qiac of Q atom %d out of range", iq);
    }
    for (int g = 0; g < t->ncgp; ++g)
        for (int a = gslot[g]; a < gslot[g + 1]; ++a) iwhich[gatom[a]] = g;   // src/simprep.f90:3658-3667
    // solvent groups: group ncgp_solute + w must hold molecule w
    std::vector<int> wsw(std::max(1, t->nwat));
    if (t->nwat > 0) {
        if (sa < 1 || sa > kMaxSolv) return fail(QNB_ERR_UNSUPPORTED, "solv_atom=%d (1..%d supported)", sa, kMaxSolv);
        if (t->ncgp - t->ncgp_solute != t->nwat)
            return fail(QNB_ERR_UNSUPPORTED, "expected one charge group per solvent molecule");
        for (int w = 0; w < t->nwat; ++w) {
            int g = t->ncgp_solute + w, first = ns + sa * w;
            if (gslot[g + 1] - gslot[g] != sa) return fail(QNB_ERR_UNSUPPORTED, "solvent group %d size", g);
            for (int a = 0; a < sa; ++a)
                if (iwhich[first + a] != g) return fail(QNB_ERR_UNSUPPORTED, "solvent group %d members", g);
            wsw[w] = t->cgp_iswitch[g];
        }
    }
    for (int g = 0; g < t->ncgp; ++g)
        gsw[g] = g < t->ncgp_solute ? t->cgp_iswitch[g] : ns + sa * (g - t->ncgp_solute);
    TRY(c->upload((int**)&m.gslot, gslot));
    TRY(c->upload((int**)&m.gatom, gatom));
    TRY(c->upload((int**)&m.gsw, gsw));
    TRY(c->upload(&c->d_iwhich, iwhich));
    TRY(c->upload(&c->d_wsw, wsw));

    // special solute pairs: excluded (listex + listexlong) and 1-4 (list14 +
    // list14long); exclusion wins as in pp_int_comp (src/simprep.f90:2992-3053)
    struct Sp {
        int i, j, k;
    };
    std::vector<Sp> sp;
    for (int p = 0; p < t->nexcl_pairs; ++p) {
        int a = t->excl_pairs[2 * p], b = t->excl_pairs[2 * p + 1];
        sp.push_back({std::min(a, b), std::max(a, b), 1});
    }
    for (int p = 0; p < t->n14_pairs; ++p) {
        int a = t->pairs14[2 * p], b = t->pairs14[2 * p + 1];
        sp.push_back({std::min(a, b), std::max(a, b), 3});
    }
    std::sort(sp.begin(), sp.end(), [](const Sp& x, const Sp& y) {
        return x.i != y.i ? x.i < y.i : (x.j != y.j ? x.j < y.j : x.k < y.k);
    });
    std::vector<int> spec_off(ns + 1, 0), spec_j;
    std::vector<uint8_t> spec_kind;
    for (size_t k = 0; k < sp.size(); ++k) {
        if (k && sp[k].i == sp[k - 1].i && sp[k].j == sp[k - 1].j) continue;   // keep the excluded entry
        if (sp[k].i < 0 || sp[k].j >= ns) return fail(QNB_ERR_ARG, "special pair outside the solute");
        spec_j.push_back(sp[k].j);
        spec_kind.push_back((uint8_t)sp[k].k);
        spec_off[sp[k].i + 1]++;
    }
    for (int i = 0; i < ns; ++i) spec_off[i + 1] += spec_off[i];
    TRY(c->upload((int**)&m.spec_off, spec_off));
    TRY(c->upload((int**)&m.spec_j, spec_j));
    TRY(c->upload((uint8_t**)&m.spec_kind, spec_kind));

    // LJ tables per code (1..3) and type pair: precompute_set_values_pp's A/B
    std::vector<double2> lj(3 * (size_t)nt * nt);
    std::vector<float2> ljf(lj.size());
    std::vector<uint8_t> ljset(lj.size()), ljcod(t->ljcod, t->ljcod + (size_t)nt * nt);
    for (int k = 0; k < 3; ++k)
        for (int a = 0; a < nt; ++a)
            for (int b = 0; b < nt; ++b) {
                double A, B;
                combine(t->ivdw_rule, t->avdw[a * 3 + k], t->avdw[b * 3 + k], t->bvdw[a * 3 + k],
                        t->bvdw[b * 3 + k], &A, &B);
                size_t o = ((size_t)k * nt + a) * nt + b;
                lj[o] = make_double2(A, B);
                ljf[o] = make_float2((float)A, (float)B);
                ljset[o] = (fabs(A) > kQrealEps || fabs(B) > kQrealEps) ? 1 : 0;
            }
    for (auto v : ljcod)
        if (v < 1 || v > 2) return fail(QNB_ERR_ARG, "ljcod entries must be 1 or 2");
    TRY(c->upload((double2**)&m.lj, lj));
    TRY(c->upload((float2**)&m.ljf, ljf));
    TRY(c->upload((uint8_t**)&m.ljset, ljset));
    TRY(c->upload((uint8_t**)&m.ljcod, ljcod));

    // solvent template: types and charges of the first molecule
    // (aLJ_solv/bLJ_solv/chg_solv, src/simprep.f90:3616-3621) and ww_precomp
    std::vector<uint8_t> heavy_solv(kMaxSolv, 0);
    if (t->nwat > 0) {
        for (int a = 0; a < sa; ++a) {
            m.wtype[a] = t->iac[ns + a];
            m.wcrg[a] = t->crg[ns + a];
            m.wcrgf[a] = (float)t->crg[ns + a];
            heavy_solv[a] = t->heavy ? t->heavy[ns + a] : 1;
        }
        for (int a = 0; a < sa; ++a)
            for (int b = 0; b < sa; ++b) {
                int ta = m.wtype[a], tb = m.wtype[b];
                int code = t->ljcod[ta * nt + tb];
                double A, B;
                combine(t->ivdw_rule, t->avdw[ta * 3 + code - 1], t->avdw[tb * 3 + code - 1],
                        t->bvdw[ta * 3 + code - 1], t->bvdw[tb * 3 + code - 1], &A, &B);
                int k = a * kMaxSolv + b;
                m.wwA[k] = A;
                m.wwB[k] = B;
                m.wwE[k] = m.wcrg[a] * m.wcrg[b];
                m.wwAf[k] = (float)A;
                m.wwBf[k] = (float)B;
                m.wwEf[k] = (float)m.wwE[k];
            }
    }
    TRY(c->upload(&c->d_heavy_solv, heavy_solv));

    // ---- Q atoms -------------------------------------------------------------
    auto QC = [&](int s, int i, int iq) { return (int)t->qconn[s + S * (i + ns * iq)]; };
    auto QCRG = [&](int iq, int s) { return t->qcrg[iq + nq * s]; };
    auto QIAC = [&](int iq, int s) { return t->qiac[iq + nq * s]; };
    auto SCL = [&](int iq, int ty, int s) { return t->sc_lookup[iq + nq * (ty + (nt + nq) * s)]; };
    std::vector<uint8_t> qnear(natom, 0);
    for (int i = 0; i < ns; ++i)
        for (int iq = 0; iq < nq && !qnear[i]; ++iq)
            for (int s = 0; s < S; ++s)
                if (QC(s, i, iq) <= 3) { qnear[i] = 1; break; }
    TRY(c->upload(&c->d_qnear, qnear));

    // precompute_set_values_qp, src/simprep.f90:3390-3438
    auto qp_values = [&](int iq, int j, int s, int vdw, int* set) {
        QPar p{};
        int i = t->iqseq[iq];
        int qvdw = (vdw == 2) ? 1 : vdw;
        int k = vdw - 1, qk = qvdw - 1, tj = t->iac[j];
        double qa, qb;
        if (t->qvdw_flag) {
            qa = t->qavdw[QIAC(iq, s) * 3 + qk];
            qb = t->qbvdw[QIAC(iq, s) * 3 + qk];
        } else {
            qa = t->avdw[t->iac[i] * 3 + k];
            qb = t->bvdw[t->iac[i] * 3 + k];
        }
        combine(t->ivdw_rule, qa, t->avdw[tj * 3 + k], qb, t->bvdw[tj * 3 + k], &p.A, &p.B);
        p.el = t->qq_use_library_charges ? t->crg[i] * t->crg[j] : QCRG(iq, s) * t->crg[j];
        *set = (fabs(p.A) > kQrealEps || fabs(p.B) > kQrealEps || fabs(p.el) > kQrealEps);
        p.sc = SCL(iq, tj, s);
        if (vdw == 3) p.el = p.el * t->el14_scale;
        return p;
    };
    // qp_int_comp, src/simprep.f90:3112-3148 (atoms not bonded/angled to Q)
    std::vector<QPar> qp_tab((size_t)std::max(ns, 1) * std::max(nq, 1) * std::max(S, 1));
    if (nq > 0)
        for (int ig = 0; ig < ns; ++ig) {
            if (qnear[ig]) continue;
            for (int jq = 0; jq < nq; ++jq) {
                int vdw = t->ljcod[t->iac[ig] * nt + t->iac[t->iqseq[jq]]];
                for (int s = 0; s < S; ++s) {
                    if (QC(s, ig, jq) == 4) vdw = 3;   // kept for later states, as the reference does
                    int set;
                    qp_tab[((size_t)ig * nq + jq) * S + s] = qp_values(jq, ig, s, vdw, &set);
                }
            }
        }
    std::vector<QParF> qp_tabf(qp_tab.size());
    for (size_t k = 0; k < qp_tab.size(); ++k)
        qp_tabf[k] = QParF{(float)qp_tab[k].A, (float)qp_tab[k].B, (float)qp_tab[k].el, (float)qp_tab[k].sc};
    TRY(c->upload((QPar**)&m.qp_tab, qp_tab));
    TRY(c->upload((QParF**)&m.qp_tabf, qp_tabf));

    // qw_int_comp + precompute_set_values_qw, src/simprep.f90:3272-3292, 3517-3558
    std::vector<QPar> qw_tab((size_t)std::max(nq, 1) * std::max(sa, 1) * std::max(S, 1));
    if (nq > 0 && t->nwat > 0)
        for (int iq = 0; iq < nq; ++iq)
            for (int a = 0; a < sa; ++a) {
                int tw = t->iac[ns + a];
                int vdw = t->ljcod[tw * nt + t->iac[t->iqseq[iq]]];
                int qvdw = (vdw == 2) ? 1 : vdw;
                int i = t->iqseq[iq];
                for (int s = 0; s < S; ++s) {
                    QPar p{};
                    double qa = t->qvdw_flag ? t->qavdw[QIAC(iq, s) * 3 + qvdw - 1] : t->avdw[t->iac[i] * 3 + vdw - 1];
                    double qb = t->qvdw_flag ? t->qbvdw[QIAC(iq, s) * 3 + qvdw - 1] : t->bvdw[t->iac[i] * 3 + vdw - 1];
                    combine(t->ivdw_rule, qa, t->avdw[tw * 3 + vdw - 1], qb, t->bvdw[tw * 3 + vdw - 1], &p.A, &p.B);
                    p.el = t->qq_use_library_charges ? t->crg[i] * t->crg[ns + a] : QCRG(iq, s) * t->crg[ns + a];
                    p.sc = SCL(iq, tw, s);
                    qw_tab[((size_t)iq * sa + a) * S + s] = p;
                }
            }
    std::vector<QParF> qw_tabf(qw_tab.size());
    for (size_t k = 0; k < qw_tab.size(); ++k)
        qw_tabf[k] = QParF{(float)qw_tab[k].A, (float)qw_tab[k].B, (float)qw_tab[k].el, (float)qw_tab[k].sc};
    TRY(c->upload((QPar**)&m.qw_tab, qw_tab));
    TRY(c->upload((QParF**)&m.qw_tabf, qw_tabf));

    // static lists: qq_int_comp + nbqqlist (src/simprep.f90:3152-3268,
    // src/nonbondene.f90:3231-3282)
    std::vector<QQEntry> qq;
    for (int iq = 0; iq + 1 < nq; ++iq) {
        int ia = t->iqseq[iq];
        for (int jq = iq + 1; jq < nq; ++jq) {
            int ja = t->iqseq[jq];
            for (int s = 0; s < S; ++s) {
                int qc = QC(s, ja, iq);
                if (qc < 4) continue;
                double els = 1.0;
                for (int e = 0; e < t->nel_scale; ++e) {
                    int k = t->el_scale_pairs[2 * e], l = t->el_scale_pairs[2 * e + 1];
                    if ((iq == k && jq == l) || (iq == l && jq == k)) {
                        els = t->el_scale[e * S + s];
                        break;
                    }
                }
                int vdw;
                if (qc == 4) vdw = 3;
                else if (!t->qvdw_flag) vdw = t->ljcod[t->iac[ia] * nt + t->iac[ja]];
                else {
                    vdw = 1;
                    for (int e = 0; e < t->nqexpnb; ++e) {
                        int a = t->qexpnb_pairs[2 * e], b = t->qexpnb_pairs[2 * e + 1];
                        if ((iq == a && jq == b) || (jq == a && iq == b)) {
                            vdw = 2;
                            break;
                        }
                    }
                }
                // precompute_set_values_qq, src/simprep.f90:3442-3512
                int k = vdw - 1, ti = QIAC(iq, s), tj = QIAC(jq, s);
                double A, B;
                if (t->ivdw_rule == 1) {
                    if (t->qvdw_flag) {
                        A = t->qavdw[ti * 3 + k] * t->qavdw[tj * 3 + k];
                        B = t->qbvdw[ti * 3 + k] * t->qbvdw[tj * 3 + k];
                    } else {
                        A = t->avdw[t->iac[ia] * 3 + k] * t->avdw[t->iac[ja] * 3 + k];
                        B = t->bvdw[t->iac[ia] * 3 + k] * t->bvdw[t->iac[ja] * 3 + k];
                    }
                } else {
                    double tA, tB;
                    if (t->qvdw_flag) {
                        tA = (vdw == 2) ? t->qavdw[ti * 3 + k] * t->qavdw[tj * 3 + k]
                                        : t->qavdw[ti * 3 + k] + t->qavdw[tj * 3 + k];
                        tB = t->qbvdw[ti * 3 + k] * t->qbvdw[tj * 3 + k];
                    } else {
                        tA = t->avdw[t->iac[ia] * 3 + k] + t->avdw[t->iac[ja] * 3 + k];
                        tB = t->bvdw[t->iac[ia] * 3 + k] * t->bvdw[t->iac[ja] * 3 + k];
                    }
                    if (vdw == 2 && t->qvdw_flag) {
                        A = tA;
                        B = tB;
                    } else {
                        tA = tA * tA;
                        tA = tA * tA * tA;
                        A = (tA * tA) * tB;
                        B = 2.0 * tA * tB;
                    }
                }
                double el = t->qq_use_library_charges ? t->crg[ia] * t->crg[ja] : QCRG(iq, s) * QCRG(jq, s);
                el = el * els;
                double sc = SCL(iq, nt + jq, s);
                bool set = fabs(A) > kQrealEps || fabs(B) > kQrealEps || fabs(el) > kQrealEps;
                if (vdw == 3) el = el * t->el14_scale;
                if (!set) continue;
                qq.push_back(QQEntry{ia, ja, s, (vdw == 2 && t->qvdw_flag) ? 1 : 0, A, B, el, sc});
            }
        }
    }
    int nqq_qq = (int)qq.size();
    for (int ja = 0; ja < ns; ++ja) {
        if (iqatom[ja] >= 0 || !qnear[ja]) continue;
        for (int iq = 0; iq < nq; ++iq) {
            int ia = t->iqseq[iq];
            for (int s = 0; s < S; ++s) {
                int qc = QC(s, ja, iq);
                if (qc < 4) continue;
                int vdw;
                if (qc == 4) vdw = 3;
                else if (t->qvdw_flag) vdw = 1;
                else vdw = t->ljcod[t->iac[ia] * nt + t->iac[ja]];
                int set;
                QPar p = qp_values(iq, ja, s, vdw, &set);
                if (!set) continue;
                qq.push_back(QQEntry{ia, ja, s, 0, p.A, p.B, p.el, p.sc});
            }
        }
    }
    c->s.nqq = (int)qq.size();
    c->s.nqq_qq = nqq_qq;
    TRY(c->upload(&c->s.qq, qq));
    return QNB_OK;
}

int alloc_state(qnb_context* c) {
    DevState& s = c->s;
    const DevModel& m = c->m;
    TRY(c->alloc(&s.x, 3 * (size_t)m.natom));
    TRY(c->alloc(&s.d, 3 * (size_t)m.natom));
    TRY(c->alloc(&s.xq, (size_t)m.natom));
    TRY(c->alloc(&s.fix, 3 * (size_t)m.natom));
    TRY(c->alloc(&s.e, (size_t)kNumE));
    TRY(c->alloc(&s.efix, (size_t)kNumE));
    TRY(c->alloc(&s.lambda, (size_t)std::max(1, m.S)));
    TRY(c->alloc(&s.lrf, (size_t)std::max(1, m.ncgp) * kLrfLen));
    TRY(c->alloc(&s.cnt, (size_t)C_NUM));
    TRY(c->alloc(&s.theta, (size_t)std::max(1, m.nwat)));
    TRY(c->alloc(&s.shell, (size_t)std::max(1, m.nwat)));
    TRY(c->alloc(&s.rank, (size_t)std::max(1, m.nwat)));
    TRY(c->alloc(&s.n_insh, (size_t)kMaxShell));
    TRY(c->alloc(&s.wstate, (size_t)3 * kMaxShell));
    TRY(c->alloc(&c->d_shell_tsum, (size_t)kMaxShell));
    CU(cudaMemset(s.d, 0, sizeof(double) * 3 * m.natom));
    CU(cudaMemset(s.fix, 0, sizeof(unsigned long long) * 3 * m.natom));
    CU(cudaMemset(s.cnt, 0, sizeof(int) * C_NUM));
    CU(cudaMemset(s.wstate, 0, sizeof(double) * 3 * kMaxShell));
    CU(cudaMemset(s.lrf, 0, sizeof(double) * std::max(1, m.ncgp) * kLrfLen));
    std::vector<double> lam(std::max(1, m.S), 1.0);
    CU(cudaMemcpy(s.lambda, lam.data(), lam.size() * sizeof(double), cudaMemcpyHostToDevice));
    // initial list capacities (grown on overflow)
    const double rho = 0.04;   // generous water density (molecules / A^3)
    int64_t per_w = (int64_t)(4.0 / 3.0 * M_PI * 1000.0 * rho) + 64;
    TRY(ensure_cap(c, &s.ww, &s.cap_ww, std::max<int64_t>(1024, (int64_t)m.nwat * per_w / 2)));
    TRY(ensure_cap(c, &s.pw, &s.cap_pw, std::max<int64_t>(1024, (int64_t)m.nat_solute * per_w)));
    TRY(ensure_cap(c, &s.pp, &s.cap_pp, std::max<int64_t>(1024, (int64_t)m.nat_solute * 256)));
    TRY(ensure_cap(c, &s.qp, &s.cap_qp, std::max<int64_t>(1024, (int64_t)m.nat_solute)));
    TRY(ensure_cap(c, &s.qw, &s.cap_qw, std::max<int64_t>(1024, (int64_t)m.nwat)));
    CU(cudaMallocHost((void**)&c->h_stage, sizeof(double) * std::max(3 * m.natom, 64)));
    CU(cudaMallocHost((void**)&c->h_e, sizeof(double) * 2 * kNumE));
    return QNB_OK;
}

int zero_acc(qnb_context* c) {
    CU(cudaMemsetAsync(c->s.e, 0, sizeof(double) * kNumE, c->stream));
    CU(cudaMemsetAsync(c->s.efix, 0, sizeof(unsigned long long) * kNumE, c->stream));
    return QNB_OK;
}

// read energies (FP64 slots + fixed-point slots)
int read_energies(qnb_context* c, double* out) {
    CU(cudaMemcpyAsync(c->h_e, c->s.e, sizeof(double) * kNumE, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(c->h_e + kNumE, c->s.efix, sizeof(double) * kNumE, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    const long long* fx = (const long long*)(c->h_e + kNumE);
    for (int k = 0; k < kNumE; ++k) out[k] = c->h_e[k] + (double)fx[k] * (1.0 / kFix);
    return QNB_OK;
}

int stage_x(qnb_context* c, const double* x) {
    size_t n = 3 * (size_t)c->natom;
    memcpy(c->h_stage, x, n * sizeof(double));
    CU(cudaMemcpyAsync(c->s.x, c->h_stage, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return QNB_OK;
}

// device gradient -> add into the caller's d, then clear the device gradient
int unstage_d(qnb_context* c, double* d) {
    size_t n = 3 * (size_t)c->natom;
    if (c->mixed) {
        launch_apply_fixed(c->m, c->s, c->stream);
        c->launches++;
        TRY(check_launch());
    }
    CU(cudaMemcpyAsync(c->h_stage, c->s.d, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemsetAsync(c->s.d, 0, n * sizeof(double), c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (size_t k = 0; k < n; ++k) d[k] += c->h_stage[k];
    return QNB_OK;
}

int build_lists(qnb_context* c, const Cut& cut) {
    DevState& s = c->s;
    const DevModel& m = c->m;
    bool do_qp = !(c->qp_done && cut.rcq2 > c->rexcl_o2);   // src/nonbondene.f90:3678
    bool do_qw = !(c->qw_done && cut.rcq2 > c->rexcl_o2);   // src/nonbondene.f90:3889
    for (int attempt = 0; attempt < 4; ++attempt) {
        CU(cudaMemsetAsync(s.cnt + C_WW, 0, sizeof(int) * 3, c->stream));   // WW, PW, PP
        CU(cudaMemsetAsync(s.cnt + C_PP14, 0, sizeof(int), c->stream));
        if (do_qp) CU(cudaMemsetAsync(s.cnt + C_QP, 0, sizeof(int), c->stream));
        if (do_qw) CU(cudaMemsetAsync(s.cnt + C_QW, 0, sizeof(int), c->stream));
        if (c->use_lrf) {
            launch_group_centres(m, s, c->stream);
            c->launches++;
        }
        launch_build_pp(m, s, cut, c->stream);
        launch_build_pw(m, s, cut, c->stream);
        if (do_qp) launch_build_qp_impl(m, s, c->d_qnear, cut.rcq2, c->stream);
        launch_build_ww(m, s, cut, c->stream);
        if (do_qw) launch_build_qw(m, s, cut, c->stream);
        c->launches += 5;
        if (c->use_lrf) {
            launch_lrf_accumulate(m, s, cut, c->mixed, c->stream);
            c->launches++;
        }
        TRY(check_launch());
        CU(cudaMemcpyAsync(c->counts, s.cnt, sizeof(int) * C_NUM, cudaMemcpyDeviceToHost, c->stream));
        CU(cudaStreamSynchronize(c->stream));
        bool grow = false;
        auto need = [&](int64_t n, int64_t cap) { return n > cap; };
        if (need(c->counts[C_WW], s.cap_ww)) { TRY(ensure_cap(c, &s.ww, &s.cap_ww, c->counts[C_WW] * 5 / 4 + 1024)); grow = true; }
        if (need(c->counts[C_PW], s.cap_pw)) { TRY(ensure_cap(c, &s.pw, &s.cap_pw, c->counts[C_PW] * 5 / 4 + 1024)); grow = true; }
        if (need(c->counts[C_PP], s.cap_pp)) { TRY(ensure_cap(c, &s.pp, &s.cap_pp, c->counts[C_PP] * 5 / 4 + 1024)); grow = true; }
        if (need(c->counts[C_QP], s.cap_qp)) { TRY(ensure_cap(c, &s.qp, &s.cap_qp, c->counts[C_QP] + 1024)); grow = true; do_qp = true; }
        if (need(c->counts[C_QW], s.cap_qw)) { TRY(ensure_cap(c, &s.qw, &s.cap_qw, c->counts[C_QW] + 1024)); grow = true; do_qw = true; }
        if (!grow) {
            if (do_qp) c->qp_done = true;
            if (do_qw) c->qw_done = true;
            c->lists_built = true;
            return QNB_OK;
        }
    }
    return fail(QNB_ERR_CAPACITY, "pair lists kept overflowing");
}

int compute_nonbond(qnb_context* c, int md) {
    if (!c->lists_built) return fail(QNB_ERR_STATE, "pair lists not built");
    int nl = 0;
    if (c->mixed) {
        launch_pack_mixed(c->m, c->s, c->stream);
        ++nl;
    }
    launch_nonbond(c->m, c->s, c->mixed, md, c->stream, &nl);
    if (c->use_lrf && md) {
        launch_lrf_taylor_impl(c->m, c->s, c->d_iwhich, c->mixed, c->stream);
        ++nl;
    }
    c->launches += nl;
    return check_launch();
}

void add_energies(const double* e, qnb_energies* E, qnb_qenergies* EQ, int S) {
    if (E) {
        E->pp_el += e[E_PP_EL];
        E->pp_vdw += e[E_PP_VDW];
        E->pw_el += e[E_PW_EL];
        E->pw_vdw += e[E_PW_VDW];
        E->ww_el += e[E_WW_EL];
        E->ww_vdw += e[E_WW_VDW];
        E->lrf += e[E_LRF];
    }
    if (EQ)
        for (int s = 0; s < S; ++s) {
            EQ[s].qq_el += e[eq_slot(s, 0)];
            EQ[s].qq_vdw += e[eq_slot(s, 1)];
            EQ[s].qp_el += e[eq_slot(s, 2)];
            EQ[s].qp_vdw += e[eq_slot(s, 3)];
            EQ[s].qw_el += e[eq_slot(s, 4)];
            EQ[s].qw_vdw += e[eq_slot(s, 5)];
        }
}

int64_t list_pairs(const qnb_context* c, int kind) {
    int64_t sa = c->sa;
    switch (kind) {
        case QNB_LIST_PP: return c->counts[C_PP];
        case QNB_LIST_PP14: return c->counts[C_PP14];
        case QNB_LIST_PW: return (int64_t)c->counts[C_PW] * sa;
        case QNB_LIST_WW: return (int64_t)c->counts[C_WW] * sa * sa;
        case QNB_LIST_QP: return (int64_t)c->counts[C_QP] * c->nqat;
        case QNB_LIST_QW: return (int64_t)c->counts[C_QW] * c->nqat * sa;
    }
    return -1;
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" {

const char* qnb_last_error(void) { return g_err.c_str(); }

int32_t qnb_version(void) { return 0x000100; }

int qnb_create(const qnb_topology* t, const qnb_options* opt, qnb_context** out) {
    if (!t || !opt || !out) return fail(QNB_ERR_ARG, "null argument");
    *out = nullptr;
    if (t->natom <= 0 || t->nat_solute < 0 || t->nat_solute > t->natom || t->nwat < 0)
        return fail(QNB_ERR_ARG, "bad atom counts");
    if (t->natom != t->nat_solute + t->nwat * t->solv_atom) return fail(QNB_ERR_ARG, "natom != nat_solute + nwat*solv_atom");
    if (t->nstates < 0 || t->nstates > kMaxStates) return fail(QNB_ERR_UNSUPPORTED, "nstates %d > %d", t->nstates, kMaxStates);
    if (t->nqat > 64) return fail(QNB_ERR_UNSUPPORTED, "nqat %d > 64", t->nqat);
    if (t->nqat > 0 && t->nstates < 1) return fail(QNB_ERR_ARG, "Q atoms need nstates >= 1");
    if (t->iuse_switch_atom != 1) return fail(QNB_ERR_UNSUPPORTED, "any-atom charge-group cut-off (switch atoms off)");
    if (t->natom >= (1 << 28)) return fail(QNB_ERR_UNSUPPORTED, "natom >= 2^28");
    if (opt->precision != QNB_PREC_FP64 && opt->precision != QNB_PREC_MIXED) return fail(QNB_ERR_ARG, "precision");
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return fail(QNB_ERR_CUDA, "no CUDA device: %s", e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
    if (opt->device < 0 || opt->device >= ndev) return fail(QNB_ERR_ARG, "device %d of %d", opt->device, ndev);
    qnb_context* c = new qnb_context();
    c->device = opt->device;
    c->mixed = opt->precision == QNB_PREC_MIXED;
    c->use_lrf = opt->use_lrf ? 1 : 0;
    c->natom = t->natom;
    c->nat_solute = t->nat_solute;
    c->nwat = t->nwat;
    c->sa = t->solv_atom;
    c->ncgp = t->ncgp;
    c->ncgp_solute = t->ncgp_solute;
    c->nqat = t->nqat;
    c->S = t->nstates;
    int rc = QNB_OK;
    if (cudaSetDevice(c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
        rc = fail(QNB_ERR_CUDA, "stream creation failed");
    if (!rc) rc = build_model(c, t);
    if (!rc) rc = alloc_state(c);
    if (rc) {
        qnb_destroy(c);
        return rc;
    }
    *out = c;
    return QNB_OK;
}

int qnb_destroy(qnb_context* c) {
    if (!c) return QNB_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : c->allocs) cudaFree(p);
    if (c->h_stage) cudaFreeHost(c->h_stage);
    if (c->h_e) cudaFreeHost(c->h_e);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return QNB_OK;
}

int qnb_set_lambda(qnb_context* c, const double* lambda) {
    if (!c || (!lambda && c->S > 0)) return fail(QNB_ERR_ARG, "null argument");
    if (c->S == 0) return QNB_OK;
    CU(cudaSetDevice(c->device));
    memcpy(c->h_stage, lambda, sizeof(double) * c->S);
    CU(cudaMemcpyAsync(c->s.lambda, c->h_stage, sizeof(double) * c->S, cudaMemcpyHostToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return QNB_OK;
}

int qnb_make_pair_lists_dev(qnb_context* c, double Rq, double Rcq2, double RcLRF2, double Rcpp2, double Rcpw2,
                            double Rcww2) {
    (void)Rq;
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    Cut cut{Rcq2, RcLRF2, Rcpp2, Rcpw2, Rcww2};
    return build_lists(c, cut);
}

int qnb_make_pair_lists(qnb_context* c, const double* x, double Rq, double Rcq2, double RcLRF2, double Rcpp2,
                        double Rcpw2, double Rcww2) {
    if (!c || !x) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    return qnb_make_pair_lists_dev(c, Rq, Rcq2, RcLRF2, Rcpp2, Rcpw2, Rcww2);
}

int qnb_pot_energy_nonbonds(qnb_context* c, const double* x, double* d, qnb_energies* E, qnb_qenergies* EQ,
                            int32_t md) {
    if (!c || !x || !d) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    TRY(zero_acc(c));
    TRY(compute_nonbond(c, md));
    TRY(unstage_d(c, d));
    double e[kNumE];
    TRY(read_energies(c, e));
    add_energies(e, E, EQ, c->S);
    return QNB_OK;
}

int qnb_nonbond_qq(qnb_context* c, const double* x, double* d, qnb_qenergies* EQ) {
    if (!c || !x || !d) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    TRY(zero_acc(c));
    launch_nonbond_qq(c->m, c->s, c->mixed, c->stream);
    c->launches++;
    TRY(check_launch());
    TRY(unstage_d(c, d));
    double e[kNumE];
    TRY(read_energies(c, e));
    add_energies(e, nullptr, EQ, c->S);
    return QNB_OK;
}

int qnb_set_solvent_params(qnb_context* c, const qnb_solvent_params* p) {
    if (!c || !p) return fail(QNB_ERR_ARG, "null argument");
    if (p->wpol_restr && (p->nwpolr_shell < 1 || p->nwpolr_shell > kMaxShell))
        return fail(QNB_ERR_ARG, "nwpolr_shell must be 1..%d", kMaxShell);
    CU(cudaSetDevice(c->device));
    SolventDev& s = c->solv;
    s.fk_wsphere = p->fk_wsphere;
    s.Dwmz = p->Dwmz;
    s.awmz = p->awmz;
    s.rwat = p->rwat;
    s.boltz = p->boltz;
    s.fkwpol = p->fkwpol;
    s.itdis = p->itdis;
    s.wpol = p->wpol_restr;
    s.nshell = p->nwpolr_shell;
    for (int k = 0; k < kMaxShell; ++k) {
        s.rout[k] = p->shell_rout[k];
        s.dr[k] = p->shell_dr[k];
        s.cstb[k] = p->shell_cstb[k];
    }
    double ws[3 * kMaxShell] = {0};
    for (int k = 0; k < kMaxShell; ++k) ws[k] = p->theta_corr[k];
    CU(cudaMemcpyAsync(c->s.wstate, ws, sizeof(ws), cudaMemcpyHostToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    c->have_solv = true;
    return QNB_OK;
}

int qnb_restrain_solvent(qnb_context* c, const double* x, double* d, double Tfree, double* E) {
    if (!c || !x || !d || !E) return fail(QNB_ERR_ARG, "null argument");
    if (!c->have_solv) return fail(QNB_ERR_STATE, "solvent parameters not set");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    TRY(zero_acc(c));
    launch_restrain_solvent_impl(c->m, c->s, c->solv, Tfree, c->mixed, c->d_wsw, c->d_heavy_solv, c->stream);
    c->launches++;
    TRY(check_launch());
    TRY(unstage_d(c, d));
    double e[kNumE];
    TRY(read_energies(c, e));
    *E += e[E_RST_RAD];
    return QNB_OK;
}

int qnb_watpol(qnb_context* c, const double* x, double* d, int32_t istep, int32_t md, double* E) {
    if (!c || !x || !d || !E) return fail(QNB_ERR_ARG, "null argument");
    if (!c->have_solv) return fail(QNB_ERR_STATE, "solvent parameters not set");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    TRY(zero_acc(c));
    int nl = 0;
    launch_watpol_impl(c->m, c->s, c->solv, istep, md, c->mixed, c->d_shell_tsum, c->stream, &nl);
    c->launches += nl;
    TRY(check_launch());
    TRY(unstage_d(c, d));
    double e[kNumE];
    TRY(read_energies(c, e));
    *E += e[E_RST_POL];
    return QNB_OK;
}

int qnb_get_watpol_state(qnb_context* c, double* theta_corr, double* avtheta, double* avn_insh) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    double ws[3 * kMaxShell];
    CU(cudaMemcpyAsync(ws, c->s.wstate, sizeof(ws), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (int k = 0; k < kMaxShell; ++k) {
        if (theta_corr) theta_corr[k] = ws[k];
        if (avtheta) avtheta[k] = ws[kMaxShell + k];
        if (avn_insh) avn_insh[k] = ws[2 * kMaxShell + k];
    }
    return QNB_OK;
}

int qnb_list_size(qnb_context* c, int32_t kind, int64_t* n) {
    if (!c || !n) return fail(QNB_ERR_ARG, "null argument");
    int64_t v = list_pairs(c, kind);
    if (v < 0) return fail(QNB_ERR_ARG, "list kind %d", kind);
    *n = v;
    return QNB_OK;
}

int qnb_export_pairs(qnb_context* c, int32_t kind, int32_t* i, int32_t* j, int64_t cap, int64_t* n) {
    if (!c || !n) return fail(QNB_ERR_ARG, "null argument");
    int64_t cnt = list_pairs(c, kind);
    if (cnt < 0) return fail(QNB_ERR_ARG, "list kind %d", kind);
    *n = cnt;
    if (cnt > cap) return fail(QNB_ERR_CAPACITY, "export needs %lld pairs", (long long)cnt);
    if (cnt == 0) return QNB_OK;
    CU(cudaSetDevice(c->device));
    int32_t *di = nullptr, *dj = nullptr;
    int* dc = nullptr;
    CU(cudaMalloc(&di, cnt * sizeof(int32_t)));
    CU(cudaMalloc(&dj, cnt * sizeof(int32_t)));
    CU(cudaMalloc(&dc, sizeof(int)));
    CU(cudaMemsetAsync(dc, 0, sizeof(int), c->stream));
    launch_export_pairs(c->m, c->s, kind, di, dj, cnt, dc, c->stream);
    int rc = check_launch();
    if (!rc) {
        cudaMemcpyAsync(i, di, cnt * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
        cudaMemcpyAsync(j, dj, cnt * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) rc = fail(QNB_ERR_CUDA, "export copy failed");
    }
    cudaFree(di);
    cudaFree(dj);
    cudaFree(dc);
    return rc;
}

int qnb_get_lrf(qnb_context* c, double* lrf) {
    if (!c || !lrf) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    CU(cudaMemcpyAsync(lrf, c->s.lrf, sizeof(double) * kLrfLen * c->ncgp, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return QNB_OK;
}

int qnb_device_buffers(qnb_context* c, double** x_dev, double** d_dev) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    if (x_dev) *x_dev = c->s.x;
    if (d_dev) *d_dev = c->s.d;
    return QNB_OK;
}

int qnb_stream(qnb_context* c, void** stream) {
    if (!c || !stream) return fail(QNB_ERR_ARG, "null argument");
    *stream = (void*)c->stream;
    return QNB_OK;
}

int qnb_compute_dev(qnb_context* c, double Tfree, int32_t istep, int32_t sync, qnb_energies* E, qnb_qenergies* EQ,
                    double* Erst) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    TRY(zero_acc(c));
    TRY(compute_nonbond(c, 1));
    launch_nonbond_qq(c->m, c->s, c->mixed, c->stream);
    c->launches++;
    if (c->have_solv) {
        launch_restrain_solvent_impl(c->m, c->s, c->solv, Tfree, c->mixed, c->d_wsw, c->d_heavy_solv, c->stream);
        c->launches++;
        int nl = 0;
        launch_watpol_impl(c->m, c->s, c->solv, istep, 1, c->mixed, c->d_shell_tsum, c->stream, &nl);
        c->launches += nl;
    }
    if (c->mixed) {
        launch_apply_fixed(c->m, c->s, c->stream);
        c->launches++;
    }
    TRY(check_launch());
    if (sync) {
        double e[kNumE];
        TRY(read_energies(c, e));
        add_energies(e, E, EQ, c->S);
        if (Erst) {
            Erst[0] += e[E_RST_RAD];
            Erst[1] += e[E_RST_POL];
        }
    }
    return QNB_OK;
}

int qnb_take_launch_count(qnb_context* c, int64_t* n) {
    if (!c || !n) return fail(QNB_ERR_ARG, "null argument");
    *n = c->launches;
    c->launches = 0;
    return QNB_OK;
}

}  // extern "C"
