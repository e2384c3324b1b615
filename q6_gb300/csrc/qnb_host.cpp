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
#include <functional>
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

int qnb::set_error(int code, const char* msg) {
    g_err = msg;
    return code;
}

struct qnb_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;   // list build: the LRF accumulation runs beside the row build
    // mixed form's evaluation: after the coordinate pack the rows run on the
    // main stream, the Q-environment / LRF Taylor kernels on stream2 and the
    // rest of the step's terms on stream3, joined before the gradient apply
    cudaStream_t stream3 = nullptr;
    cudaEvent_t ev_pk = nullptr, ev_jb = nullptr, ev_jc = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int mixed = 0;
    int use_lrf = 1;
    // host copies of the model pieces the host logic needs
    int natom = 0, nat_solute = 0, nwat = 0, sa = 0, ncgp = 0, ncgp_solute = 0, nqat = 0, S = 0;
    double rexcl_o2 = 0.0;
    DevModel m{};
    int nwin = 1;
    std::vector<DevState> st;      // per-window device state (host copy of the pointers)
    QQEntry* st_qq = nullptr;      // static Q-Q / Q-bonded lists (shared by the windows)
    float4* st_qqf = nullptr;      // their (A, B, el, sc) in FP32 for the mixed form
    float* lambdaf_all = nullptr;  // [W][kMaxStates] lambda in FP32
    int nqq = 0, nqq_qq = 0;
    DevState* d_states = nullptr;  // the same, on the device
    double* x_all = nullptr;       // [nwin][natom][3]
    double* e_all = nullptr;       // [nwin][kNumE] FP64 energy slots
    unsigned long long* efix_all = nullptr;   // [nwin][kNumE] fixed-point slots
    int* cnt_all = nullptr;        // [nwin][C_NUM] list counters
    double* d_all = nullptr;       // [nwin][natom][3]
    int* d_iwhich = nullptr;
    int* d_lrf_src = nullptr;      // per atom: LRF source distance atom | solute flag << 30, or -1
    // LRF source tables of the two boundaries: [0] the sphere's (groups whose
    // distance atom is excluded are no source), [1] the box's (the box lists
    // test no exclusion); qnb_set_box switches DevModel and d_lrf_src between them
    struct LrfTables {
        int* src = nullptr;
        int* gmeta = nullptr;
        int* goff = nullptr;
        int* gatom = nullptr;
        int n = 0;
    } lrft[2];
    // exclusion flags: the topology's, and all-clear for the box (excluded
    // atoms take part in every box list, in lrf_taylor and in temperature())
    uint8_t* d_excl_top = nullptr;
    uint8_t* d_excl_none = nullptr;
    uint8_t* d_qnear = nullptr;
    int* d_wsw = nullptr;
    uint8_t* d_heavy_solv = nullptr;
    double* d_shell_tsum = nullptr;
    std::vector<void*> allocs;
    bool lists_built = false, qp_done = false, qw_done = false;
    bool diag_valid = false;       // mixed form: half lists for inspection built from x_build
    Cut last_cut{};
    int last_build_nw = 1;
    int maxg = 1;                  // largest solute charge group
    bool rows_pending = false;     // mixed form: frow not yet added into d
    // CUDA-graph replay of qnb_compute_dev: one instantiated graph per
    // variant (watpol theta_corr update step or not), valid while its key
    // (launch-geometry epoch, Tfree) matches
    bool use_graphs = true;
    bool branches = true;            // mixed form: the evaluation's parallel branches (qnb_set_concurrency)
    uint64_t epoch = 1;            // bumped whenever launch parameters change
    struct Pending {
        int k;
        cudaEvent_t a, b;
        bool owned;    // the events belong to a captured graph (not pooled)
    };
    struct GraphSlot {
        cudaGraphExec_t exec = nullptr;
        uint64_t key_epoch = 0;
        double key_tfree = 0.0;
        unsigned key_mask = 0;
        int64_t nlaunch = 0;
        std::vector<Pending> prof;   // profiled graphs: the event pairs their nodes record
    } gslot[2][2];                   // [watpol update step][profiled]
    bool capturing = false;          // timed() is recording into a graph capture
    std::vector<Pending> cap_pending;
    bool qenv_pending = false;     // mixed form: fq not yet added into d
    int nsi = 0;                   // nonbnd_solv_int pairs (solvents with torsions)
    int2* d_si = nullptr;
    double* d_sip = nullptr;       // [nsi][A, B, el]
    DevState* d_diag = nullptr;    // scratch device state for inspection builds
    std::vector<int> counts;       // [nwin][C_NUM] after the last build
    SolventDev solv{};
    bool have_solv = false;
    int64_t launches = 0;
    // optional per-kernel-class event timing (qnb_profile)
    bool profiling = false;
    unsigned prof_mask = ~0u;      // kernel classes bracketed with events while profiling
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> ev_pool;
    double prof_ms[K_NUM] = {0};
    int64_t prof_n[K_NUM] = {0};
    double* h_stage = nullptr;   // pinned staging for x / d (natom*3)
    double* h_e = nullptr;       // pinned energies (nwin x (kNumE doubles + kNumE fixed))

    std::vector<uint8_t> h_heavy;  // topology heavy-atom flags
    // p_restrain (qnb_set_restraints)
    RestrDev restr{};
    bool have_restr = false;
    std::vector<void*> restr_bufs;
    // offdiag (qnb_set_offdiag)
    OffdDev offd{};
    std::vector<void*> offd_bufs;
    // pair parameters kept from build_model for the listed pair sets
    struct PairSrc {
        std::vector<QQEntry> qq;        // the static Q-Q and Q-bonded-P entries (qq first, nqq_qq of them)
        std::vector<QPar> qp;           // [nat_solute][nqat][S] (Q atoms with atoms not bonded/angled to Q)
        std::vector<uint8_t> qp_set;    // same layout
        std::vector<uint8_t> qnear;     // [natom] bonded/angled to a Q atom in some state
        std::vector<int> iqatom;        // [natom] Q index or -1
        std::vector<int> iqseq;         // [nqat] atom of each Q atom
        std::vector<double> crg;        // [natom]
        std::vector<int> iac;           // [natom]
        std::vector<double2> lj;        // [3][nt][nt]
        std::vector<uint8_t> ljcod;     // [nt][nt]
        std::vector<std::pair<long long, int>> special;   // (i*natom + j, 1 excluded | 3 1-4), i < j, sorted
        int nt = 0;
        double el14 = 1.0;
    } psrc;
    // monitor groups and group contributions (one device list, monitor slots first)
    std::vector<PairSetEntry> mon_e, exc_e;
    std::vector<int> mon_first, exc_first;   // per slot entry counts turned into offsets
    int mon_pairs = 0, exc_groups = 0;
    PairSetDev psets{};
    std::vector<void*> pset_bufs;
    // fix_shell (qnb_set_shell_restraint)
    bool have_shell = false;
    uint8_t* d_shell_flags = nullptr;
    double* d_xtop = nullptr;
    double fk_fix = 0.0, fk_pshell = 0.0;
    int freeze = 0;                // excluded_freeze (qnb_set_freeze)
    // bonded terms (qnb_set_bonded)
    bool have_bonded = false;
    BondedDev bonded{};
    std::vector<void*> bonded_bufs;
    // device-resident MD (qnb_md_*)
    bool md_ready = false;         // qnb_md_init done
    bool md_prepared = false;      // qnb_md_prepare done since the last state change
    qnb_md_params mdp{};
    MdDev md{};
    double* md_rec = nullptr;      // [md_rec_steps][nwin][kMdRec] step records
    int md_rec_steps = 0;
    double* h_md_rec = nullptr;    // pinned copy of one chunk of records

    Tune tune = kTuneDefault;
    Launch all() const { return Launch{m, st[0], d_states, nwin, stream, tune}; }
    Launch one() const { return Launch{m, st[0], d_states, 1, stream, tune}; }   // window 0 only

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

cudaEvent_t take_event(qnb_context* c) {
    if (!c->ev_pool.empty()) {
        cudaEvent_t e = c->ev_pool.back();
        c->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// runs f (which enqueues kernels on c->stream), bracketed by events when
// profiling is on
template <typename F>
void timed_on(qnb_context* c, cudaStream_t st, int k, F&& f) {
    if (!c->profiling || !((c->prof_mask >> k) & 1u)) {
        f();
        return;
    }
    cudaEvent_t a = take_event(c), b = take_event(c);
    // inside a capture, an external record becomes an event-record node that
    // records the event on every replay (a plain record only orders streams)
    const unsigned fl = c->capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    cudaEventRecordWithFlags(a, st, fl);
    f();
    cudaEventRecordWithFlags(b, st, fl);
    if (c->capturing) c->cap_pending.push_back({k, a, b, true});
    else c->pending.push_back({k, a, b, false});
}
template <typename F>
void timed(qnb_context* c, int k, F&& f) {
    timed_on(c, c->stream, k, f);
}

void collect_profile(qnb_context* c) {
    if (c->pending.empty()) return;
    cudaStreamSynchronize(c->stream);
    for (auto& p : c->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            c->prof_ms[p.k] += ms;
            c->prof_n[p.k] += 1;
        } else {
            cudaGetLastError();   // a missing time must not surface as a later launch error
        }
        if (!p.owned) {
            c->ev_pool.push_back(p.a);
            c->ev_pool.push_back(p.b);
        }
    }
    c->pending.clear();
}

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

// points the model's LRF source tables (and the per-atom source array) at
// the sphere's (0) or the box's (1)
void use_lrf_tables(qnb_context* c, int tab) {
    const auto& T = c->lrft[tab];
    c->m.nlrf_groups = T.n;
    c->m.lrf_gmeta = T.gmeta;
    c->m.lrf_goff = T.goff;
    c->m.lrf_gatom = T.gatom;
    c->d_lrf_src = T.src;
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
    m.el14f = (float)m.el14;
    m.use_lrf = c->use_lrf;
    m.any_atom = t->iuse_switch_atom == 0;   // nbpplis2/nbpwlis2/nbqplis2 group tests
    m.spc = (t->ivdw_rule == 1 && t->solvent_type == 0) ? 1 : 0;   // src/potene.f90:347-349
    for (int k = 0; k < 3; ++k) {
        m.xpcent[k] = t->xpcent[k];
        m.xwcent[k] = t->xwcent[k];
        m.wcoff[k] = (float)(t->xpcent[k] - t->xwcent[k]);
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
    TRY(c->upload(&c->d_excl_top, excl));
    TRY(c->upload(&c->d_excl_none, std::vector<uint8_t>(natom, 0)));
    m.excl = c->d_excl_top;
    TRY(c->upload((int**)&m.iqatom, iqatom));
    std::vector<int> iqseq(t->iqseq, t->iqseq + nq);
    TRY(c->upload((int**)&m.iqseq, iqseq));

    // charge groups: slot ranges must be consecutive (as the topology stores them)
    // iwhich: an atom's charge group, -1 for atoms in none (a sphere topology
    // leaves excluded atoms out of the groups)
    std::vector<int> gslot(t->ncgp + 1), gsw(t->ncgp), iwhich(natom, -1);
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
    {   // each atom's unit reference atom (the lattice shifts of the box rows)
        std::vector<int> swat(natom);
        for (int i = 0; i < natom; ++i)
            swat[i] = i >= ns ? ns + sa * ((i - ns) / sa) : (iwhich[i] >= 0 ? gsw[iwhich[i]] : i);
        TRY(c->upload((int**)&m.swat, swat));
    }
    // lrf_update sources: non-Q atoms (src/nonbondene.f90:658-660); in the
    // sphere only of groups whose distance atom is not excluded (the list
    // builders' excl skips), in the box of every group
    for (int tab = 0; tab < 2; ++tab) {
        std::vector<int> lrf_src(natom, -1);
        for (int i = 0; i < natom; ++i) {
            if (iqatom[i] >= 0 || iwhich[i] < 0) continue;
            int g = iwhich[i];
            int d = g < t->ncgp_solute ? t->cgp_iswitch[g] : ns + sa * (g - t->ncgp_solute);
            if (tab == 0 && t->excl[d]) continue;
            lrf_src[i] = d | ((g < t->ncgp_solute ? 1 : 0) << 30);
        }
        // the same sources grouped by charge group, in group order
        std::vector<int> gmeta, goff{0}, gat;
        for (int g = 0; g < t->ncgp; ++g) {
            int n0 = (int)gat.size(), meta = -1;
            for (int a = gslot[g]; a < gslot[g + 1]; ++a) {
                int i = gatom[a];
                if (lrf_src[i] < 0) continue;
                meta = lrf_src[i];
                gat.push_back(i);
            }
            if ((int)gat.size() > n0) {
                gmeta.push_back(meta);
                goff.push_back((int)gat.size());
            }
        }
        auto& T = c->lrft[tab];
        T.n = (int)gmeta.size();
        TRY(c->upload(&T.src, lrf_src));
        TRY(c->upload(&T.gmeta, gmeta));
        TRY(c->upload(&T.goff, goff));
        TRY(c->upload(&T.gatom, gat));
    }
    use_lrf_tables(c, 0);
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
    // per solute group pair: the special atom pairs, keyed g1*ncgp_solute+g2
    std::vector<int> slot_of(natom, -1);
    // a group of Q atoms only has no pair rows (Q atoms take no part in the
    // pp / pw lists or as LRF sources), so its size is not bounded
    std::vector<uint8_t> gallq(std::max(1, t->ncgp_solute), 0);
    for (int g = 0; g < t->ncgp_solute; ++g) {
        int nonq = 0;
        for (int a = gslot[g]; a < gslot[g + 1]; ++a) nonq += iqatom[gatom[a]] < 0 ? 1 : 0;
        gallq[g] = nonq == 0 ? 1 : 0;
        if (gslot[g + 1] - gslot[g] > kMaxGroup && !gallq[g])
            return fail(QNB_ERR_UNSUPPORTED, "solute charge group %d has %d atoms (max %d unless all are Q atoms)", g,
                        gslot[g + 1] - gslot[g], kMaxGroup);
        for (int a = gslot[g]; a < gslot[g + 1]; ++a) slot_of[gatom[a]] = a - gslot[g];
        if (!gallq[g]) c->maxg = std::max(c->maxg, gslot[g + 1] - gslot[g]);
    }
    TRY(c->upload((uint8_t**)&m.gallq, gallq));
    // must agree with k_rows_solute's template choice (MAXG <= 8)
    m.type_in_entry = (c->maxg <= 8 && t->natyps <= 0xffff) ? 1 : 0;
    struct SG {
        long long key;
        int ent;
    };
    std::vector<SG> sg;
    for (size_t k = 0; k < sp.size(); ++k) {
        if (k && sp[k].i == sp[k - 1].i && sp[k].j == sp[k - 1].j) continue;   // the excluded entry wins
        if (sp[k].i < 0 || sp[k].j >= ns) return fail(QNB_ERR_ARG, "special pair outside the solute");
        int i = sp[k].i, j = sp[k].j;   // i < j
        int gi = iwhich[i], gj = iwhich[j];
        if (gi < 0 || gj < 0) continue;   // an atom in no charge group is in no pair list
        int si = slot_of[i], sj = slot_of[j];
        if (gi > gj) {
            std::swap(gi, gj);
            std::swap(si, sj);
        }
        sg.push_back({(long long)gi * t->ncgp_solute + gj, si | (sj << 8) | (sp[k].k << 16)});
    }
    std::stable_sort(sg.begin(), sg.end(), [](const SG& a, const SG& b) { return a.key < b.key; });
    std::vector<long long> sg_key;
    std::vector<int> sg_off, sg_ent;
    for (size_t k = 0; k < sg.size(); ++k) {
        if (k == 0 || sg[k].key != sg[k - 1].key) {
            sg_key.push_back(sg[k].key);
            sg_off.push_back((int)k);
        }
        sg_ent.push_back(sg[k].ent);
    }
    sg_off.push_back((int)sg.size());
    m.nsg = (int)sg_key.size();
    TRY(c->upload((long long**)&m.sg_key, sg_key));
    TRY(c->upload((int**)&m.sg_off, sg_off));
    TRY(c->upload((int**)&m.sg_ent, sg_ent));
    {
        std::vector<std::vector<int2>> per(std::max(1, t->ncgp_solute));
        for (int k = 0; k < m.nsg; ++k) {
            int gi = (int)(sg_key[k] / t->ncgp_solute), gj = (int)(sg_key[k] % t->ncgp_solute);
            per[gi].push_back(make_int2(gj, k));
            if (gj != gi) per[gj].push_back(make_int2(gi, k));
        }
        std::vector<int> off{0};
        std::vector<int2> ent;
        for (int g = 0; g < t->ncgp_solute; ++g) {
            ent.insert(ent.end(), per[g].begin(), per[g].end());
            off.push_back((int)ent.size());
        }
        if (ent.empty()) ent.push_back(make_int2(-1, -1));
        TRY(c->upload((int**)&m.sgl_off, off));
        TRY(c->upload((int2**)&m.sgl_ent, ent));
        // kind masks of both orientations (the entries hold (slot in gl,
        // slot in gu); a group's own pairs are stored with i < j and hold for
        // both orders)
        std::vector<int> moff{0};
        std::vector<unsigned> mk;
        for (int k = 0; k < m.nsg; ++k) {
            int gl = (int)(sg_key[k] / t->ncgp_solute), gu = (int)(sg_key[k] % t->ncgp_solute);
            int nl = gslot[gl + 1] - gslot[gl], nu = gslot[gu + 1] - gslot[gu];
            size_t base = mk.size();
            mk.resize(base + nu + (gl == gu ? 0 : nl), 0u);
            if (gallq[gl] || gallq[gu]) {   // no row of a Q-only group; the other row skips its (Q) atoms
                moff.push_back((int)mk.size());
                continue;
            }
            unsigned* lo = mk.data() + base;           // row gl, partner b of gu
            unsigned* hi = lo + nu;                    // row gu, partner b of gl
            if (gl == gu)
                for (int b = 0; b < nu; ++b) lo[b] |= 1u << (2 * b);
            for (int q = sg_off[k]; q < sg_off[k + 1]; ++q) {
                int e = sg_ent[q], sa = e & 0xff, sb = (e >> 8) & 0xff;
                unsigned kind = (unsigned)(e >> 16);
                lo[sb] |= kind << (2 * sa);
                if (gl == gu) lo[sa] |= kind << (2 * sb);
                else hi[sa] |= kind << (2 * sb);
            }
            moff.push_back((int)mk.size());
        }
        if (mk.empty()) mk.push_back(0u);
        TRY(c->upload((int**)&m.sgm_off, moff));
        TRY(c->upload((unsigned**)&m.sgm, mk));
    }

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
                // geometric rule: the FP32 product of the FP32 factors, which
                // the plain partners of the solute rows form in the kernel
                ljf[o] = t->ivdw_rule == 1
                             ? make_float2((float)t->avdw[a * 3 + k] * (float)t->avdw[b * 3 + k],
                                           (float)t->bvdw[a * 3 + k] * (float)t->bvdw[b * 3 + k])
                             : make_float2((float)A, (float)B);
                ljset[o] = (fabs(A) > kQrealEps || fabs(B) > kQrealEps) ? 1 : 0;
            }
    for (auto v : ljcod)
        if (v < 1 || v > 2) return fail(QNB_ERR_ARG, "ljcod entries must be 1 or 2");
    std::vector<float4> ljpair((size_t)nt * nt);
    for (int a = 0; a < nt; ++a)
        for (int b = 0; b < nt; ++b) {
            int code = t->ljcod[a * nt + b];
            float2 p1 = ljf[((size_t)(code - 1) * nt + a) * nt + b], p3 = ljf[((size_t)2 * nt + a) * nt + b];
            ljpair[(size_t)a * nt + b] = make_float4(p1.x, p1.y, p3.x, p3.y);
        }
    TRY(c->upload((float4**)&m.ljpair, ljpair));
    {   // plain solute partners (see DevModel::gtmask)
        m.geom = t->ivdw_rule == 1 ? 1 : 0;
        std::vector<ulonglong2> gtm(std::max(1, t->ncgp_solute), make_ulonglong2(0ull, 0ull));
        for (int g = 0; g < t->ncgp_solute; ++g) {
            if (nt > 128) {   // every partner takes the general path
                gtm[g] = make_ulonglong2(~0ull, ~0ull);
                continue;
            }
            for (int a = gslot[g]; a < gslot[g + 1]; ++a) {
                int i = gatom[a];
                if (iqatom[i] >= 0) continue;
                for (int b = 0; b < nt; ++b)
                    if (t->ljcod[t->iac[i] * nt + b] != 1) {
                        if (b < 64) gtm[g].x |= 1ull << b;
                        else gtm[g].y |= 1ull << (b - 64);
                    }
            }
        }
        std::vector<float2> f1(std::max(1, natom));
        for (int i = 0; i < natom; ++i)
            f1[i] = make_float2((float)t->avdw[t->iac[i] * 3], (float)t->bvdw[t->iac[i] * 3]);
        TRY(c->upload((ulonglong2**)&m.gtmask, gtm));
        TRY(c->upload((float2**)&m.ljf1, f1));
    }
    TRY(c->upload((double2**)&m.lj, lj));
    TRY(c->upload((float2**)&m.ljf, ljf));
    TRY(c->upload((uint8_t**)&m.ljset, ljset));
    TRY(c->upload((uint8_t**)&m.ljcod, ljcod));

    // solvent template: types and charges of the first molecule
    // (aLJ_solv/bLJ_solv/chg_solv, src/simprep.f90:3616-3621) and ww_precomp
    std::vector<uint8_t> heavy_solv(kMaxSolv, 0);
    c->h_heavy.assign(t->natom, 1);
    if (t->heavy)
        for (int i = 0; i < t->natom; ++i) c->h_heavy[i] = t->heavy[i] ? 1 : 0;
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
    // solvent atoms without LJ against every type (SPC hydrogens): their
    // solute pairs reduce to the Coulomb term exactly
    m.wlj_mask = 0;
    if (t->nwat > 0)
        for (int a = 0; a < sa; ++a)
            for (int b = 0; b < nt; ++b) {
                float4 p = ljpair[(size_t)b * nt + m.wtype[a]];
                if (p.x != 0.f || p.y != 0.f) m.wlj_mask |= 1u << a;
            }

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
    std::vector<uint8_t> qp_set(qp_tab.size(), 0);
    if (nq > 0)
        for (int ig = 0; ig < ns; ++ig) {
            if (qnear[ig]) continue;
            for (int jq = 0; jq < nq; ++jq) {
                int vdw = t->ljcod[t->iac[ig] * nt + t->iac[t->iqseq[jq]]];
                for (int s = 0; s < S; ++s) {
                    if (QC(s, ig, jq) == 4) vdw = 3;   // kept for later states, as the reference does
                    int set;
                    qp_tab[((size_t)ig * nq + jq) * S + s] = qp_values(jq, ig, s, vdw, &set);
                    qp_set[((size_t)ig * nq + jq) * S + s] = (uint8_t)set;
                }
            }
        }
    // adjoint factors of qp pairs: charge factor crg_j (x el14 for 1-4) and
    // the LJ chain factors when the Q side uses its code-1 factor
    auto q_side_code1 = [&](int vdw) { return t->qvdw_flag ? (vdw == 1 || vdw == 2) : (vdw == 1); };
    // the Q atom's code-1 factors in state s
    auto q_code1 = [&](int iq, int s2, double* qa, double* qb) {
        if (t->qvdw_flag) {
            *qa = t->qavdw[QIAC(iq, s2) * 3];
            *qb = t->qbvdw[QIAC(iq, s2) * 3];
        } else {
            *qa = t->avdw[t->iac[t->iqseq[iq]] * 3];
            *qb = t->bvdw[t->iac[t->iqseq[iq]] * 3];
        }
    };
    // d/d(qa), d/d(qb) of A u^2 - B u for the Q side (qa, qb) against (ea, eb)
    auto lj_chain = [&](double qa, double qb, double ea, double eb, QAdjF* f) {
        if (t->ivdw_rule == 1) {
            f->a2 = ea; f->a1 = 0.0; f->b2 = 0.0; f->b1 = -eb;
        } else {
            double S1 = qa + ea, S5 = S1 * S1 * S1 * S1 * S1, S6 = S5 * S1, tB = qb * eb;
            f->a2 = 12.0 * S6 * S5 * tB; f->a1 = -12.0 * S5 * tB;
            f->b2 = S6 * S6 * eb;        f->b1 = -2.0 * S6 * eb;
        }
    };
    std::vector<QAdjF> qp_adj(qp_tab.size());
    if (nq > 0)
        for (int ig = 0; ig < ns; ++ig) {
            if (qnear[ig]) continue;
            for (int jq = 0; jq < nq; ++jq) {
                int vdw = t->ljcod[t->iac[ig] * nt + t->iac[t->iqseq[jq]]];
                for (int s2 = 0; s2 < S; ++s2) {
                    if (QC(s2, ig, jq) == 4) vdw = 3;
                    QAdjF f{};
                    f.c = t->qq_use_library_charges ? 0.0 : t->crg[ig] * (vdw == 3 ? t->el14_scale : 1.0);
                    if (q_side_code1(vdw)) {
                        double qa, qb;
                        q_code1(jq, s2, &qa, &qb);
                        lj_chain(qa, qb, t->avdw[t->iac[ig] * 3 + vdw - 1], t->bvdw[t->iac[ig] * 3 + vdw - 1], &f);
                    }
                    qp_adj[((size_t)ig * nq + jq) * S + s2] = f;
                }
            }
        }
    TRY(c->upload((QAdjF**)&m.qp_adj, qp_adj));
    std::vector<QParF> qp_tabf(qp_tab.size());
    for (size_t k = 0; k < qp_tab.size(); ++k)
        qp_tabf[k] = QParF{(float)qp_tab[k].A, (float)qp_tab[k].B, (float)qp_tab[k].el, (float)qp_tab[k].sc};
    TRY(c->upload((QPar**)&m.qp_tab, qp_tab));
    TRY(c->upload((QParF**)&m.qp_tabf, qp_tabf));
    // the same FP32 table ordered [Q atom][solute atom][state]: lanes that
    // take consecutive solute atoms read consecutive entries
    std::vector<QParF> qp_tabft(qp_tabf.size());
    for (int jq = 0; jq < nq; ++jq)
        for (int ig = 0; ig < ns; ++ig)
            for (int s2 = 0; s2 < S; ++s2)
                qp_tabft[((size_t)jq * ns + ig) * S + s2] = qp_tabf[((size_t)ig * nq + jq) * S + s2];
    TRY(c->upload((QParF**)&m.qp_tabft, qp_tabft));

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
    std::vector<QAdjF> qw_adj(qw_tab.size());
    if (nq > 0 && t->nwat > 0)
        for (int iq = 0; iq < nq; ++iq)
            for (int a = 0; a < sa; ++a) {
                int tw = t->iac[ns + a];
                int vdw = t->ljcod[tw * nt + t->iac[t->iqseq[iq]]];
                for (int s2 = 0; s2 < S; ++s2) {
                    QAdjF f{};
                    f.c = t->qq_use_library_charges ? 0.0 : t->crg[ns + a];
                    if (q_side_code1(vdw)) {
                        double qa, qb;
                        q_code1(iq, s2, &qa, &qb);
                        lj_chain(qa, qb, t->avdw[tw * 3 + vdw - 1], t->bvdw[tw * 3 + vdw - 1], &f);
                    }
                    qw_adj[((size_t)iq * sa + a) * S + s2] = f;
                }
            }
    TRY(c->upload((QAdjF**)&m.qw_adj, qw_adj));
    std::vector<QParF> qw_tabf(qw_tab.size());
    for (size_t k = 0; k < qw_tab.size(); ++k)
        qw_tabf[k] = QParF{(float)qw_tab[k].A, (float)qw_tab[k].B, (float)qw_tab[k].el, (float)qw_tab[k].sc};
    TRY(c->upload((QPar**)&m.qw_tab, qw_tab));
    TRY(c->upload((QParF**)&m.qw_tabf, qw_tabf));

    // static lists: qq_int_comp + nbqqlist (src/simprep.f90:3152-3268,
    // src/nonbondene.f90:3231-3282)
    std::vector<QQEntry> qq;
    std::vector<QQAdj> qadj;
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
                {
                    double f14 = vdw == 3 ? t->el14_scale : 1.0;
                    bool lib = t->qq_use_library_charges != 0;
                    QQAdj f{iq, jq, s, 0, QAdjF{}, QAdjF{}};
                    f.fi.c = lib ? 0.0 : QCRG(jq, s) * els * f14;
                    f.fj.c = lib ? 0.0 : QCRG(iq, s) * els * f14;
                    if (vdw == 1) {   // both sides' code-1 factors
                        double ai, bi, aj, bj;
                        q_code1(iq, s, &ai, &bi);
                        q_code1(jq, s, &aj, &bj);
                        lj_chain(ai, bi, aj, bj, &f.fi);
                        lj_chain(aj, bj, ai, bi, &f.fj);
                    }
                    qadj.push_back(f);
                }
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
                {
                    QQAdj f{iq, -1, s, 0, QAdjF{}, QAdjF{}};
                    f.fi.c = t->qq_use_library_charges ? 0.0 : t->crg[ja] * (vdw == 3 ? t->el14_scale : 1.0);
                    if (q_side_code1(vdw)) {
                        double qa, qb;
                        q_code1(iq, s, &qa, &qb);
                        lj_chain(qa, qb, t->avdw[t->iac[ja] * 3 + vdw - 1], t->bvdw[t->iac[ja] * 3 + vdw - 1], &f.fi);
                    }
                    qadj.push_back(f);
                }
            }
        }
    }
    c->nqq = (int)qq.size();
    c->nqq_qq = nqq_qq;
    {   // parameter sources of the listed pair sets (monitors, group contributions)
        auto& ps = c->psrc;
        ps.qq = qq;
        ps.qp = qp_tab;
        ps.qp_set = qp_set;
        ps.qnear = qnear;
        ps.iqatom = iqatom;
        ps.iqseq.assign(t->iqseq, t->iqseq + nq);
        ps.crg.assign(t->crg, t->crg + natom);
        ps.iac.assign(t->iac, t->iac + natom);
        ps.lj = lj;
        ps.ljcod = ljcod;
        ps.nt = nt;
        ps.el14 = t->el14_scale;
        ps.special.clear();
        for (const Sp& q : sp) ps.special.emplace_back((long long)q.i * natom + q.j, q.k);
    }
    TRY(c->upload(&c->st_qq, qq));
    std::vector<float4> qqf(qq.size());
    for (size_t k = 0; k < qq.size(); ++k)
        qqf[k] = make_float4((float)qq[k].A, (float)qq[k].B, (float)qq[k].el, (float)qq[k].sc);
    TRY(c->upload(&c->st_qqf, qqf));
    TRY(c->upload((QQAdj**)&m.qq_adj, qadj));
    return QNB_OK;
}

int upload_states(qnb_context* c) {
    ++c->epoch;   // capacities / buffers may have changed: captured graphs are stale
    CU(cudaMemcpyAsync(c->d_states, c->st.data(), sizeof(DevState) * c->nwin, cudaMemcpyHostToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return QNB_OK;
}

int alloc_state(qnb_context* c) {
    const DevModel& m = c->m;
    const int W = c->nwin;
    const size_t n3 = 3 * (size_t)m.natom;
    c->st.assign(W, DevState{});
    TRY(c->alloc(&c->x_all, n3 * W));
    TRY(c->alloc(&c->d_all, n3 * W));
    TRY(c->alloc(&c->e_all, (size_t)kNumE * W));
    TRY(c->alloc(&c->efix_all, (size_t)kNumE * W));
    TRY(c->alloc(&c->cnt_all, (size_t)C_NUM * W));
    CU(cudaMemset(c->cnt_all, 0, sizeof(int) * C_NUM * W));
    CU(cudaMemset(c->d_all, 0, sizeof(double) * n3 * W));
    const double rho = 0.04;   // generous water density (molecules / A^3)
    int64_t per_w = (int64_t)(4.0 / 3.0 * M_PI * 1000.0 * rho) + 64;
    std::vector<double> lam(std::max(1, m.S), 1.0);
    std::vector<float> lamf((size_t)kMaxStates * W, 1.0f);
    TRY(c->upload(&c->lambdaf_all, lamf));
    for (int w = 0; w < W; ++w) {
        DevState& s = c->st[w];
        s.x = c->x_all + n3 * w;
        s.d = c->d_all + n3 * w;
        TRY(c->alloc(&s.xq, (size_t)m.natom));
        TRY(c->alloc(&s.frow, (size_t)3 * m.natom));
        CU(cudaMemset(s.frow, 0, sizeof(float) * 3 * m.natom));   // atoms outside every row stay 0
        TRY(c->alloc(&s.fq, (size_t)3 * m.natom));
        CU(cudaMemset(s.fq, 0, sizeof(float) * 3 * m.natom));     // atoms outside the Q lists stay 0
        TRY(c->alloc(&s.fix, n3));
        s.e = c->e_all + (size_t)kNumE * w;
        s.efix = c->efix_all + (size_t)kNumE * w;
        TRY(c->alloc(&s.lambda, (size_t)std::max(1, m.S)));
        TRY(c->alloc(&s.lrf, (size_t)std::max(1, m.ncgp) * kLrfLen));
        if (c->mixed && c->use_lrf)
            TRY(c->alloc(&s.lrf_part, (size_t)kLrfSplitMax * std::max(1, m.ncgp) * kLrfMoments));
        s.cnt = c->cnt_all + (size_t)C_NUM * w;
        TRY(c->alloc(&s.theta, (size_t)std::max(1, m.nwat)));
        TRY(c->alloc(&s.rkey, (size_t)std::max(1, m.nwat)));
        TRY(c->alloc(&s.wvec, (size_t)8 * std::max(1, m.nwat)));
        TRY(c->alloc(&s.shell, (size_t)std::max(1, m.nwat)));
        TRY(c->alloc(&s.rank, (size_t)std::max(1, m.nwat)));
        TRY(c->alloc(&s.n_insh, (size_t)kMaxShell));
        TRY(c->alloc(&s.wstate, (size_t)3 * kMaxShell));
        TRY(c->alloc(&s.shell_tsum, (size_t)kMaxShell));
        TRY(c->alloc(&s.theta_sorted, (size_t)kMaxShell * std::max(1, m.nwat)));
        TRY(c->alloc(&s.adj, (size_t)3 * std::max(1, m.nqat * m.S)));
        TRY(c->alloc(&s.shell_list, (size_t)kMaxShell * std::max(1, m.nwat)));
        CU(cudaMemset(s.fix, 0, sizeof(unsigned long long) * n3));
        CU(cudaMemset(s.wstate, 0, sizeof(double) * 3 * kMaxShell));
        CU(cudaMemset(s.lrf, 0, sizeof(double) * std::max(1, m.ncgp) * kLrfLen));
        CU(cudaMemcpy(s.lambda, lam.data(), lam.size() * sizeof(double), cudaMemcpyHostToDevice));
        TRY(ensure_cap(c, &s.ww, &s.cap_ww, std::max<int64_t>(1024, (int64_t)m.nwat * per_w / 2)));
        TRY(ensure_cap(c, &s.pw, &s.cap_pw, std::max<int64_t>(1024, (int64_t)m.nat_solute * per_w)));
        TRY(ensure_cap(c, &s.pp, &s.cap_pp, std::max<int64_t>(1024, (int64_t)m.nat_solute * 256)));
        TRY(ensure_cap(c, &s.ppg, &s.cap_ppg, std::max<int64_t>(1024, (int64_t)m.ncgp_solute * 96)));
        TRY(ensure_cap(c, &s.qp, &s.cap_qp, std::max<int64_t>(1024, (int64_t)m.nat_solute)));
        TRY(ensure_cap(c, &s.qw, &s.cap_qw, std::max<int64_t>(1024, (int64_t)m.nwat)));
        if (c->mixed) {
            s.cap_gp = 256;
            s.cap_gf = 1024;
            s.cap_gw = 256;
            s.cap_rww = 256;
            s.cap_wg = 192;
            TRY(c->alloc(&s.row_gp, (size_t)std::max(1, m.ncgp_solute) * s.cap_gp));
            TRY(c->alloc(&s.row_gf, (size_t)std::max(1, m.ncgp_solute) * s.cap_gf));
            TRY(c->alloc(&s.cnt_gf, (size_t)std::max(1, m.ncgp_solute)));
            TRY(c->alloc(&s.row_gw, (size_t)std::max(1, m.ncgp_solute) * s.cap_gw));
            TRY(c->alloc(&s.row_ww, (size_t)std::max(1, m.nwat) * s.cap_rww));
            TRY(c->alloc(&s.row_wg, (size_t)std::max(1, m.nwat) * s.cap_wg));
            TRY(c->alloc(&s.cnt_gp, (size_t)std::max(1, m.ncgp_solute)));
            TRY(c->alloc(&s.cnt_gw, (size_t)std::max(1, m.ncgp_solute)));
            TRY(c->alloc(&s.cnt_ww, (size_t)std::max(1, m.nwat)));
            TRY(c->alloc(&s.cnt_wg, (size_t)std::max(1, m.nwat)));
            TRY(c->alloc(&s.x_build, n3));
            if (!m.any_atom) {
                s.cap_cells = kCellCap;
                TRY(c->alloc(&s.grid, (size_t)1));
                TRY(c->alloc(&s.cend_s, (size_t)s.cap_cells));
                TRY(c->alloc(&s.cend_w, (size_t)s.cap_cells));
                TRY(c->alloc(&s.bin_s, (size_t)std::max(1, m.ncgp_solute)));
                TRY(c->alloc(&s.bin_w, (size_t)std::max(1, m.nwat)));
            }
        }
        s.qq = c->st_qq;
        s.qqf = c->st_qqf;
        s.lambdaf = c->lambdaf_all + (size_t)kMaxStates * w;
        s.nqq = c->nqq;
        s.nqq_qq = c->nqq_qq;
    }
    TRY(c->alloc(&c->d_states, (size_t)W));
    TRY(c->alloc(&c->d_diag, (size_t)1));
    c->counts.assign((size_t)W * C_NUM, 0);
    CU(cudaMallocHost((void**)&c->h_stage, sizeof(double) * std::max(3 * m.natom, 64)));
    CU(cudaMallocHost((void**)&c->h_e, sizeof(double) * 2 * kNumE * W));
    return upload_states(c);
}

int zero_acc(qnb_context* c, int nw) {
    CU(cudaMemsetAsync(c->e_all, 0, sizeof(double) * kNumE * nw, c->stream));
    CU(cudaMemsetAsync(c->efix_all, 0, sizeof(unsigned long long) * kNumE * nw, c->stream));
    return QNB_OK;
}

// energies of the first nw windows: out[w*kNumE + k] (FP64 slots + fixed-point slots)
// the energy records of nw windows copied to the pinned h_e (enqueued)
int enqueue_energies(qnb_context* c, int nw) {
    CU(cudaMemcpyAsync(c->h_e, c->e_all, sizeof(double) * kNumE * nw, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(c->h_e + (size_t)kNumE * c->nwin, c->efix_all, sizeof(double) * kNumE * nw,
                       cudaMemcpyDeviceToHost, c->stream));
    return QNB_OK;
}
// after the copies have landed: FP64 part + fixed-point part per slot
void finish_energies(const qnb_context* c, int nw, double* out) {
    const long long* fx = (const long long*)(c->h_e + (size_t)kNumE * c->nwin);
    for (int k = 0; k < kNumE * nw; ++k) out[k] = c->h_e[k] + (double)fx[k] * (1.0 / kFix);
}
int read_energies(qnb_context* c, int nw, double* out) {
    TRY(enqueue_energies(c, nw));
    CU(cudaStreamSynchronize(c->stream));
    finish_energies(c, nw, out);
    return QNB_OK;
}

int stage_x(qnb_context* c, const double* x) {
    size_t n = 3 * (size_t)c->natom;
    memcpy(c->h_stage, x, n * sizeof(double));
    CU(cudaMemcpyAsync(c->st[0].x, c->h_stage, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    return QNB_OK;
}

// window 0's device gradient -> added into the caller's d; device gradient cleared
int unstage_d(qnb_context* c, double* d) {
    size_t n = 3 * (size_t)c->natom;
    if (c->mixed) {
        launch_apply_fixed(c->one(), c->rows_pending ? 1 : 0, c->qenv_pending ? 1 : 0);
        c->rows_pending = c->qenv_pending = false;
        c->launches++;
        TRY(check_launch());
    }
    CU(cudaMemcpyAsync(c->h_stage, c->st[0].d, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemsetAsync(c->st[0].d, 0, n * sizeof(double), c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (size_t k = 0; k < n; ++k) d[k] += c->h_stage[k];
    return QNB_OK;
}

// grows the lists of every window to at least the sizes the last build counted
int grow_lists(qnb_context* c, bool* grew, bool* do_qp, bool* do_qw) {
    *grew = false;
    int64_t need[C_NUM] = {0};
    for (int w = 0; w < c->nwin; ++w)
        for (int k = 0; k < C_NUM; ++k) need[k] = std::max<int64_t>(need[k], c->counts[w * C_NUM + k]);
    DevState& s0 = c->st[0];
    struct G {
        int k;
        int64_t cap;
    } gs[] = {{C_WW, s0.cap_ww}, {C_PW, s0.cap_pw}, {C_PP, s0.cap_pp}, {C_PPG, s0.cap_ppg},
              {C_QP, s0.cap_qp}, {C_QW, s0.cap_qw}};
    for (auto& g : gs) {
        if (need[g.k] <= g.cap) continue;
        int64_t n = need[g.k] * 5 / 4 + 1024;
        for (int w = 0; w < c->nwin; ++w) {
            DevState& s = c->st[w];
            switch (g.k) {
                case C_WW: TRY(ensure_cap(c, &s.ww, &s.cap_ww, n)); break;
                case C_PW: TRY(ensure_cap(c, &s.pw, &s.cap_pw, n)); break;
                case C_PP: TRY(ensure_cap(c, &s.pp, &s.cap_pp, n)); break;
                case C_PPG: TRY(ensure_cap(c, &s.ppg, &s.cap_ppg, n)); break;
                case C_QP: TRY(ensure_cap(c, &s.qp, &s.cap_qp, n)); *do_qp = true; break;
                case C_QW: TRY(ensure_cap(c, &s.qw, &s.cap_qw, n)); *do_qw = true; break;
            }
        }
        *grew = true;
    }
    if (c->mixed) {
        struct R {
            int k;
            int* cap;
            int** row;
            int nrows;
        };
        for (int w = 0; w < c->nwin; ++w) {
            DevState& s = c->st[w];
            if (need[C_RGP] > s.cap_gp) {
                int cap = ((int)(need[C_RGP] + need[C_RGP] / 4 + 32) + 3) & ~3;   // 16-byte row starts
                c->release(s.row_gp);
                s.row_gp = nullptr;
                TRY(c->alloc(&s.row_gp, (size_t)std::max(1, c->ncgp_solute) * cap));
                s.cap_gp = cap;
                *grew = true;
            }
            R rs[] = {{C_RGF, &s.cap_gf, &s.row_gf, c->ncgp_solute}, {C_RGW, &s.cap_gw, &s.row_gw, c->ncgp_solute},
                      {C_RWW, &s.cap_rww, &s.row_ww, c->nwat}, {C_RWG, &s.cap_wg, &s.row_wg, c->nwat}};
            for (auto& r : rs) {
                if (need[r.k] <= *r.cap) continue;
                int cap = ((int)(need[r.k] + need[r.k] / 4 + 32) + 3) & ~3;   // 16-byte row starts
                c->release(*r.row);
                *r.row = nullptr;
                TRY(c->alloc(r.row, (size_t)std::max(1, r.nrows) * cap));
                *r.cap = cap;
                *grew = true;
            }
        }
    }
    if (*grew) TRY(upload_states(c));
    return QNB_OK;
}

int build_lists(qnb_context* c, const Cut& cut, int nw) {
    Launch L = nw == 1 ? c->one() : c->all();
    bool do_qp = !(c->qp_done && cut.rcq2 > c->rexcl_o2);   // src/nonbondene.f90:3678
    bool do_qw = !(c->qw_done && cut.rcq2 > c->rexcl_o2);   // src/nonbondene.f90:3889
    if (c->m.box) {
        // the minimum image needs every cut-off within half the shortest box edge
        double h = 0.5 * std::min(c->m.boxl[0], std::min(c->m.boxl[1], c->m.boxl[2]));
        if (cut.rcpp2 > h * h || cut.rcpw2 > h * h || cut.rcww2 > h * h || cut.rcq2 > h * h)
            return fail(QNB_ERR_ARG, "periodic box: cut-offs must not exceed half the box (%.3f A)", h);
        do_qp = do_qw = true;
    }
    for (int attempt = 0; attempt < 4; ++attempt) {
        unsigned keep = (do_qp ? 0u : 1u << C_QP) | (do_qw ? 0u : 1u << C_QW);   // everything else restarts
        launch_reset_counts(L, keep);
        int nl = 2;   // reset + pack
        timed(c, K_BUILD, [&] {
            launch_pack(L);
            if (c->use_lrf) launch_group_centres(L), ++nl;
        });
        // the LRF accumulation (needs the packed coordinates and the group
        // centres only) runs on the second stream beside the list builds
        if (c->use_lrf) {
            CU(cudaEventRecord(c->ev_fork, c->stream));
            CU(cudaStreamWaitEvent(c->stream2, c->ev_fork, 0));
            Launch L2{L.m, L.s0, L.ds, L.nwin, c->stream2, L.tu};
            timed_on(c, c->stream2, K_LRF_BUILD, [&] { nl += launch_lrf_accumulate(L2, cut, c->mixed, c->d_lrf_src); });
            CU(cudaEventRecord(c->ev_join, c->stream2));
        }
        timed(c, K_BUILD, [&] {
            if (c->m.box) {
                // the mixed form's box path builds the gather rows (switch
                // atoms, minimum image); the Q lists keep the box builder
                if (c->m.box_rows) nl += launch_build_rows(L, cut);
                launch_build_box(L, cut, c->d_qnear, !c->m.box_rows), nl += c->m.box_rows ? 1 : 3;
            } else if (c->mixed) {
                nl += launch_build_rows(L, cut);
            } else {
                launch_build_pp(L, cut), nl += 2;
                launch_build_pw(L, cut), ++nl;
                launch_build_ww(L, cut), ++nl;
            }
            if (!c->m.box) {
                if (do_qp) launch_build_qp(L, c->d_qnear, cut.rcq2), ++nl;
                if (do_qw) launch_build_qw(L, cut), ++nl;
            }
            if (c->mixed && (do_qp || do_qw)) launch_clear_fq(L), ++nl;   // atoms may leave the Q lists
        });
        c->launches += nl;
        if (c->use_lrf) CU(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
        TRY(check_launch());
        CU(cudaMemcpyAsync(c->counts.data(), c->cnt_all, sizeof(int) * C_NUM * nw, cudaMemcpyDeviceToHost,
                           c->stream));
        CU(cudaStreamSynchronize(c->stream));
        bool grew = false;
        TRY(grow_lists(c, &grew, &do_qp, &do_qw));
        if (!grew) {
            if (do_qp) c->qp_done = true;
            if (do_qw) c->qw_done = true;
            c->lists_built = true;
            c->last_cut = cut;
            c->last_build_nw = nw;
            if (c->mixed) {   // keep window 0's build coordinates for list inspection
                CU(cudaMemcpyAsync(c->st[0].x_build, c->st[0].x, sizeof(double) * 3 * c->natom,
                                   cudaMemcpyDeviceToDevice, c->stream));
                c->diag_valid = false;
            }
            return QNB_OK;
        }
    }
    return fail(QNB_ERR_CAPACITY, "pair lists kept overflowing");
}

// side: the caller's further terms of the step (qq, bonded, restraints,
// watpol), enqueued on the Launch it is given
using SideWork = std::function<int(const Launch&)>;

int compute_nonbond(qnb_context* c, int md, int nw, const SideWork& side = SideWork()) {
    if (!c->lists_built) return fail(QNB_ERR_STATE, "pair lists not built");
    Launch L = nw == 1 ? c->one() : c->all();
    int mx = c->mixed, nl = 0;
    if (mx) {
        timed(c, K_PACK, [&] { launch_pack(L); });
        ++nl;
    }
    if (mx && (!c->m.box || c->m.box_rows)) {
        const bool br = c->branches;
        // three branches after the pack (every sum is fixed point, so the
        // result does not depend on their interleaving); src/potene.f90:340-379
        // for the nonbonded terms' meaning (in a box 326-343: the rows at each
        // unit pair's image, the box Q kernels)
        Launch LB = L, LC = L;
        if (br) {
            CU(cudaEventRecord(c->ev_pk, c->stream));
            CU(cudaStreamWaitEvent(c->stream2, c->ev_pk, 0));
            CU(cudaStreamWaitEvent(c->stream3, c->ev_pk, 0));
            LB.st = c->stream2;
            LC.st = c->stream3;
        }
        // rows: pp + the solute side of pw on the main stream, ww + the water
        // side of pw first on the third branch (each row adds its energies to
        // the window's fixed-point slots itself)
        if (md) {
            if (c->m.natom > c->m.nat_solute) timed_on(c, LC.st, K_WW, [&] { launch_rows_water(LC); }), ++nl;
            timed(c, K_PP, [&] { launch_rows_solute(L, c->maxg); });   // the class times the solute rows alone
            ++nl;
            c->rows_pending = true;   // frow holds this evaluation's row gradients
        }
        // Q environment, solvent internal pairs, LRF Taylor terms
        if (c->m.box) {
            int nb = 0;
            timed_on(c, LB.st, K_QW, [&] { nb = launch_box_nonbond(LB, md, mx, c->d_iwhich, c->last_cut.rcq2, 0); });
            nl += nb;
            c->qenv_pending = true;   // the box Q terms store the environment atoms' gradients in fq
            if (md && c->nsi) timed_on(c, LB.st, K_WW, [&] { launch_solvent_internal(LB, c->d_si, c->d_sip, c->nsi, mx); }), ++nl;
        } else {
            if (c->m.natom > c->m.nat_solute) {
                timed_on(c, LB.st, K_QW, [&] { launch_qw(LB, mx); }), ++nl;
                if (md && c->nsi) timed_on(c, LB.st, K_WW, [&] { launch_solvent_internal(LB, c->d_si, c->d_sip, c->nsi, mx); }), ++nl;
            }
            timed_on(c, LB.st, K_QP, [&] { launch_qp(LB, mx); }), ++nl;
            c->qenv_pending = true;   // fq holds this evaluation's Q-environment gradients
        }
        if (c->use_lrf && md) timed_on(c, LB.st, K_LRF_TAYLOR, [&] { launch_lrf_taylor(LB, c->d_iwhich, mx); }), ++nl;
        // the caller's further terms
        int rc = side ? side(LC) : QNB_OK;
        if (br) {
            CU(cudaEventRecord(c->ev_jb, c->stream2));
            CU(cudaEventRecord(c->ev_jc, c->stream3));
            CU(cudaStreamWaitEvent(c->stream, c->ev_jb, 0));
            CU(cudaStreamWaitEvent(c->stream, c->ev_jc, 0));
        }
        c->launches += nl;
        TRY(rc);
        return check_launch();
    }
    if (c->m.box) {   // periodic box: the *_box routines, src/potene.f90:326-343
        int nb = 0;
        timed(c, K_PP, [&] { nb = launch_box_nonbond(L, md, mx, c->d_iwhich, c->last_cut.rcq2, 1); });
        if (mx) c->qenv_pending = true;   // the box Q terms store the environment atoms' gradients in fq
        // src/potene.f90:326-339 and 373-377: solvent internal pairs, then the LRF Taylor terms
        if (md && c->nsi) timed(c, K_WW, [&] { launch_solvent_internal(L, c->d_si, c->d_sip, c->nsi, mx); }), ++nl;
        if (c->use_lrf && md) timed(c, K_LRF_TAYLOR, [&] { launch_lrf_taylor(L, c->d_iwhich, mx); }), ++nl;
        c->launches += nl + nb;
        if (side) TRY(side(L));
        return check_launch();
    }
    // call order of pot_energy_nonbonds, src/potene.f90:340-379
    if (mx) {
        // gather rows: water rows carry ww + the water side of pw, solute
        // group rows pp + the solute side of pw
        if (c->m.natom > c->m.nat_solute) {
            if (md) timed(c, K_WW, [&] { launch_rows_water(L); }), ++nl;
            timed(c, K_QW, [&] { launch_qw(L, mx); }), ++nl;
            // src/potene.f90:361-366
            if (md && c->nsi) timed(c, K_WW, [&] { launch_solvent_internal(L, c->d_si, c->d_sip, c->nsi, mx); }), ++nl;
        }
        if (md) {
            timed(c, K_PP, [&] { launch_rows_solute(L, c->maxg); });
            ++nl;
            c->rows_pending = true;   // frow holds this evaluation's row gradients
        }
    } else {
        if (c->m.natom > c->m.nat_solute) {
            if (md) timed(c, K_WW, [&] { launch_ww(L, mx); }), ++nl;
            timed(c, K_QW, [&] { launch_qw(L, mx); }), ++nl;
            if (md && c->nsi) timed(c, K_WW, [&] { launch_solvent_internal(L, c->d_si, c->d_sip, c->nsi, mx); }), ++nl;
            if (md) timed(c, K_PW, [&] { launch_pw(L, mx); }), ++nl;
        }
        if (md) timed(c, K_PP, [&] { launch_pp(L, mx); }), ++nl;
    }
    timed(c, K_QP, [&] { launch_qp(L, mx); }), ++nl;
    if (mx) c->qenv_pending = true;   // fq holds this evaluation's Q-environment gradients
    if (c->use_lrf && md) {
        timed(c, K_LRF_TAYLOR, [&] { launch_lrf_taylor(L, c->d_iwhich, mx); });
        ++nl;
    }
    c->launches += nl;
    if (side) TRY(side(L));
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

// mixed form: the inspection entry points report the reference's atom-pair
// lists; they are built on demand from window 0's build coordinates with the
// same exact selection as the rows
int ensure_half_lists(qnb_context* c) {
    // the FP64 form's builders (and the box builders of the box path without
    // rows) already write the half lists
    if (!c->mixed || (c->m.box && !c->m.box_rows) || c->diag_valid || !c->lists_built) return QNB_OK;
    for (int attempt = 0; attempt < 4; ++attempt) {
        DevState tmp = c->st[0];
        tmp.x = c->st[0].x_build;
        CU(cudaMemcpyAsync(c->d_diag, &tmp, sizeof(DevState), cudaMemcpyHostToDevice, c->stream));
        Launch L{c->m, tmp, c->d_diag, 1, c->stream, c->tune};
        unsigned keep = ~((1u << C_WW) | (1u << C_PW) | (1u << C_PP) | (1u << C_PP14) | (1u << C_PPG));
        launch_reset_counts(L, keep);
        launch_pack(L);
        if (c->m.box) {
            launch_build_box_pairs(L, c->last_cut);
        } else {
            launch_build_pp(L, c->last_cut);
            launch_build_pw(L, c->last_cut);
            launch_build_ww(L, c->last_cut);
        }
        TRY(check_launch());
        CU(cudaMemcpyAsync(c->counts.data(), c->cnt_all, sizeof(int) * C_NUM, cudaMemcpyDeviceToHost, c->stream));
        CU(cudaStreamSynchronize(c->stream));
        bool grew = false, dq = false, dw = false;
        TRY(grow_lists(c, &grew, &dq, &dw));
        if (!grew) {
            c->diag_valid = true;
            return QNB_OK;
        }
    }
    return fail(QNB_ERR_CAPACITY, "inspection lists kept overflowing");
}

int64_t list_pairs(const qnb_context* c, int kind) {
    int64_t sa = c->sa;
    const int* cnt = c->counts.data();   // window 0
    switch (kind) {
        case QNB_LIST_PP: return cnt[C_PP];
        case QNB_LIST_PP14: return cnt[C_PP14];
        case QNB_LIST_PW: return (int64_t)cnt[C_PW] * sa;
        case QNB_LIST_WW: return (int64_t)cnt[C_WW] * sa * sa;
        case QNB_LIST_QP: return (int64_t)cnt[C_QP] * c->nqat;
        case QNB_LIST_QW: return (int64_t)cnt[C_QW] * c->nqat * sa;
    }
    return -1;
}

}  // namespace

// =============================================================================
// C ABI
// =============================================================================
extern "C" {

const char* qnb_last_error(void) { return g_err.c_str(); }

int32_t qnb_version(void) { return 0x000300; }

int qnb_create_batch(const qnb_topology* t, const qnb_options* opt, int32_t nwin, qnb_context** out) {
    if (!t || !opt || !out) return fail(QNB_ERR_ARG, "null argument");
    *out = nullptr;
    if (nwin < 1 || nwin > 65535) return fail(QNB_ERR_ARG, "nwin must be 1..65535");
    if (t->natom <= 0 || t->nat_solute < 0 || t->nat_solute > t->natom || t->nwat < 0)
        return fail(QNB_ERR_ARG, "bad atom counts");
    if (t->natom != t->nat_solute + t->nwat * t->solv_atom) return fail(QNB_ERR_ARG, "natom != nat_solute + nwat*solv_atom");
    if (t->nstates < 0 || t->nstates > kMaxStates) return fail(QNB_ERR_UNSUPPORTED, "nstates %d > %d", t->nstates, kMaxStates);
    if (t->nqat > 64) return fail(QNB_ERR_UNSUPPORTED, "nqat %d > 64", t->nqat);
    if (t->nqat > 0 && t->nstates < 1) return fail(QNB_ERR_ARG, "Q atoms need nstates >= 1");
    if (t->iuse_switch_atom != 0 && t->iuse_switch_atom != 1) return fail(QNB_ERR_ARG, "iuse_switch_atom must be 0 or 1");
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
    c->nwin = nwin;
    c->natom = t->natom;
    c->nat_solute = t->nat_solute;
    c->nwat = t->nwat;
    c->sa = t->solv_atom;
    c->ncgp = t->ncgp;
    c->ncgp_solute = t->ncgp_solute;
    c->nqat = t->nqat;
    c->S = t->nstates;
    int rc = QNB_OK;
    if (cudaSetDevice(c->device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream3, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_pk, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_jb, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_jc, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess)
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

int qnb_create(const qnb_topology* t, const qnb_options* opt, qnb_context** out) {
    return qnb_create_batch(t, opt, 1, out);
}

int qnb_destroy(qnb_context* c) {
    if (!c) return QNB_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : c->allocs) cudaFree(p);
    for (auto& p : c->pending)
        if (!p.owned) {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
    for (auto e : c->ev_pool) cudaEventDestroy(e);
    for (auto& row : c->gslot)
        for (auto& g : row) {
            if (g.exec) cudaGraphExecDestroy(g.exec);
            for (auto& p : g.prof) {
                cudaEventDestroy(p.a);
                cudaEventDestroy(p.b);
            }
        }
    if (c->h_stage) cudaFreeHost(c->h_stage);
    if (c->h_e) cudaFreeHost(c->h_e);
    if (c->h_md_rec) cudaFreeHost(c->h_md_rec);
    if (c->stream2) cudaStreamSynchronize(c->stream2), cudaStreamDestroy(c->stream2);
    if (c->stream3) cudaStreamSynchronize(c->stream3), cudaStreamDestroy(c->stream3);
    if (c->ev_pk) cudaEventDestroy(c->ev_pk);
    if (c->ev_jb) cudaEventDestroy(c->ev_jb);
    if (c->ev_jc) cudaEventDestroy(c->ev_jc);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return QNB_OK;
}

int qnb_window_count(qnb_context* c, int32_t* n) {
    if (!c || !n) return fail(QNB_ERR_ARG, "null argument");
    *n = c->nwin;
    return QNB_OK;
}

int qnb_set_lambda_window(qnb_context* c, int32_t w, const double* lambda) {
    if (!c || (!lambda && c->S > 0)) return fail(QNB_ERR_ARG, "null argument");
    if (w < 0 || w >= c->nwin) return fail(QNB_ERR_ARG, "window %d of %d", w, c->nwin);
    if (c->S == 0) return QNB_OK;
    CU(cudaSetDevice(c->device));
    memcpy(c->h_stage, lambda, sizeof(double) * c->S);
    float* lf = reinterpret_cast<float*>(c->h_stage + c->S);   // staging holds >= 64 doubles, S <= kMaxStates
    for (int k = 0; k < c->S; ++k) lf[k] = (float)lambda[k];
    CU(cudaMemcpyAsync(c->st[w].lambda, c->h_stage, sizeof(double) * c->S, cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(c->lambdaf_all + (size_t)kMaxStates * w, lf, sizeof(float) * c->S, cudaMemcpyHostToDevice,
                       c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return QNB_OK;
}

int qnb_set_lambda(qnb_context* c, const double* lambda) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    for (int w = 0; w < c->nwin; ++w) TRY(qnb_set_lambda_window(c, w, lambda));
    return QNB_OK;
}

int qnb_make_pair_lists_dev(qnb_context* c, double Rq, double Rcq2, double RcLRF2, double Rcpp2, double Rcpw2,
                            double Rcww2) {
    (void)Rq;
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    Cut cut = make_cut(Rcq2, RcLRF2, Rcpp2, Rcpw2, Rcww2);
    return build_lists(c, cut, c->nwin);
}

int qnb_make_pair_lists(qnb_context* c, const double* x, double Rq, double Rcq2, double RcLRF2, double Rcpp2,
                        double Rcpw2, double Rcww2) {
    (void)Rq;
    if (!c || !x) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    Cut cut = make_cut(Rcq2, RcLRF2, Rcpp2, Rcpw2, Rcww2);
    return build_lists(c, cut, 1);
}

int qnb_pot_energy_nonbonds(qnb_context* c, const double* x, double* d, qnb_energies* E, qnb_qenergies* EQ,
                            int32_t md) {
    if (!c || !x || !d) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    TRY(zero_acc(c, 1));
    TRY(compute_nonbond(c, md, 1));
    TRY(unstage_d(c, d));
    std::vector<double> e(kNumE);
    TRY(read_energies(c, 1, e.data()));
    add_energies(e.data(), E, EQ, c->S);
    return QNB_OK;
}

int qnb_nonbond_qq(qnb_context* c, const double* x, double* d, qnb_qenergies* EQ) {
    if (!c || !x || !d) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    TRY(zero_acc(c, 1));
    launch_nonbond_qq(c->one(), c->mixed);
    c->launches++;
    TRY(check_launch());
    TRY(unstage_d(c, d));
    std::vector<double> e(kNumE);
    TRY(read_energies(c, 1, e.data()));
    add_energies(e.data(), nullptr, EQ, c->S);
    return QNB_OK;
}

int qnb_set_solvent_params(qnb_context* c, const qnb_solvent_params* p) {
    if (c && c->m.box) return fail(QNB_ERR_UNSUPPORTED, "solvent restraints are for the sphere, not a periodic box");
    if (!c || !p) return fail(QNB_ERR_ARG, "null argument");
    if (p->wpol_restr && (p->nwpolr_shell < 1 || p->nwpolr_shell > kMaxShell))
        return fail(QNB_ERR_ARG, "nwpolr_shell must be 1..%d", kMaxShell);
    if (p->wpol_restr && !(p->itdis >= 1.0)) return fail(QNB_ERR_ARG, "itdis must be >= 1");
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
        s.cstbf[k] = (float)p->shell_cstb[k];
    }
    s.fk_wspheref = (float)s.fk_wsphere;
    s.Dwmzf = (float)s.Dwmz;
    s.awmzf = (float)s.awmz;
    s.fkwpolf = (float)s.fkwpol;
    double ws[3 * kMaxShell] = {0};
    for (int k = 0; k < kMaxShell; ++k) ws[k] = p->theta_corr[k];
    for (int w = 0; w < c->nwin; ++w)
        CU(cudaMemcpyAsync(c->st[w].wstate, ws, sizeof(ws), cudaMemcpyHostToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    c->have_solv = true;
    ++c->epoch;   // SolventDev is passed by value: captured graphs are stale
    return QNB_OK;
}

int qnb_restrain_solvent(qnb_context* c, const double* x, double* d, double Tfree, double* E) {
    if (!c || !x || !d || !E) return fail(QNB_ERR_ARG, "null argument");
    if (!c->have_solv) return fail(QNB_ERR_STATE, "solvent parameters not set");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    TRY(zero_acc(c, 1));
    if (c->mixed) launch_pack(c->one()), c->launches++;   // the mixed kernels read the FP32 copy
    launch_restrain_solvent(c->one(), c->solv, Tfree, c->mixed, c->d_wsw, c->d_heavy_solv);
    c->launches++;
    TRY(check_launch());
    TRY(unstage_d(c, d));
    std::vector<double> e(kNumE);
    TRY(read_energies(c, 1, e.data()));
    *E += e[E_RST_RAD];
    return QNB_OK;
}

int qnb_watpol(qnb_context* c, const double* x, double* d, int32_t istep, int32_t md, double* E) {
    if (!c || !x || !d || !E) return fail(QNB_ERR_ARG, "null argument");
    if (!c->have_solv) return fail(QNB_ERR_STATE, "solvent parameters not set");
    CU(cudaSetDevice(c->device));
    TRY(stage_x(c, x));
    TRY(zero_acc(c, 1));
    if (c->mixed) launch_pack(c->one()), c->launches++;   // the mixed kernels read the FP32 copy
    c->launches += launch_watpol(c->one(), c->solv, istep, md, c->mixed);
    TRY(check_launch());
    TRY(unstage_d(c, d));
    std::vector<double> e(kNumE);
    TRY(read_energies(c, 1, e.data()));
    *E += e[E_RST_POL];
    return QNB_OK;
}

int qnb_get_watpol_state(qnb_context* c, double* theta_corr, double* avtheta, double* avn_insh) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    double ws[3 * kMaxShell];
    CU(cudaMemcpyAsync(ws, c->st[0].wstate, sizeof(ws), cudaMemcpyDeviceToHost, c->stream));
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
    CU(cudaSetDevice(c->device));
    TRY(ensure_half_lists(c));
    int64_t v = list_pairs(c, kind);
    if (v < 0) return fail(QNB_ERR_ARG, "list kind %d", kind);
    *n = v;
    return QNB_OK;
}

int qnb_export_pairs(qnb_context* c, int32_t kind, int32_t* i, int32_t* j, int64_t cap, int64_t* n) {
    if (!c || !n) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    TRY(ensure_half_lists(c));
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
    launch_export_pairs(c->all(), 0, kind, di, dj, cnt, dc);
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

int qnb_export_rows(qnb_context* c, int32_t win, int32_t kind, int32_t* row, int32_t* partner, int64_t cap,
                    int64_t* n) {
    if (!c || !n) return fail(QNB_ERR_ARG, "null argument");
    if (!c->mixed) return fail(QNB_ERR_ARG, "rows exist in the mixed form only");
    if (win < 0 || win >= c->nwin) return fail(QNB_ERR_ARG, "window %d", win);
    if (kind < QNB_ROWS_GP || kind > QNB_ROWS_WG) return fail(QNB_ERR_ARG, "row kind %d", kind);
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    const DevState& s = c->st[win];
    const bool solute = kind == QNB_ROWS_GP || kind == QNB_ROWS_GW;
    const int nrows = solute ? c->m.ncgp_solute : c->m.nwat;
    // (count array, entry array, capacity, entry stride in ints, id mask) of each part
    struct Part { const int* cnt; const int* rows; int cap; int stride; unsigned mask; };
    std::vector<Part> parts;
    if (kind == QNB_ROWS_GP) {
        parts.push_back({s.cnt_gp, reinterpret_cast<const int*>(s.row_gp), s.cap_gp, 2, 0x0fffffffu});
        parts.push_back({s.cnt_gf, s.row_gf, s.cap_gf, 1, 0xffffffffu});
    } else if (kind == QNB_ROWS_GW) {
        parts.push_back({s.cnt_gw, s.row_gw, s.cap_gw, 1, 0xffffffffu});
    } else if (kind == QNB_ROWS_WW) {
        parts.push_back({s.cnt_ww, s.row_ww, s.cap_rww, 1, 0xffffffffu});
    } else {
        parts.push_back({s.cnt_wg, s.row_wg, s.cap_wg, 1, 0xffffffffu});
    }
    std::vector<int32_t> ri, pj;
    for (const Part& p : parts) {
        if (nrows == 0 || !p.cnt || !p.rows) continue;
        std::vector<int> cnt(nrows), ent((size_t)nrows * p.cap * p.stride);
        CU(cudaMemcpy(cnt.data(), p.cnt, sizeof(int) * nrows, cudaMemcpyDeviceToHost));
        CU(cudaMemcpy(ent.data(), p.rows, sizeof(int) * ent.size(), cudaMemcpyDeviceToHost));
        for (int r = 0; r < nrows; ++r)
            for (int k = 0; k < cnt[r]; ++k) {
                ri.push_back(r);
                pj.push_back((int32_t)((unsigned)ent[((size_t)r * p.cap + k) * p.stride] & p.mask));
            }
    }
    *n = (int64_t)ri.size();
    if (*n > cap) return fail(QNB_ERR_CAPACITY, "export needs %lld entries", (long long)*n);
    if (*n && (!row || !partner)) return fail(QNB_ERR_ARG, "null output");
    std::copy(ri.begin(), ri.end(), row);
    std::copy(pj.begin(), pj.end(), partner);
    return QNB_OK;
}

int qnb_get_lrf(qnb_context* c, double* lrf) {
    if (!c || !lrf) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    CU(cudaMemcpyAsync(lrf, c->st[0].lrf, sizeof(double) * kLrfLen * c->ncgp, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return QNB_OK;
}

int qnb_device_buffers(qnb_context* c, double** x_dev, double** d_dev) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    if (x_dev) *x_dev = c->x_all;
    if (d_dev) *d_dev = c->d_all;
    return QNB_OK;
}

int qnb_upload_coordinates(qnb_context* c, const double* x_all) {
    if (!c || !x_all) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    CU(cudaMemcpyAsync(c->x_all, x_all, sizeof(double) * 3 * (size_t)c->natom * c->nwin, cudaMemcpyHostToDevice,
                       c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return QNB_OK;
}

int qnb_download_gradient(qnb_context* c, double* d_all, int32_t clear) {
    if (!c || !d_all) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    size_t n = 3 * (size_t)c->natom * c->nwin;
    CU(cudaMemcpyAsync(d_all, c->d_all, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (clear) CU(cudaMemsetAsync(c->d_all, 0, sizeof(double) * n, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return QNB_OK;
}

int qnb_stream(qnb_context* c, void** stream) {
    if (!c || !stream) return fail(QNB_ERR_ARG, "null argument");
    *stream = (void*)c->stream;
    return QNB_OK;
}

}  // extern "C"

namespace {

// One evaluation of every window (accumulators zeroed, pot_energy_nonbonds,
// nonbond_qq/qqp, restrain_solvent, watpol, gradient applied), enqueued on
// c->stream without any host synchronisation, so it can be captured.
int enqueue_compute(qnb_context* c, double Tfree, int istep) {
    Launch L = c->all();
    TRY(zero_acc(c, c->nwin));
    // the step's terms beside the nonbonded ones (their own branch in the
    // mixed form: none reads what the pair kernels write)
    auto side = [&](const Launch& S) -> int {
        const cudaStream_t st = S.st;
        timed_on(c, st, K_QQ, [&] { launch_nonbond_qq(S, c->mixed); });
        c->launches++;
        if (c->have_bonded) {
            timed_on(c, st, K_BONDED, [&] { launch_bonded(S, c->bonded, c->mixed); });
            c->launches++;
        }
        if (c->have_shell) {
            timed_on(c, st, K_RESTRAIN, [&] { launch_fix_shell(S, c->d_shell_flags, c->d_xtop, c->fk_fix, c->fk_pshell, c->mixed, c->freeze, c->md_ready ? c->md.v : nullptr); });
            c->launches++;
        }
        if (c->offd.n > 0) {
            launch_offdiag(S, c->offd);
            c->launches++;
        }
        if (c->psets.nslots > 0) {
            launch_pair_sets(S, c->psets);
            c->launches++;
        }
        if (c->have_restr) {
            timed_on(c, st, K_RESTRAIN, [&] { launch_restraints(S, c->restr, c->mixed); });
            c->launches++;
        }
        if (c->have_solv) {
            timed_on(c, st, K_RESTRAIN, [&] { launch_restrain_solvent(S, c->solv, Tfree, c->mixed, c->d_wsw, c->d_heavy_solv); });
            c->launches++;
            int nl = 0;
            timed_on(c, st, K_WATPOL, [&] { nl = launch_watpol(S, c->solv, istep, 1, c->mixed); });
            c->launches += nl;
        }
        return check_launch();
    };
    TRY(compute_nonbond(c, 1, c->nwin, side));
    if (c->mixed) {
        timed(c, K_APPLY, [&] { launch_apply_fixed(L, c->rows_pending ? 1 : 0, c->qenv_pending ? 1 : 0); });
        c->rows_pending = c->qenv_pending = false;
        c->launches++;
    }
    return check_launch();
}

// whether this step runs watpol's theta_corr update (src/nonbondene.f90:6630)
bool watpol_update_step(const qnb_context* c, int istep) {
    return c->have_solv && c->solv.wpol && c->solv.nshell > 0 && istep > 0 &&
           (istep % (int)llround(c->solv.itdis)) == 0;
}

// Captures f (which enqueues on `st`) into an instantiated graph.
template <typename F>
int capture_graph(cudaStream_t st, cudaGraphExec_t* exec, F&& f) {
    *exec = nullptr;
    CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int rc = f();
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &graph);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return fail(QNB_ERR_CUDA, "stream capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
        *exec = nullptr;
        return fail(QNB_ERR_CUDA, "graph instantiation: %s", cudaGetErrorString(e));
    }
    return QNB_OK;
}

// enqueue_compute through a cached CUDA graph: one launch per step instead
// of one per kernel.  A graph is captured per variant (watpol update step or
// not; profiled or not) and re-captured when the launch geometry (list
// capacities, solvent parameters) or Tfree changed.  A profiled graph holds
// event-record nodes around each kernel class; after every replay its event
// pairs are queued for collect_profile, which must run (qnb_profile_collect)
// before the next replay re-records them -- run_compute collects first if the
// caller did not.
int run_compute(qnb_context* c, double Tfree, int istep) {
    if (!c->use_graphs) return enqueue_compute(c, Tfree, istep);
    const int prof = c->profiling ? 1 : 0;
    auto& g = c->gslot[watpol_update_step(c, istep) ? 1 : 0][prof];
    for (auto& p : c->pending)
        if (p.owned) {   // an earlier replay's times were not collected yet
            collect_profile(c);
            break;
        }
    const unsigned mask = prof ? c->prof_mask : 0u;
    if (!g.exec || g.key_epoch != c->epoch || g.key_tfree != Tfree || g.key_mask != mask) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        for (auto& p : g.prof) {
            cudaEventDestroy(p.a);
            cudaEventDestroy(p.b);
        }
        g.prof.clear();
        int64_t l0 = c->launches;
        c->capturing = true;
        c->cap_pending.clear();
        int rc = capture_graph(c->stream, &g.exec, [&] { return enqueue_compute(c, Tfree, istep); });
        c->capturing = false;
        g.prof.swap(c->cap_pending);
        if (rc) {
            for (auto& p : g.prof) {
                cudaEventDestroy(p.a);
                cudaEventDestroy(p.b);
            }
            g.prof.clear();
            return rc;
        }
        g.key_epoch = c->epoch;
        g.key_tfree = Tfree;
        g.key_mask = mask;
        g.nlaunch = c->launches - l0;
        c->launches = l0;   // counted when the graph runs
    }
    CU(cudaGraphLaunch(g.exec, c->stream));
    c->launches += g.nlaunch;
    if (prof) c->pending.insert(c->pending.end(), g.prof.begin(), g.prof.end());
    return QNB_OK;
}

// adds the energies of every window, as read into e, into E / EQ / Erst
void add_window_energies(const qnb_context* c, const double* e, qnb_energies* E, qnb_qenergies* EQ, double* Erst) {
    for (int w = 0; w < c->nwin; ++w) {
        add_energies(e + (size_t)w * kNumE, E ? E + w : nullptr, EQ ? EQ + (size_t)w * c->S : nullptr, c->S);
        if (Erst) {
            Erst[2 * w] += e[(size_t)w * kNumE + E_RST_RAD];
            Erst[2 * w + 1] += e[(size_t)w * kNumE + E_RST_POL];
        }
    }
}

int energies_out(qnb_context* c, qnb_energies* E, qnb_qenergies* EQ, double* Erst) {
    std::vector<double> e((size_t)kNumE * c->nwin);
    TRY(read_energies(c, c->nwin, e.data()));
    add_window_energies(c, e.data(), E, EQ, Erst);
    return QNB_OK;
}

}  // namespace

extern "C" {

int qnb_compute_dev(qnb_context* c, double Tfree, int32_t istep, int32_t sync, qnb_energies* E, qnb_qenergies* EQ,
                    double* Erst) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    if (!c->lists_built) return fail(QNB_ERR_STATE, "pair lists not built");
    TRY(run_compute(c, Tfree, istep));
    if (sync) TRY(energies_out(c, E, EQ, Erst));
    return QNB_OK;
}

int qnb_step_host(qnb_context* c, const double* x_all, double* d_all, double Tfree, int32_t istep,
                  int32_t rebuild_lists, qnb_energies* E, qnb_qenergies* EQ, double* Erst) {
    if (!c || !x_all || !d_all) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    if (!c->lists_built) return fail(QNB_ERR_STATE, "pair lists not built (build them once with qnb_make_pair_lists_dev)");
    const size_t n = 3 * (size_t)c->natom * c->nwin;
    CU(cudaMemcpyAsync(c->x_all, x_all, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
    if (rebuild_lists) {   // waits for its list counts
        const Cut cut = c->last_cut;
        TRY(build_lists(c, cut, c->nwin));
    }
    TRY(run_compute(c, Tfree, istep));
    CU(cudaMemcpyAsync(d_all, c->d_all, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemsetAsync(c->d_all, 0, sizeof(double) * n, c->stream));
    TRY(enqueue_energies(c, c->nwin));
    CU(cudaStreamSynchronize(c->stream));
    std::vector<double> e((size_t)kNumE * c->nwin);
    finish_energies(c, c->nwin, e.data());
    add_window_energies(c, e.data(), E, EQ, Erst);
    return QNB_OK;
}

int qnb_pot_energy_step(qnb_context* c, const double* x, double* d, double Tfree, int32_t istep, qnb_energies* E,
                        qnb_qenergies* EQ, double* Erst) {
    if (!c || !x || !d) return fail(QNB_ERR_ARG, "null argument");
    if (c->nwin != 1) return fail(QNB_ERR_ARG, "single-window contexts only (batches: qnb_compute_dev)");
    CU(cudaSetDevice(c->device));
    if (!c->lists_built) return fail(QNB_ERR_STATE, "pair lists not built");
    TRY(stage_x(c, x));
    TRY(run_compute(c, Tfree, istep));   // gradient applied into window 0's FP64 accumulator
    const size_t n = 3 * (size_t)c->natom;
    // stream order: the coordinate copy out of h_stage precedes this copy into it
    CU(cudaMemcpyAsync(c->h_stage, c->st[0].d, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemsetAsync(c->st[0].d, 0, n * sizeof(double), c->stream));
    CU(cudaMemcpyAsync(c->h_e, c->e_all, sizeof(double) * kNumE, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaMemcpyAsync(c->h_e + (size_t)kNumE * c->nwin, c->efix_all, sizeof(double) * kNumE,
                       cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (size_t k = 0; k < n; ++k) d[k] += c->h_stage[k];
    const long long* fx = (const long long*)(c->h_e + (size_t)kNumE * c->nwin);
    double e[kNumE];
    for (int k = 0; k < kNumE; ++k) e[k] = c->h_e[k] + (double)fx[k] * (1.0 / kFix);
    add_energies(e, E, EQ, c->S);
    if (Erst) {
        Erst[0] += e[E_RST_RAD];
        Erst[1] += e[E_RST_POL];
    }
    return QNB_OK;
}

int qnb_set_solvent_internal(qnb_context* c, int32_t n, const int32_t* ij, const double* A, const double* B,
                             const double* el) {
    if (!c || n < 0 || (n > 0 && (!ij || !A || !B || !el))) return fail(QNB_ERR_ARG, "null argument");
    for (int k = 0; k < n; ++k)
        if (ij[2 * k] < 0 || ij[2 * k] >= c->m.sa || ij[2 * k + 1] < 0 || ij[2 * k + 1] >= c->m.sa ||
            ij[2 * k] == ij[2 * k + 1])
            return fail(QNB_ERR_ARG, "solvent pair %d: atoms must be distinct offsets 0..%d", k, c->m.sa - 1);
    CU(cudaSetDevice(c->device));
    if (c->d_si) c->release(c->d_si), c->d_si = nullptr;
    if (c->d_sip) c->release(c->d_sip), c->d_sip = nullptr;
    c->nsi = 0;
    if (n > 0) {
        std::vector<int2> v(n);
        std::vector<double> p(3 * (size_t)n);
        for (int k = 0; k < n; ++k) {
            v[k] = make_int2(ij[2 * k], ij[2 * k + 1]);
            p[3 * k] = A[k];
            p[3 * k + 1] = B[k];
            p[3 * k + 2] = el[k];
        }
        TRY(c->upload(&c->d_si, v));
        TRY(c->upload(&c->d_sip, p));
        c->nsi = n;
    }
    ++c->epoch;   // a launch more (or less) per step
    return QNB_OK;
}

int qnb_get_tuning(qnb_context* c, int32_t* values) {
    if (!c || !values) return fail(QNB_ERR_ARG, "null argument");
    for (int k = 0; k < T_NUM; ++k) values[k] = c->tune.v[k];
    return QNB_OK;
}

int qnb_set_tuning(qnb_context* c, const int32_t* values) {
    if (!c || !values) return fail(QNB_ERR_ARG, "null argument");
    for (int k = 0; k < T_NUM; ++k)
        if (values[k] < 1 || values[k] > 256) return fail(QNB_ERR_ARG, "tuning value %d out of 1..256", k);
    for (int k = 0; k < T_NUM; ++k) c->tune.v[k] = values[k];
    ++c->epoch;   // new launch geometry: captured graphs are stale
    return QNB_OK;
}

// Autotuner: coordinate search over the launch geometry of the per-step
// kernels (blocks per SM of the solute rows, water rows, qp, qw and LRF
// Taylor kernels) and of the list build (row build, LRF accumulation), each
// candidate timed with CUDA events over `reps` evaluations (or builds) of the
// current lists and coordinates after one untimed run.  Results do not
// depend on these choices (the mixed form is bit-identical for every one).
// The Q-kernel chunk size is not searched: it sets the grouping of the Q
// energies' FP32 partial sums (qnb_set_tuning can still change it).  The
// watpol running averages are restored afterwards; the gradient accumulators
// are cleared.
int qnb_autotune(qnb_context* c, int32_t reps, int32_t* values) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    if (!c->lists_built) return fail(QNB_ERR_STATE, "pair lists not built");
    if (reps < 1) reps = 1;
    CU(cudaSetDevice(c->device));
    const size_t wsn = 3 * kMaxShell;
    std::vector<double> ws(wsn * c->nwin);
    for (int w = 0; w < c->nwin; ++w)
        CU(cudaMemcpyAsync(ws.data() + wsn * w, c->st[w].wstate, sizeof(double) * wsn, cudaMemcpyDeviceToHost,
                           c->stream));
    CU(cudaStreamSynchronize(c->stream));
    collect_profile(c);
    // each candidate is timed with the evaluation's branches off: beside the
    // other branches a kernel's span includes its wait for block slots
    const bool prof0 = c->profiling, graphs0 = c->use_graphs, branches0 = c->branches;
    const unsigned mask0 = c->prof_mask;
    c->branches = false;
    double ms0[K_NUM];
    int64_t n0[K_NUM];
    for (int k = 0; k < K_NUM; ++k) ms0[k] = c->prof_ms[k], n0[k] = c->prof_n[k];
    c->use_graphs = false;
    const int nw = c->last_build_nw;
    auto run = [&](bool build, unsigned mask, int count) -> int {
        c->profiling = true;
        c->prof_mask = mask;
        for (int r = 0; r < count; ++r) {
            if (build) TRY(build_lists(c, c->last_cut, nw));
            else TRY(enqueue_compute(c, 300.0, 1));
        }
        collect_profile(c);
        return QNB_OK;
    };
    auto measure = [&](bool build, unsigned mask, double* ms) -> int {
        TRY(run(build, mask, 1));   // untimed: first launch of this geometry
        for (int k = 0; k < K_NUM; ++k) c->prof_ms[k] = 0.0, c->prof_n[k] = 0;
        TRY(run(build, mask, reps));
        double t = 0.0;
        for (int k = 0; k < K_NUM; ++k)
            if ((mask >> k) & 1u) t += c->prof_ms[k];
        *ms = t;
        return QNB_OK;
    };
    struct Plan {
        int t;
        std::vector<int> vals;
        unsigned mask;
        bool build;
    };
    const unsigned B = 1u;
    std::vector<Plan> plan = {
        {T_ROWS_SOLUTE, {4, 6, 8, 12, 16, 24, 32, 48}, B << K_PP, false},
        {T_ROWS_WATER, {4, 8, 12, 16, 24, 32, 48}, B << K_WW, false},
        {T_QP, {2, 3, 4, 6, 8, 12, 16}, B << K_QP, false},
        {T_QW, {2, 3, 4, 6, 8, 12, 16}, B << K_QW, false},
        {T_TAYLOR, {8, 16, 24, 32, 48, 64}, B << K_LRF_TAYLOR, false},
    };
    if (c->mixed) plan.push_back({T_BUILD, {8, 16, 24, 32, 48, 64}, B << K_BUILD, true});
    if (c->mixed && c->use_lrf) plan.push_back({T_LRF, {2, 3, 4, 6, 8, 12}, B << K_LRF_BUILD, true});
    int rc = QNB_OK;
    for (auto& p : plan) {
        int best = c->tune.v[p.t];
        double best_ms = 1e30;
        for (int v : p.vals) {
            c->tune.v[p.t] = v;
            double ms = 0.0;
            rc = measure(p.build, p.mask, &ms);
            if (rc) break;
            if (ms < best_ms) best_ms = ms, best = v;
        }
        c->tune.v[p.t] = best;
        if (rc) break;
    }
    // restore: profiling state, totals, watpol averages; clear the gradients
    c->profiling = prof0;
    c->prof_mask = mask0;
    c->use_graphs = graphs0;
    c->branches = branches0;
    for (int k = 0; k < K_NUM; ++k) c->prof_ms[k] = ms0[k], c->prof_n[k] = n0[k];
    for (int w = 0; w < c->nwin; ++w)
        CU(cudaMemcpyAsync(c->st[w].wstate, ws.data() + wsn * w, sizeof(double) * wsn, cudaMemcpyHostToDevice,
                           c->stream));
    CU(cudaMemsetAsync(c->d_all, 0, sizeof(double) * 3 * (size_t)c->natom * c->nwin, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    ++c->epoch;
    if (rc) return rc;
    if (values)
        for (int k = 0; k < T_NUM; ++k) values[k] = c->tune.v[k];
    return QNB_OK;
}

int qnb_get_energies_dev(qnb_context* c, qnb_energies* E, qnb_qenergies* EQ, double* Erst) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    return energies_out(c, E, EQ, Erst);
}

int qnb_set_graphs(qnb_context* c, int32_t enable) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    c->use_graphs = enable != 0;
    return QNB_OK;
}

int qnb_set_concurrency(qnb_context* c, int32_t enable) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    if (c->branches != (enable != 0)) {
        c->branches = enable != 0;
        ++c->epoch;   // the captured graphs hold the old structure
    }
    return QNB_OK;
}

}  // extern "C"

// ---- groups: several contexts (uneven systems) in one graph launch ---------
struct qnb_group {
    std::vector<qnb_context*> ctx;
    cudaEvent_t fork = nullptr, done = nullptr;
    std::vector<cudaEvent_t> join;
    struct Slot {
        cudaGraphExec_t exec = nullptr;
        std::vector<uint64_t> epochs;
        std::vector<char> update;
        double tfree = 0.0;
        int64_t nlaunch = 0;
    };
    std::vector<Slot> slots;   // one per distinct pattern of watpol update steps seen
};

extern "C" {

int qnb_group_create(qnb_context** ctxs, int32_t n, qnb_group** out) {
    if (!ctxs || !out || n < 1) return fail(QNB_ERR_ARG, "null argument or empty group");
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!ctxs[i]) return fail(QNB_ERR_ARG, "null context %d", i);
        if (ctxs[i]->device != ctxs[0]->device) return fail(QNB_ERR_ARG, "group contexts on different devices");
        for (int j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) return fail(QNB_ERR_ARG, "context %d repeated in the group", i);
    }
    CU(cudaSetDevice(ctxs[0]->device));
    qnb_group* g = new qnb_group();
    g->ctx.assign(ctxs, ctxs + n);
    g->join.assign(n, nullptr);
    cudaError_t e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming);
    for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&g->join[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        qnb_group_destroy(g);
        return fail(QNB_ERR_CUDA, "group events: %s", cudaGetErrorString(e));
    }
    *out = g;
    return QNB_OK;
}

int qnb_group_destroy(qnb_group* g) {
    if (!g) return QNB_OK;
    for (auto& s : g->slots)
        if (s.exec) cudaGraphExecDestroy(s.exec);
    if (g->fork) cudaEventDestroy(g->fork);
    if (g->done) cudaEventDestroy(g->done);
    for (auto e : g->join)
        if (e) cudaEventDestroy(e);
    delete g;
    return QNB_OK;
}

// One evaluation of every window of every context of the group, as one CUDA
// graph launch on the first context's stream: the contexts' kernel
// sequences are independent branches of the graph, so systems of different
// sizes run concurrently.  The other contexts' streams wait for the graph.
int qnb_group_compute(qnb_group* g, double Tfree, int32_t istep) {
    if (!g) return fail(QNB_ERR_ARG, "null group");
    const int n = (int)g->ctx.size();
    qnb_context* c0 = g->ctx[0];
    CU(cudaSetDevice(c0->device));
    std::vector<uint64_t> epochs(n);
    std::vector<char> update(n);
    for (int i = 0; i < n; ++i) {
        if (!g->ctx[i]->lists_built) return fail(QNB_ERR_STATE, "pair lists of group context %d not built", i);
        if (g->ctx[i]->profiling) return fail(QNB_ERR_STATE, "profiling is on for group context %d", i);
        epochs[i] = g->ctx[i]->epoch;
        update[i] = watpol_update_step(g->ctx[i], istep) ? 1 : 0;
    }
    qnb_group::Slot* slot = nullptr;
    for (auto& s : g->slots)
        if (s.update == update) slot = &s;
    if (!slot) {
        g->slots.emplace_back();
        slot = &g->slots.back();
        slot->update = update;
    }
    if (!slot->exec || slot->epochs != epochs || slot->tfree != Tfree) {
        if (slot->exec) cudaGraphExecDestroy(slot->exec);
        std::vector<int64_t> l0(n);
        for (int i = 0; i < n; ++i) l0[i] = g->ctx[i]->launches;
        TRY(capture_graph(c0->stream, &slot->exec, [&]() -> int {
            CU(cudaEventRecord(g->fork, c0->stream));
            for (int i = 1; i < n; ++i) CU(cudaStreamWaitEvent(g->ctx[i]->stream, g->fork, 0));
            for (int i = 0; i < n; ++i) TRY(enqueue_compute(g->ctx[i], Tfree, istep));
            for (int i = 1; i < n; ++i) {
                CU(cudaEventRecord(g->join[i], g->ctx[i]->stream));
                CU(cudaStreamWaitEvent(c0->stream, g->join[i], 0));
            }
            return QNB_OK;
        }));
        slot->epochs = epochs;
        slot->tfree = Tfree;
        slot->nlaunch = 0;
        for (int i = 0; i < n; ++i) {
            slot->nlaunch += g->ctx[i]->launches - l0[i];
            g->ctx[i]->launches = l0[i];
        }
    }
    CU(cudaGraphLaunch(slot->exec, c0->stream));
    c0->launches += slot->nlaunch;
    CU(cudaEventRecord(g->done, c0->stream));
    for (int i = 1; i < n; ++i) CU(cudaStreamWaitEvent(g->ctx[i]->stream, g->done, 0));
    return QNB_OK;
}

int qnb_q_adjoint_dev(qnb_context* c, double* dq, double* dA, double* dB) {
    if (!c || !dq || !dA || !dB) return fail(QNB_ERR_ARG, "null argument");
    if (!c->lists_built) return fail(QNB_ERR_STATE, "pair lists not built");
    CU(cudaSetDevice(c->device));
    const size_t n = (size_t)c->nqat * c->S;
    if (n == 0) return QNB_OK;
    for (int w = 0; w < c->nwin; ++w) CU(cudaMemsetAsync(c->st[w].adj, 0, sizeof(double) * 3 * n, c->stream));
    launch_q_adjoint(c->all());
    c->launches += 3;
    TRY(check_launch());
    std::vector<double> h(3 * n);
    for (int w = 0; w < c->nwin; ++w) {
        CU(cudaMemcpyAsync(h.data(), c->st[w].adj, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
        CU(cudaStreamSynchronize(c->stream));
        memcpy(dq + w * n, h.data(), sizeof(double) * n);
        memcpy(dA + w * n, h.data() + n, sizeof(double) * n);
        memcpy(dB + w * n, h.data() + 2 * n, sizeof(double) * n);
    }
    return QNB_OK;
}

int qnb_profile(qnb_context* c, int32_t enable) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    collect_profile(c);
    c->profiling = enable != 0;
    c->prof_mask = ~0u;
    return QNB_OK;
}
int qnb_profile_classes(qnb_context* c, uint32_t mask) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    collect_profile(c);
    c->profiling = mask != 0;
    c->prof_mask = mask;
    return QNB_OK;
}

int qnb_profile_collect(qnb_context* c) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    collect_profile(c);
    return QNB_OK;
}
int qnb_kernel_times(qnb_context* c, double* ms, int64_t* launches, int32_t n) {
    if (!c || !ms || !launches) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    collect_profile(c);
    for (int k = 0; k < n && k < K_NUM; ++k) {
        ms[k] = c->prof_ms[k];
        launches[k] = c->prof_n[k];
        c->prof_ms[k] = 0.0;
        c->prof_n[k] = 0;
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

// =============================================================================
// Device-resident MD step (qnb_md_*)
// =============================================================================
namespace {

constexpr double kMagicStepConv = 0.020462;   // fs -> internal time, src/globals.f90:47
constexpr double kBoltz = 0.001986;           // src/globals.f90:46
constexpr int kMdChunk = 256;                 // steps recorded on the device between read-backs

// Eb[0..7] classical bonded, Eb[8 + 4s + k] Q bonded of state s
void bonded_out(const qnb_context* c, const double* e, double* Eb) {
    for (int k = 0; k < 8; ++k) Eb[k] = e[E_B0 + k];
    for (int st = 0; st < c->S; ++st)
        for (int k = 0; k < 4; ++k) Eb[8 + 4 * st + k] = e[qb_slot(st, k)];
}

int md_check(qnb_context* c) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    if (!c->md_ready) return fail(QNB_ERR_STATE, "qnb_md_init not called");
    return QNB_OK;
}

// windows whose SHAKE failed since the flags were cleared
int md_fail_check(qnb_context* c) {
    std::vector<int> f(c->nwin);
    CU(cudaMemcpyAsync(f.data(), c->md.fail, sizeof(int) * c->nwin, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (int w = 0; w < c->nwin; ++w)
        if (f[w]) return fail(QNB_ERR_CONSTRAINT, "SHAKE failed in window %d, molecule %d", w, f[w] - 1);
    return QNB_OK;
}

}  // namespace

extern "C" {

int qnb_md_init(qnb_context* c, const qnb_md_params* p, const double* mass, int32_t nmol, const int32_t* mol_first,
                const int32_t* con_ij, const double* con_dist) {
    if (!c || !p || !mass || nmol < 0 || (nmol > 0 && (!mol_first || !con_ij || !con_dist)))
        return fail(QNB_ERR_ARG, "null argument");
    if (c->md_ready) return fail(QNB_ERR_STATE, "qnb_md_init already called on this context");
    const int n = c->natom;
    if (!(p->stepsize > 0.0) || !(p->temp0 > 0.0) || !(p->tau_t >= p->stepsize))
        return fail(QNB_ERR_ARG, "stepsize > 0, temp0 > 0 and tau_t >= stepsize required");
    if (p->ntgroups < 1 || p->ntgroups > kMaxTg) return fail(QNB_ERR_ARG, "ntgroups %d not in 1..%d", p->ntgroups, kMaxTg);
    if (p->nbcycle < 1) return fail(QNB_ERR_ARG, "nbcycle %d < 1", p->nbcycle);
    if (!(p->ndegf > 0.0) || !(p->ndegfree > 0.0)) return fail(QNB_ERR_ARG, "degrees of freedom must be positive");
    for (int g = 0; g < p->ntgroups; ++g) {
        if (p->tg_first[g] < 0 || p->tg_last[g] >= n || p->tg_first[g] > p->tg_last[g])
            return fail(QNB_ERR_ARG, "temperature group %d: bad atom range", g);
        if (!(p->tg_ndegf[g] > 0.0) || !(p->tg_ndegfree[g] > 0.0))
            return fail(QNB_ERR_ARG, "temperature group %d: degrees of freedom must be positive", g);
        for (int h = 0; h < g; ++h)
            if (p->tg_first[g] <= p->tg_last[h] && p->tg_first[h] <= p->tg_last[g])
                return fail(QNB_ERR_ARG, "temperature groups %d and %d overlap", h, g);
    }
    for (int i = 0; i < n; ++i)
        if (!(mass[i] > 0.0)) return fail(QNB_ERR_ARG, "mass of atom %d not positive", i);
    int ncons = 0;
    if (nmol > 0) {
        if (mol_first[0] != 0) return fail(QNB_ERR_ARG, "mol_first[0] must be 0");
        for (int m = 0; m < nmol; ++m)
            if (mol_first[m + 1] < mol_first[m]) return fail(QNB_ERR_ARG, "mol_first not ascending at %d", m);
        ncons = mol_first[nmol];
        for (int k = 0; k < ncons; ++k) {
            int i = con_ij[2 * k], j = con_ij[2 * k + 1];
            if (i < 0 || i >= n || j < 0 || j >= n || i == j || !(con_dist[k] > 0.0))
                return fail(QNB_ERR_ARG, "constraint %d: bad atoms or distance", k);
        }
    }
    CU(cudaSetDevice(c->device));
    MdDev& md = c->md;
    md = MdDev{};
    md.natom = n;
    md.ntg = p->ntgroups;
    md.nmol = nmol;
    md.ncons = ncons;
    for (int g = 0; g < kMaxTg; ++g) {
        bool on = g < p->ntgroups;
        md.tg_first[g] = on ? p->tg_first[g] : 1;
        md.tg_last[g] = on ? p->tg_last[g] : 0;
        md.tg_ndegf[g] = on ? p->tg_ndegf[g] : 1.0;
        md.tg_ndegfree[g] = on ? p->tg_ndegfree[g] : 1.0;
    }
    md.ndegf = p->ndegf;
    md.ndegfree = p->ndegfree;
    md.dt = kMagicStepConv * p->stepsize;
    md.tau = kMagicStepConv * p->tau_t;
    md.temp0 = p->temp0;
    md.boltz = kBoltz;
    std::vector<double> m(mass, mass + n), wi(n);
    for (int i = 0; i < n; ++i) wi[i] = 1.0 / m[i];
    TRY(c->upload((double**)&md.mass, m));
    TRY(c->upload((double**)&md.winv, wi));
    std::vector<int> mf(nmol + 1, 0);
    std::vector<int2> con(ncons);
    std::vector<double> d2(ncons);
    for (int k = 0; k <= nmol && nmol > 0; ++k) mf[k] = mol_first[k];
    for (int k = 0; k < ncons; ++k) {
        con[k] = make_int2(con_ij[2 * k], con_ij[2 * k + 1]);
        d2[k] = con_dist[k] * con_dist[k];
    }
    TRY(c->upload((int**)&md.mol_first, mf));
    TRY(c->upload((int2**)&md.con, con));
    TRY(c->upload((double**)&md.dist2, d2));
    const size_t n3 = 3 * (size_t)n;
    TRY(c->alloc(&md.ready, (size_t)std::max(1, ncons) * c->nwin));
    TRY(c->alloc(&md.v, n3 * c->nwin));
    TRY(c->alloc(&md.xx, n3 * c->nwin));
    TRY(c->alloc(&md.win, (size_t)c->nwin));
    TRY(c->alloc(&md.fail, (size_t)c->nwin));
    CU(cudaMemset(md.v, 0, sizeof(double) * n3 * c->nwin));
    CU(cudaMemset(md.xx, 0, sizeof(double) * n3 * c->nwin));
    CU(cudaMemset(md.win, 0, sizeof(MdWin) * c->nwin));
    CU(cudaMemset(md.fail, 0, sizeof(int) * c->nwin));
    TRY(c->alloc(&c->md_rec, (size_t)kMdChunk * c->nwin * kMdRec));
    c->md_rec_steps = kMdChunk;
    CU(cudaMallocHost((void**)&c->h_md_rec, sizeof(double) * kMdChunk * c->nwin * kMdRec));
    // restrain_solvent of an MD step reads the window's Tfree on the device
    for (int w = 0; w < c->nwin; ++w) c->st[w].md_tfree = &md.win[w].tfree;
    TRY(upload_states(c));
    c->mdp = *p;
    c->md_ready = true;
    c->md_prepared = false;
    return QNB_OK;
}

int qnb_md_set_thermostat(qnb_context* c, int32_t thermostat, int32_t integrator, int32_t nhchains, double nhq) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    TRY(md_check(c));
    if (thermostat < 0 || thermostat > 1) return fail(QNB_ERR_ARG, "thermostat %d (0 Berendsen, 1 Nose-Hoover)", thermostat);
    if (integrator < 0 || integrator > 1) return fail(QNB_ERR_ARG, "integrator %d (0 leap-frog, 1 velocity Verlet)", integrator);
    if (thermostat == 1 && (nhchains < 2 || nhchains > kMaxNh))
        return fail(QNB_ERR_ARG, "nhchains %d (2..%d supported)", nhchains, kMaxNh);
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    c->md.thermostat = thermostat;
    c->md.vv = integrator;
    c->md.nhchains = thermostat == 1 ? nhchains : 0;
    // nose-hoover_mass default kbT / tau_T^2 (src/md.f90:282-285), tau_T in internal units
    c->md.nhq = nhq > 0.0 ? nhq : c->md.boltz * c->md.temp0 / (c->md.tau * c->md.tau);
    // chain start, src/simprep.f90:2477-2485
    std::vector<MdWin> win(c->nwin);
    CU(cudaMemcpy(win.data(), c->md.win, sizeof(MdWin) * c->nwin, cudaMemcpyDeviceToHost));
    for (auto& mw : win) {
        for (int i = 0; i < kMaxNh; ++i) {
            mw.qnh[i] = c->md.nhq;
            mw.vnh[i] = 0.0;
            mw.xnh[i] = 0.0;
        }
        mw.qnh[0] = c->md.ndegf * c->md.nhq;
        mw.nh_s = 1.0;
    }
    CU(cudaMemcpy(c->md.win, win.data(), sizeof(MdWin) * c->nwin, cudaMemcpyHostToDevice));
    ++c->epoch;
    return QNB_OK;
}

int qnb_md_set_langevin(qnb_context* c, int32_t integrator, double friction, uint64_t seed) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    TRY(md_check(c));
    if (integrator < 0 || integrator > 1) return fail(QNB_ERR_ARG, "integrator %d (0 leap-frog, 1 velocity Verlet)", integrator);
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    c->md.thermostat = 2;
    c->md.vv = integrator;
    // langevin_friction default 1/tau_T (src/md.f90:250-253); gkT with
    // uniform draws, src/md.f90:1637-1648
    c->md.lan_friction = friction > 0.0 ? friction : 1.0 / c->md.tau;
    const double step = integrator ? 0.5 * c->md.dt : c->md.dt;
    c->md.lan_gkT = 24.0 * c->md.lan_friction * c->md.boltz * c->md.temp0 / step;
    c->md.lan_seed = seed;
    ++c->epoch;
    return QNB_OK;
}

int qnb_set_put_back_in_box(qnb_context* c, int32_t nmol, const int32_t* mol_first, const int32_t* atoms,
                            int32_t nmol_solute, int32_t put_solute, int32_t put_solvent, const double* boxcentre) {
    if (!c || nmol < 0 || (nmol > 0 && (!mol_first || !atoms))) return fail(QNB_ERR_ARG, "null argument");
    TRY(md_check(c));
    if (nmol_solute < 0 || nmol_solute > nmol) return fail(QNB_ERR_ARG, "nmol_solute out of range");
    for (int q = 0; q < nmol; ++q)
        if (mol_first[q] < 0 || mol_first[q + 1] <= mol_first[q]) return fail(QNB_ERR_ARG, "molecule %d empty", q);
    for (int q = 0; nmol > 0 && q < mol_first[nmol]; ++q)
        if (atoms[q] < 0 || atoms[q] >= c->natom) return fail(QNB_ERR_ARG, "molecule atom %d out of range", q);
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    MdDev& md = c->md;
    md.pb_nmol = nmol;
    md.pb_first_mol = put_solute ? 0 : nmol_solute;
    md.pb_last_mol = put_solvent ? nmol : nmol_solute;
    md.pb_rigid = boxcentre != nullptr;
    md.pb_nslu = c->nat_solute > 0 ? c->nat_solute : c->natom;
    for (int k = 0; k < 3; ++k) md.pb_centre[k] = boxcentre ? boxcentre[k] : 0.0;
    if (nmol > 0) {
        std::vector<int> first(mol_first, mol_first + nmol + 1), at(atoms, atoms + mol_first[nmol]);
        TRY(c->upload((int**)&md.pb_mol_first, first));
        TRY(c->upload((int**)&md.pb_atoms, at));
        if (!md.pb_boxc) TRY(c->alloc(&md.pb_boxc, (size_t)3 * c->nwin));
    }
    ++c->epoch;
    return QNB_OK;
}

int qnb_put_back_in_box(qnb_context* c, double* boxcentre) {
    TRY(md_check(c));
    if (!c->m.box) return fail(QNB_ERR_STATE, "no periodic box (qnb_set_box)");
    if (c->md.pb_last_mol <= c->md.pb_first_mol) return QNB_OK;
    CU(cudaSetDevice(c->device));
    launch_md_put_back(c->all(), c->md);
    c->launches++;
    TRY(check_launch());
    if (boxcentre)
        CU(cudaMemcpyAsync(boxcentre, c->md.pb_boxc, sizeof(double) * 3 * c->nwin, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return QNB_OK;
}

int qnb_md_set_velocities(qnb_context* c, int32_t w, const double* v) {
    TRY(md_check(c));
    if (!v || w < 0 || w >= c->nwin) return fail(QNB_ERR_ARG, "bad window or null velocities");
    CU(cudaSetDevice(c->device));
    size_t n3 = 3 * (size_t)c->natom;
    CU(cudaMemcpy(c->md.v + n3 * w, v, sizeof(double) * n3, cudaMemcpyHostToDevice));
    c->md_prepared = false;
    return QNB_OK;
}

int qnb_md_get_state(qnb_context* c, int32_t w, double* x, double* v) {
    TRY(md_check(c));
    if (w < 0 || w >= c->nwin) return fail(QNB_ERR_ARG, "window %d of %d", w, c->nwin);
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    size_t n3 = 3 * (size_t)c->natom;
    if (x) CU(cudaMemcpy(x, c->st[w].x, sizeof(double) * n3, cudaMemcpyDeviceToHost));
    if (v) CU(cudaMemcpy(v, c->md.v + n3 * w, sizeof(double) * n3, cudaMemcpyDeviceToHost));
    return QNB_OK;
}

int qnb_md_prepare(qnb_context* c, int32_t stop_cm) {
    TRY(md_check(c));
    CU(cudaSetDevice(c->device));
    Launch L = c->all();
    CU(cudaMemsetAsync(c->md.fail, 0, sizeof(int) * c->nwin, c->stream));
    // initial_constraint: xx = x, SHAKE x; xx = x - v dt, SHAKE xx against x; v = (x - xx)/dt
    launch_md_copy_x(L, c->md, 1);
    launch_md_shake(L, c->md, 0);
    launch_md_copy_x(L, c->md, 2);
    launch_md_shake(L, c->md, 1);
    launch_md_velocity(L, c->md);
    if (stop_cm) launch_md_stop_cm(L, c->md);
    launch_md_temperature(L, c->md, c->m.excl);
    c->launches += 6 + (stop_cm ? 1 : 0) + 1;
    TRY(check_launch());
    TRY(md_fail_check(c));
    c->md_prepared = true;
    return QNB_OK;
}

int qnb_md_minimize(qnb_context* c, int32_t nsteps, double initial_step, double force_cutoff, double max_move,
                    double* maxf) {
    TRY(md_check(c));
    if (nsteps < 0 || !(initial_step > 0.0) || force_cutoff < 0.0 || max_move < 0.0)
        return fail(QNB_ERR_ARG, "bad minimisation arguments");
    CU(cudaSetDevice(c->device));
    const qnb_md_params& p = c->mdp;
    const int W = c->nwin;
    CU(cudaMemsetAsync(c->md.fail, 0, sizeof(int) * W, c->stream));
    std::vector<MdWin> mw(W);
    CU(cudaMemcpy(mw.data(), c->md.win, sizeof(MdWin) * W, cudaMemcpyDeviceToHost));
    for (auto& m : mw) m.min_oldmax = 0.0, m.min_scale = initial_step, m.min_state = 0;
    CU(cudaMemcpy(c->md.win, mw.data(), sizeof(MdWin) * W, cudaMemcpyHostToDevice));
    Cut cut = make_cut(p.rcq * p.rcq, p.rclrf * p.rclrf, p.rcpp * p.rcpp, p.rcpw * p.rcpw, p.rcww * p.rcww);
    for (int k = 0; k < nsteps; ++k) {
        if (k % p.nbcycle == 0 || !c->lists_built) {
            if (k > 0) TRY(md_fail_check(c));
            TRY(build_lists(c, cut, W));
        }
        Launch L = c->all();
        launch_md_clear_d(L, c->md);
        TRY(run_compute(c, 0.0, k));
        launch_md_min_step(L, c->md, initial_step, force_cutoff, max_move);
        launch_md_shake(L, c->md, 0);
        c->launches += 3;
        TRY(check_launch());
    }
    TRY(md_fail_check(c));
    CU(cudaMemcpy(mw.data(), c->md.win, sizeof(MdWin) * W, cudaMemcpyDeviceToHost));
    if (maxf)
        for (int w = 0; w < W; ++w) maxf[w] = mw[w].min_maxf;
    c->md_prepared = false;
    return QNB_OK;
}

int qnb_md_run(qnb_context* c, int32_t nsteps, int32_t istep0, qnb_md_record* rec, qnb_qenergies* EQ,
               double* Eb) {
    TRY(md_check(c));
    if (nsteps < 0 || istep0 < 0) return fail(QNB_ERR_ARG, "nsteps and istep0 must be >= 0");
    if (!c->md_prepared) return fail(QNB_ERR_STATE, "qnb_md_prepare not called since the last state change");
    CU(cudaSetDevice(c->device));
    const qnb_md_params& p = c->mdp;
    const int W = c->nwin;
    CU(cudaMemsetAsync(c->md.fail, 0, sizeof(int) * W, c->stream));
    for (int k0 = 0; k0 < nsteps; k0 += kMdChunk) {
        const int nk = std::min(kMdChunk, nsteps - k0);
        for (int k = 0; k < nk; ++k) {
            const int istep = istep0 + k0 + k;
            if (istep % p.nbcycle == 0 || !c->lists_built) {
                if (k0 + k > 0) TRY(md_fail_check(c));   // no list build on coordinates of a failed SHAKE
                // every NBcycle steps, before the lists (src/md.f90:1663-1671)
                if (c->m.box && c->md.pb_last_mol > c->md.pb_first_mol) launch_md_put_back(c->all(), c->md), c->launches++;
                Cut cut = make_cut(p.rcq * p.rcq, p.rclrf * p.rclrf, p.rcpp * p.rcpp, p.rcpw * p.rcpw, p.rcww * p.rcww);
                TRY(build_lists(c, cut, W));
            }
            Launch L = c->all();
            launch_md_clear_d(L, c->md);
            c->launches++;
            TRY(run_compute(c, -1.0, istep));   // Tfree < 0: restrain_solvent reads it on the device
            // md_run's step, src/md.f90:1768-1812: thermostat + move, SHAKE,
            // v = (x - xx)/dt, Nose-Hoover again after SHAKE, temperature
            const bool nh = c->md.thermostat == 1;
            c->md.istep = istep;
            timed(c, K_MD, [&] {
                if (nh) launch_md_nh(L, c->md);
                launch_md_newvel(L, c->md);
                launch_md_shake(L, c->md, 0);
                if (c->md.nmol > 0) {
                    launch_md_velocity(L, c->md);
                    if (nh) launch_md_nh(L, c->md);
                }
                launch_md_temperature(L, c->md, c->m.excl);
                launch_md_record(L, c->md, c->e_all, c->efix_all, c->md_rec + (size_t)k * W * kMdRec);
            });
            c->launches += 4 + (c->md.nmol > 0 ? 1 : 0) + (nh ? (c->md.nmol > 0 ? 4 : 2) : 0);
            TRY(check_launch());
        }
        if (rec || EQ || Eb) {
            CU(cudaMemcpyAsync(c->h_md_rec, c->md_rec, sizeof(double) * nk * W * kMdRec, cudaMemcpyDeviceToHost,
                               c->stream));
            CU(cudaStreamSynchronize(c->stream));
            for (int k = 0; k < nk; ++k)
                for (int w = 0; w < W; ++w) {
                    const double* r = c->h_md_rec + ((size_t)k * W + w) * kMdRec;
                    const long long* fx = reinterpret_cast<const long long*>(r + kNumE);
                    double e[kNumE];
                    for (int q = 0; q < kNumE; ++q) e[q] = r[q] + (double)fx[q] * (1.0 / kFix);
                    size_t idx = (size_t)(k0 + k) * W + w;
                    if (rec) {
                        qnb_md_record& o = rec[idx];
                        o = qnb_md_record{};
                        add_energies(e, &o.E, nullptr, c->S);
                        o.solvent_radial = e[E_RST_RAD];
                        o.water_pol = e[E_RST_POL];
                        o.fix = e[E_RST_FIX];
                        o.shell = e[E_RST_SHELL];
                        o.protein = e[E_RST_PROT];
                        o.ekin = r[2 * kNumE];
                        o.temp = r[2 * kNumE + 1];
                        o.tfree = r[2 * kNumE + 2];
                        o.shake_iterations = r[2 * kNumE + 3];
                    }
                    if (EQ) {
                        for (int s = 0; s < c->S; ++s) EQ[idx * c->S + s] = qnb_qenergies{};
                        add_energies(e, nullptr, EQ + idx * c->S, c->S);
                    }
                    if (Eb) bonded_out(c, e, Eb + idx * (8 + 4 * (size_t)c->S));
                }
        }
        TRY(md_fail_check(c));
    }
    return QNB_OK;
}

}  // extern "C"

// =============================================================================
// Bonded terms (qnb_set_bonded)
// =============================================================================
extern "C" {

int qnb_set_bonded(qnb_context* c, const qnb_bonded* b) {
    if (!c || !b) return fail(QNB_ERR_ARG, "null argument");
    const int n = c->natom, S = c->S;
    auto atoms_ok = [&](const int32_t* v, int cnt, int stride, int na) -> bool {
        for (int k = 0; k < cnt; ++k)
            for (int a = 0; a < na; ++a)
                if (v[stride * k + a] < 0 || v[stride * k + a] >= n) return false;
        return true;
    };
    auto codes_ok = [&](const int32_t* v, int cnt, int stride, int off, int nlib) -> bool {
        for (int k = 0; k < cnt; ++k)
            if (v[stride * k + off] >= nlib) return false;
        return true;
    };
    struct L { int cnt, sol; const int32_t* v; int lib; const double* libv; const char* name; };
    const L cl[4] = {{b->nbonds, b->nbonds_solute, b->bonds, b->nbondlib, b->bondlib, "bond"},
                     {b->nangles, b->nangles_solute, b->angles, b->nanglib, b->anglib, "angle"},
                     {b->ntors, b->ntors_solute, b->torsions, b->ntorlib, b->torlib, "torsion"},
                     {b->nimps, b->nimps_solute, b->impropers, b->nimplib, b->implib, "improper"}};
    const int na[4] = {2, 3, 4, 4};
    for (int k = 0; k < 4; ++k) {
        if (cl[k].cnt < 0 || cl[k].sol < 0 || cl[k].sol > cl[k].cnt || cl[k].lib < 0 ||
            (cl[k].cnt > 0 && !cl[k].v) || (cl[k].lib > 0 && !cl[k].libv))
            return fail(QNB_ERR_ARG, "%s list: bad counts or null arrays", cl[k].name);
        if (!atoms_ok(cl[k].v, cl[k].cnt, na[k] + 1, na[k]) || !codes_ok(cl[k].v, cl[k].cnt, na[k] + 1, na[k], cl[k].lib))
            return fail(QNB_ERR_ARG, "%s list: atom or library code out of range", cl[k].name);
    }
    if (b->imp_type != 1 && b->imp_type != 2) return fail(QNB_ERR_ARG, "imp_type %d not 1 or 2", b->imp_type);
    struct Q { int cnt; const int32_t* v; const int32_t* code; int lib; const double* libv; const char* name; };
    const Q ql[4] = {{b->nqbonds, b->qbonds, b->qbond_code, b->nqbondlib, b->qbondlib, "Q bond"},
                     {b->nqangles, b->qangles, b->qangle_code, b->nqanglib, b->qanglib, "Q angle"},
                     {b->nqtors, b->qtorsions, b->qtorsion_code, b->nqtorlib, b->qtorlib, "Q torsion"},
                     {b->nqimps, b->qimpropers, b->qimproper_code, b->nqimplib, b->qimplib, "Q improper"}};
    for (int k = 0; k < 4; ++k) {
        if (ql[k].cnt < 0 || ql[k].lib < 0 || (ql[k].cnt > 0 && (!ql[k].v || !ql[k].code || S == 0)) ||
            (ql[k].lib > 0 && !ql[k].libv))
            return fail(QNB_ERR_ARG, "%s list: bad counts or null arrays", ql[k].name);
        if (!atoms_ok(ql[k].v, ql[k].cnt, na[k], na[k]) || !codes_ok(ql[k].code, ql[k].cnt * S, 1, 0, ql[k].lib))
            return fail(QNB_ERR_ARG, "%s list: atom or library code out of range", ql[k].name);
    }
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    for (void* p : c->bonded_bufs) c->release(p);
    c->bonded_bufs.clear();
    BondedDev d{};
    auto up = [&](auto** dst, const auto& vec) -> int {
        int rc = c->upload(dst, vec);
        if (!rc) c->bonded_bufs.push_back((void*)*dst);
        return rc;
    };
    std::vector<int4> bonds(b->nbonds), angles(b->nangles);
    for (int k = 0; k < b->nbonds; ++k) bonds[k] = make_int4(b->bonds[3 * k], b->bonds[3 * k + 1], b->bonds[3 * k + 2], 0);
    for (int k = 0; k < b->nangles; ++k)
        angles[k] = make_int4(b->angles[4 * k], b->angles[4 * k + 1], b->angles[4 * k + 2], b->angles[4 * k + 3]);
    std::vector<double2> bl(b->nbondlib), il(b->nimplib), qil(b->nqimplib);
    for (int k = 0; k < b->nbondlib; ++k) bl[k] = make_double2(b->bondlib[2 * k], b->bondlib[2 * k + 1]);
    for (int k = 0; k < b->nimplib; ++k) il[k] = make_double2(b->implib[2 * k], b->implib[2 * k + 1]);
    for (int k = 0; k < b->nqimplib; ++k) qil[k] = make_double2(b->qimplib[2 * k], b->qimplib[2 * k + 1]);
    auto d4 = [](const double* v, int cnt, int w) {
        std::vector<double4_16a> o(cnt);
        for (int k = 0; k < cnt; ++k) {
            o[k].x = v[w * k];
            o[k].y = v[w * k + 1];
            o[k].z = w > 2 ? v[w * k + 2] : 0.0;
            o[k].w = w > 3 ? v[w * k + 3] : 0.0;
        }
        return o;
    };
    std::vector<double4_16a> al = d4(b->anglib, b->nanglib, 4), tl = d4(b->torlib, b->ntorlib, 4),
                         qbl = d4(b->qbondlib, b->nqbondlib, 4), qal = d4(b->qanglib, b->nqanglib, 4),
                         qtl = d4(b->qtorlib, b->nqtorlib, 3);
    std::vector<int> tors(b->torsions, b->torsions + 5 * (size_t)b->ntors),
        imps(b->impropers, b->impropers + 5 * (size_t)b->nimps);
    std::vector<int2> qb(b->nqbonds);
    for (int k = 0; k < b->nqbonds; ++k) qb[k] = make_int2(b->qbonds[2 * k], b->qbonds[2 * k + 1]);
    auto i4 = [](const int32_t* v, int cnt, int w) {
        std::vector<int4> o(cnt);
        for (int k = 0; k < cnt; ++k) o[k] = make_int4(v[w * k], v[w * k + 1], v[w * k + 2], w > 3 ? v[w * k + 3] : 0);
        return o;
    };
    std::vector<int4> qa = i4(b->qangles, b->nqangles, 3), qt = i4(b->qtorsions, b->nqtors, 4),
                      qi = i4(b->qimpropers, b->nqimps, 4);
    std::vector<int> qbc(b->qbond_code, b->qbond_code + (size_t)b->nqbonds * S),
        qac(b->qangle_code, b->qangle_code + (size_t)b->nqangles * S),
        qtc(b->qtorsion_code, b->qtorsion_code + (size_t)b->nqtors * S),
        qic(b->qimproper_code, b->qimproper_code + (size_t)b->nqimps * S);
    TRY(up((int4**)&d.bonds, bonds));
    TRY(up((double2**)&d.bondlib, bl));
    TRY(up((int4**)&d.angles, angles));
    TRY(up((double4_16a**)&d.anglib, al));
    TRY(up((int**)&d.tors, tors));
    TRY(up((double4_16a**)&d.torlib, tl));
    TRY(up((int**)&d.imps, imps));
    TRY(up((double2**)&d.implib, il));
    TRY(up((int2**)&d.qbonds, qb));
    TRY(up((int**)&d.qbond_code, qbc));
    TRY(up((double4_16a**)&d.qbondlib, qbl));
    TRY(up((int4**)&d.qangles, qa));
    TRY(up((int**)&d.qangle_code, qac));
    TRY(up((double4_16a**)&d.qanglib, qal));
    TRY(up((int4**)&d.qtors, qt));
    TRY(up((int**)&d.qtor_code, qtc));
    TRY(up((double4_16a**)&d.qtorlib, qtl));
    TRY(up((int4**)&d.qimps, qi));
    TRY(up((int**)&d.qimp_code, qic));
    TRY(up((double2**)&d.qimplib, qil));
    // Morse couplings: per Q term the first matching row, bond | breaking << 30
    auto couplings = [&](int nterm, int n, const int32_t* tab, const char* what, std::vector<int>* out) -> int {
        out->assign(std::max(nterm, 1), -1);
        for (int r = 0; r < n; ++r) {
            int q = tab[3 * r], ib = tab[3 * r + 1], br = tab[3 * r + 2];
            if (q < 0 || q >= nterm || ib < 0 || ib >= b->nqbonds || br < 0 || br > 1)
                return fail(QNB_ERR_ARG, "%s coupling %d out of range", what, r);
            if ((*out)[q] < 0) (*out)[q] = ib | (br << 30);
        }
        return QNB_OK;
    };
    std::vector<int> cpa, cpt, cpi;
    TRY(couplings(b->nqangles, b->nang_coupl, b->ang_coupl, "angle", &cpa));
    TRY(couplings(b->nqtors, b->ntor_coupl, b->tor_coupl, "torsion", &cpt));
    TRY(couplings(b->nqimps, b->nimp_coupl, b->imp_coupl, "improper", &cpi));
    TRY(up((int**)&d.qang_cpl, cpa));
    TRY(up((int**)&d.qtor_cpl, cpt));
    TRY(up((int**)&d.qimp_cpl, cpi));
    d.nb = b->nbonds; d.nb_sol = b->nbonds_solute;
    d.na = b->nangles; d.na_sol = b->nangles_solute;
    d.nt = b->ntors; d.nt_sol = b->ntors_solute;
    d.ni = b->nimps; d.ni_sol = b->nimps_solute;
    d.imp_type = b->imp_type;
    d.urey = b->urey_bradley != 0;
    d.nqb = b->nqbonds; d.nqa = b->nqangles; d.nqt = b->nqtors; d.nqi = b->nqimps;
    d.nterms = d.nb + d.na + d.nt + d.ni + S * (d.nqb + d.nqa + d.nqt + d.nqi);
    c->bonded = d;
    c->have_bonded = d.nterms > 0;
    ++c->epoch;   // captured graphs lack (or hold a stale) bonded launch
    return QNB_OK;
}

int qnb_get_bonded_energies(qnb_context* c, double* Eb, double* EQb) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    std::vector<double> e((size_t)kNumE * c->nwin);
    TRY(read_energies(c, c->nwin, e.data()));
    for (int w = 0; w < c->nwin; ++w) {
        double t[8 + 4 * kMaxStates];
        bonded_out(c, e.data() + (size_t)w * kNumE, t);
        if (Eb)
            for (int k = 0; k < 8; ++k) Eb[8 * w + k] = t[k];
        if (EQb)
            for (int k = 0; k < 4 * c->S; ++k) EQb[(size_t)w * 4 * c->S + k] = t[8 + k];
    }
    return QNB_OK;
}

}  // extern "C"

extern "C" {

int qnb_set_shell_restraint(qnb_context* c, const double* xtop, const uint8_t* shell, double fk_fix, double fk_pshell) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    if (c->d_shell_flags) c->release(c->d_shell_flags), c->d_shell_flags = nullptr;
    if (c->d_xtop) c->release(c->d_xtop), c->d_xtop = nullptr;
    c->have_shell = false;
    ++c->epoch;
    if (!xtop) return QNB_OK;   // removes the restraint
    if (!shell) return fail(QNB_ERR_ARG, "null shell flags");
    if (!(fk_fix >= 0.0) || !(fk_pshell >= 0.0)) return fail(QNB_ERR_ARG, "negative force constant");
    std::vector<uint8_t> excl(c->natom);
    CU(cudaMemcpy(excl.data(), c->d_excl_top, c->natom, cudaMemcpyDeviceToHost));
    std::vector<uint8_t> flags(c->natom);
    int any = 0;
    for (int i = 0; i < c->natom; ++i) {
        flags[i] = (uint8_t)((excl[i] ? 1u : 0u) | (shell[i] ? 2u : 0u));
        any |= flags[i];
    }
    std::vector<double> xt(xtop, xtop + 3 * (size_t)c->natom);
    TRY(c->upload(&c->d_shell_flags, flags));
    TRY(c->upload(&c->d_xtop, xt));
    c->fk_fix = fk_fix;
    c->fk_pshell = fk_pshell;
    c->have_shell = any != 0;
    return QNB_OK;
}

int qnb_get_restraint_energies(qnb_context* c, double* Er) {
    if (!c || !Er) return fail(QNB_ERR_ARG, "null argument");
    CU(cudaSetDevice(c->device));
    std::vector<double> e((size_t)kNumE * c->nwin);
    TRY(read_energies(c, c->nwin, e.data()));
    const size_t stride = 5 + (size_t)c->S;
    for (int w = 0; w < c->nwin; ++w) {
        const double* ew = e.data() + (size_t)w * kNumE;
        double* o = Er + stride * w;
        o[0] = ew[E_RST_FIX];
        o[1] = ew[E_RST_SHELL];
        o[2] = ew[E_RST_RAD];
        o[3] = ew[E_RST_POL];
        o[4] = ew[E_RST_PROT];
        for (int st = 0; st < c->S; ++st) o[5 + st] = ew[qr_slot(st)];
    }
    return QNB_OK;
}

}  // extern "C"

namespace {
// per-atom codes of the restraint atom selection: bit 0 heavy, bit 1 an
// excluded atom while excluded_freeze is on
int restraint_atom_codes(qnb_context* c, std::vector<uint8_t>* out) {
    out->assign(c->h_heavy.begin(), c->h_heavy.end());
    if (c->freeze) {
        std::vector<uint8_t> excl(c->natom);
        CU(cudaMemcpy(excl.data(), c->d_excl_top, c->natom, cudaMemcpyDeviceToHost));
        for (int i = 0; i < c->natom; ++i)
            if (excl[i]) (*out)[i] |= 2;
    }
    return QNB_OK;
}
}  // namespace

extern "C" {

int qnb_set_freeze(qnb_context* c, int32_t freeze) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    c->freeze = freeze ? 1 : 0;
    if (c->have_restr && c->restr.heavy) {
        std::vector<uint8_t> codes;
        TRY(restraint_atom_codes(c, &codes));
        CU(cudaMemcpy((void*)c->restr.heavy, codes.data(), codes.size(), cudaMemcpyHostToDevice));
    }
    ++c->epoch;
    return QNB_OK;
}

int qnb_set_restraints(qnb_context* c, const qnb_restraints* r, const double* xtop) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    for (void* p : c->restr_bufs) c->release(p);
    c->restr_bufs.clear();
    c->restr = RestrDev{};
    c->have_restr = false;
    ++c->epoch;
    if (!r) return QNB_OK;
    const int n = c->natom, S = c->S;
    if (r->nseq < 0 || r->npos < 0 || r->ndist < 0 || r->nang < 0 || r->nwall < 0)
        return fail(QNB_ERR_ARG, "negative restraint count");
    if ((r->nseq > 0 && (!r->seq_ij || !r->seq_fk || !r->seq_ih || !r->seq_mode || !xtop)) ||
        (r->npos > 0 && (!r->pos_i || !r->pos_state || !r->pos_x || !r->pos_fk)) ||
        (r->ndist > 0 && (!r->dist_ij || !r->dist_state || !r->dist_d || !r->dist_fk)) ||
        (r->nang > 0 && (!r->ang_ijk || !r->ang_state || !r->ang_theta || !r->ang_fk)) ||
        (r->nwall > 0 && (!r->wall_ij || !r->wall_d || !r->wall_fk || !r->wall_aMorse || !r->wall_dMorse || !r->wall_ih)))
        return fail(QNB_ERR_ARG, "null restraint array");
    auto atom = [&](int i) { return i >= 0 && i < n; };
    auto state = [&](int st) { return st >= -1 && st < S; };
    std::vector<int4> seq(r->nseq), dist(r->ndist), ang(r->nang), wall(r->nwall);
    std::vector<int2> pos(r->npos);
    std::vector<double> sfk(r->seq_fk ? r->seq_fk : nullptr, r->seq_fk ? r->seq_fk + r->nseq : nullptr);
    std::vector<double> pxf(6 * (size_t)r->npos), dp(3 * (size_t)r->ndist), ap(2 * (size_t)r->nang),
        wp(4 * (size_t)r->nwall);
    for (int k = 0; k < r->nseq; ++k) {
        int a = r->seq_ij[2 * k], b = r->seq_ij[2 * k + 1], md = r->seq_mode[k];
        if (!atom(a) || !atom(b) || a > b || md < 0 || md > 2) return fail(QNB_ERR_ARG, "sequence restraint %d", k);
        seq[k] = make_int4(a, b, r->seq_ih[k], md);
    }
    for (int k = 0; k < r->npos; ++k) {
        if (!atom(r->pos_i[k]) || !state(r->pos_state[k])) return fail(QNB_ERR_ARG, "position restraint %d", k);
        pos[k] = make_int2(r->pos_i[k], r->pos_state[k]);
        for (int cc = 0; cc < 3; ++cc) {
            pxf[6 * k + cc] = r->pos_x[3 * k + cc];
            pxf[6 * k + 3 + cc] = r->pos_fk[3 * k + cc];
        }
    }
    for (int k = 0; k < r->ndist; ++k) {
        int a = r->dist_ij[2 * k], b = r->dist_ij[2 * k + 1];
        if (!atom(a) || !atom(b) || !state(r->dist_state[k])) return fail(QNB_ERR_ARG, "distance restraint %d", k);
        dist[k] = make_int4(a, b, r->dist_state[k], 0);
        dp[3 * k] = r->dist_d[2 * k];
        dp[3 * k + 1] = r->dist_d[2 * k + 1];
        dp[3 * k + 2] = r->dist_fk[k];
    }
    const double deg2rad = 3.14159265358979323846 / 180.0;
    for (int k = 0; k < r->nang; ++k) {
        int a = r->ang_ijk[3 * k], b = r->ang_ijk[3 * k + 1], d = r->ang_ijk[3 * k + 2];
        if (!atom(a) || !atom(b) || !atom(d) || !state(r->ang_state[k])) return fail(QNB_ERR_ARG, "angle restraint %d", k);
        ang[k] = make_int4(a, b, d, r->ang_state[k]);
        ap[2 * k] = r->ang_theta[k] * deg2rad;
        ap[2 * k + 1] = r->ang_fk[k];
    }
    for (int k = 0; k < r->nwall; ++k) {
        int a = r->wall_ij[2 * k], b = r->wall_ij[2 * k + 1];
        if (!atom(a) || !atom(b) || a > b) return fail(QNB_ERR_ARG, "wall restraint %d", k);
        wall[k] = make_int4(a, b, r->wall_ih[k], 0);
        wp[4 * k] = r->wall_d[k];
        wp[4 * k + 1] = r->wall_fk[k];
        wp[4 * k + 2] = r->wall_aMorse[k];
        wp[4 * k + 3] = r->wall_dMorse[k];
    }
    RestrDev d{};
    d.nseq = r->nseq; d.npos = r->npos; d.ndist = r->ndist; d.nang = r->nang; d.nwall = r->nwall;
    auto up = [&](auto** dst, const auto& vec) -> int {
        int rc = c->upload(dst, vec);
        if (!rc) c->restr_bufs.push_back((void*)*dst);
        return rc;
    };
    std::vector<double> xt(xtop ? xtop : nullptr, xtop ? xtop + 3 * (size_t)n : nullptr);
    std::vector<double> mass(n, 0.0);
    std::vector<uint8_t> heavy;
    TRY(restraint_atom_codes(c, &heavy));
    if (c->md_ready) CU(cudaMemcpy(mass.data(), c->md.mass, sizeof(double) * n, cudaMemcpyDeviceToHost));
    for (int k = 0; k < r->nseq; ++k)
        if (seq[k].w == 1 || seq[k].w == 2)
            for (int i = seq[k].x; i <= seq[k].y; ++i)
                if (!(mass[i] > 0.0)) return fail(QNB_ERR_STATE, "centre restraints need the masses (qnb_md_init first)");
    TRY(up((int4**)&d.seq, seq));
    TRY(up((double**)&d.seq_fk, sfk));
    TRY(up((int2**)&d.pos, pos));
    TRY(up((double**)&d.pos_xfk, pxf));
    TRY(up((int4**)&d.dist, dist));
    TRY(up((double**)&d.dist_p, dp));
    TRY(up((int4**)&d.ang, ang));
    TRY(up((double**)&d.ang_p, ap));
    TRY(up((int4**)&d.wall, wall));
    TRY(up((double**)&d.wall_p, wp));
    TRY(up((double**)&d.xtop, xt));
    TRY(up((double**)&d.mass, mass));
    TRY(up((uint8_t**)&d.heavy, heavy));
    c->restr = d;
    c->have_restr = (r->nseq + r->npos + r->ndist + r->nang + r->nwall) > 0;
    return QNB_OK;
}

}  // extern "C"

extern "C" {

int qnb_set_offdiag(qnb_context* c, int32_t n, const int32_t* states, const int32_t* qatoms, const double* A,
                    const double* mu) {
    if (!c || n < 0 || (n > 0 && (!states || !qatoms || !A || !mu))) return fail(QNB_ERR_ARG, "null argument");
    for (int k = 0; k < n; ++k) {
        if (states[2 * k] < 0 || states[2 * k] >= c->S || states[2 * k + 1] < 0 || states[2 * k + 1] >= c->S)
            return fail(QNB_ERR_ARG, "offdiag %d: state out of range", k);
        if (qatoms[2 * k] < 0 || qatoms[2 * k] >= c->nqat || qatoms[2 * k + 1] < 0 || qatoms[2 * k + 1] >= c->nqat)
            return fail(QNB_ERR_ARG, "offdiag %d: Q atom out of range", k);
    }
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    for (void* p : c->offd_bufs) c->release(p);
    c->offd_bufs.clear();
    c->offd = OffdDev{};
    ++c->epoch;
    if (n == 0) return QNB_OK;
    std::vector<int> iqseq(c->nqat);
    CU(cudaMemcpy(iqseq.data(), c->m.iqseq, sizeof(int) * c->nqat, cudaMemcpyDeviceToHost));
    std::vector<int2> kl(n);
    std::vector<double2> am(n);
    for (int k = 0; k < n; ++k) {
        kl[k] = make_int2(iqseq[qatoms[2 * k]], iqseq[qatoms[2 * k + 1]]);
        am[k] = make_double2(A[k], mu[k]);
    }
    OffdDev o{};
    o.n = n;
    TRY(c->upload((int2**)&o.kl, kl));
    c->offd_bufs.push_back((void*)o.kl);
    TRY(c->upload((double2**)&o.Amu, am));
    c->offd_bufs.push_back((void*)o.Amu);
    TRY(c->alloc(&o.out, (size_t)2 * n * c->nwin));
    c->offd_bufs.push_back((void*)o.out);
    CU(cudaMemset(o.out, 0, sizeof(double) * 2 * n * c->nwin));
    c->offd = o;
    return QNB_OK;
}

int qnb_get_offdiag(qnb_context* c, double* Hij, double* rkl) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    const int n = c->offd.n;
    if (n == 0) return QNB_OK;
    std::vector<double> v((size_t)2 * n * c->nwin);
    CU(cudaMemcpyAsync(v.data(), c->offd.out, sizeof(double) * v.size(), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (size_t k = 0; k < (size_t)n * c->nwin; ++k) {
        if (Hij) Hij[k] = v[2 * k];
        if (rkl) rkl[k] = v[2 * k + 1];
    }
    return QNB_OK;
}

}  // extern "C"

// ---- listed pair sets: monitor groups and group contributions --------------
namespace {
PairSetEntry pset_entry(int i, int j, int soft, double A, double B, double el, double sc) {
    PairSetEntry e{};
    e.i = i;
    e.j = j;
    e.soft = soft;
    e.A = A;
    e.B = B;
    e.el = el;
    e.sc = sc;
    return e;
}
// the static Q-Q entry of Q atoms a < b (atom indices) in state s, or -1
int find_qq(const qnb_context* c, int a, int b, int s) {
    const auto& qq = c->psrc.qq;
    for (int k = 0; k < c->nqq_qq; ++k)
        if (qq[k].s == s && ((qq[k].i == a && qq[k].j == b) || (qq[k].i == b && qq[k].j == a))) return k;
    return -1;
}
// the Q-bonded-P entry of Q atom qa and solute atom j in state s, or -1
int find_qqp(const qnb_context* c, int qa, int j, int s) {
    const auto& qq = c->psrc.qq;
    for (int k = c->nqq_qq; k < (int)qq.size(); ++k)
        if (qq[k].s == s && qq[k].i == qa && qq[k].j == j) return k;
    return -1;
}
// Q atom (Q index iq) with non-Q solute atom j in state s: the Q-bonded-P
// entry when j is bonded or angled to a Q atom, else the q-p table; false
// when the pair does not interact (precompute's `set` off, or 1-2/1-3 to Q)
bool q_pair(const qnb_context* c, int iq, int j, int s, PairSetEntry* e) {
    const auto& ps = c->psrc;
    const int nq = c->nqat, S = c->S;
    const int qa = ps.iqseq[iq];
    if (ps.qnear[j]) {
        int k = find_qqp(c, qa, j, s);
        if (k < 0) return false;
        const QQEntry& q = ps.qq[k];
        *e = pset_entry(qa, j, 0, q.A, q.B, q.el, q.sc);
        return true;
    }
    size_t o = ((size_t)j * nq + iq) * S + s;
    if (!ps.qp_set[o]) return false;
    const QPar& p = ps.qp[o];
    *e = pset_entry(qa, j, 0, p.A, p.B, p.el, p.sc);
    return true;
}
// two non-Q solute atoms: pp_precomp's values (src/simprep.f90:3321-3351);
// false for excluded pairs and pairs that do not interact
bool p_pair(const qnb_context* c, int a, int b, PairSetEntry* e) {
    const auto& ps = c->psrc;
    int i = std::min(a, b), j = std::max(a, b);
    long long key = (long long)i * c->natom + j;
    auto it = std::lower_bound(ps.special.begin(), ps.special.end(), std::make_pair(key, 0));
    int code = ps.ljcod[(size_t)ps.iac[i] * ps.nt + ps.iac[j]];
    if (it != ps.special.end() && it->first == key) {
        if (it->second == 1) return false;
        code = 3;
    }
    double2 lj = ps.lj[((size_t)(code - 1) * ps.nt + ps.iac[i]) * ps.nt + ps.iac[j]];
    double el = ps.crg[i] * ps.crg[j];
    if (!(fabs(lj.x) > kQrealEps || fabs(lj.y) > kQrealEps || fabs(el) > kQrealEps)) return false;
    if (code == 3) el *= ps.el14;
    *e = pset_entry(i, j, 0, lj.x, lj.y, el, 0.0);
    return true;
}
// concatenates the monitor and exclusion lists into the device list
int upload_pair_sets(qnb_context* c) {
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    for (void* p : c->pset_bufs) c->release(p);
    c->pset_bufs.clear();
    c->psets = PairSetDev{};
    ++c->epoch;
    const int nslots = (int)(c->mon_first.size() + c->exc_first.size());
    if (nslots == 0) return QNB_OK;
    std::vector<PairSetEntry> e(c->mon_e);
    e.insert(e.end(), c->exc_e.begin(), c->exc_e.end());
    if (e.empty()) e.push_back(PairSetEntry{});   // keeps the buffer non-empty
    std::vector<int> first(1, 0);
    for (int n : c->mon_first) first.push_back(first.back() + n);
    for (int n : c->exc_first) first.push_back(first.back() + n);
    PairSetDev p{};
    p.nslots = nslots;
    TRY(c->upload((PairSetEntry**)&p.e, e));
    c->pset_bufs.push_back((void*)p.e);
    TRY(c->upload((int**)&p.slot_first, first));
    c->pset_bufs.push_back((void*)p.slot_first);
    TRY(c->alloc(&p.out, (size_t)2 * nslots * c->nwin));
    c->pset_bufs.push_back((void*)p.out);
    CU(cudaMemset(p.out, 0, sizeof(double) * 2 * nslots * c->nwin));
    c->psets = p;
    return QNB_OK;
}
int read_pair_sets(qnb_context* c, int first, int n, double* out) {
    CU(cudaSetDevice(c->device));
    if (n == 0 || c->psets.nslots == 0) return QNB_OK;
    std::vector<double> v((size_t)2 * c->psets.nslots * c->nwin);
    CU(cudaMemcpyAsync(v.data(), c->psets.out, sizeof(double) * v.size(), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    for (int w = 0; w < c->nwin; ++w)
        for (int k = 0; k < n; ++k) {
            out[((size_t)w * n + k) * 2] = v[((size_t)w * c->psets.nslots + first + k) * 2];
            out[((size_t)w * n + k) * 2 + 1] = v[((size_t)w * c->psets.nslots + first + k) * 2 + 1];
        }
    return QNB_OK;
}
}  // namespace

extern "C" {

int qnb_set_monitor_groups(qnb_context* c, int32_t ngroups, const int32_t* group_first, const int32_t* atoms,
                           int32_t npairs, const int32_t* pairs) {
    if (!c || ngroups < 0 || npairs < 0 || (npairs > 0 && (!group_first || !atoms || !pairs)))
        return fail(QNB_ERR_ARG, "null argument");
    for (int g = 0; npairs > 0 && g < ngroups; ++g) {
        if (group_first[g] < 0 || group_first[g + 1] < group_first[g])
            return fail(QNB_ERR_ARG, "monitor group %d: bad group_first", g);
        for (int k = group_first[g]; k < group_first[g + 1]; ++k)
            if (atoms[k] < 0 || atoms[k] >= c->nat_solute)
                return fail(QNB_ERR_ARG, "monitor group %d: atom %d is not a solute atom", g, atoms[k]);
    }
    for (int p = 0; p < npairs; ++p)
        if (pairs[2 * p] < 0 || pairs[2 * p] >= ngroups || pairs[2 * p + 1] < 0 || pairs[2 * p + 1] >= ngroups)
            return fail(QNB_ERR_ARG, "monitor pair %d: group out of range", p);
    const auto& ps = c->psrc;
    const int S = c->S;
    std::vector<PairSetEntry> ent;
    std::vector<int> cnt;
    // nbmonitorlist, src/nonbondene.f90:4517-4630: per pair and state, every
    // interacting atom pair of the two groups
    for (int p = 0; p < npairs; ++p) {
        const int gi = pairs[2 * p], gj = pairs[2 * p + 1];
        std::vector<std::vector<PairSetEntry>> per(S);
        for (int a = group_first[gi]; a < group_first[gi + 1]; ++a)
            for (int b = group_first[gj]; b < group_first[gj + 1]; ++b) {
                const int i = atoms[a], j = atoms[b];
                if (i == j) return fail(QNB_ERR_ARG, "two paired monitor atom groups contain the same atom %d", i);
                const int qi = ps.iqatom[i], qj = ps.iqatom[j];
                PairSetEntry e;
                for (int s = 0; s < S; ++s) {
                    if (qi >= 0 && qj >= 0) {
                        int k = find_qq(c, std::min(i, j), std::max(i, j), s);
                        if (k < 0) continue;
                        const QQEntry& q = ps.qq[k];
                        per[s].push_back(pset_entry(q.i, q.j, q.soft, q.A, q.B, q.el, q.sc));
                    } else if (qi >= 0 || qj >= 0) {
                        if (q_pair(c, qi >= 0 ? qi : qj, qi >= 0 ? j : i, s, &e)) per[s].push_back(e);
                    } else if (p_pair(c, i, j, &e)) {
                        per[s].push_back(e);
                    }
                }
            }
        for (int s = 0; s < S; ++s) {
            cnt.push_back((int)per[s].size());
            ent.insert(ent.end(), per[s].begin(), per[s].end());
        }
    }
    c->mon_e.swap(ent);
    c->mon_first.swap(cnt);
    c->mon_pairs = npairs;
    return upload_pair_sets(c);
}

int qnb_get_monitor_energies(qnb_context* c, double* out) {
    if (!c || (!out && c->mon_pairs > 0)) return fail(QNB_ERR_ARG, "null argument");
    return read_pair_sets(c, 0, c->mon_pairs * c->S, out);
}

int qnb_set_group_exclusions(qnb_context* c, int32_t ngroups, const uint8_t* mask) {
    if (!c || ngroups < 0 || (ngroups > 0 && !mask)) return fail(QNB_ERR_ARG, "null argument");
    const auto& ps = c->psrc;
    const int S = c->S, nq = c->nqat, ns = c->nat_solute;
    std::vector<PairSetEntry> ent;
    std::vector<int> cnt;
    // per group and state two slots: the Q-Q pairs with an atom in the group,
    // then the Q-P pairs (Q-bonded-P and plain) whose solute atom is in it
    for (int g = 0; g < ngroups; ++g) {
        const uint8_t* mk = mask + (size_t)g * ns;
        for (int s = 0; s < S; ++s) {
            int n0 = (int)ent.size();
            for (int k = 0; k < c->nqq_qq; ++k) {
                const QQEntry& q = ps.qq[k];
                if (q.s == s && (mk[q.i] || mk[q.j]))
                    ent.push_back(pset_entry(q.i, q.j, q.soft, q.A, q.B, q.el, q.sc));
            }
            cnt.push_back((int)ent.size() - n0);
            n0 = (int)ent.size();
            for (int j = 0; j < ns; ++j) {
                if (!mk[j] || ps.iqatom[j] >= 0) continue;
                for (int iq = 0; iq < nq; ++iq) {
                    PairSetEntry e;
                    if (q_pair(c, iq, j, s, &e)) ent.push_back(e);
                }
            }
            cnt.push_back((int)ent.size() - n0);
        }
    }
    c->exc_e.swap(ent);
    c->exc_first.swap(cnt);
    c->exc_groups = ngroups;
    return upload_pair_sets(c);
}

int qnb_get_group_exclusions(qnb_context* c, double* out) {
    if (!c || (!out && c->exc_groups > 0)) return fail(QNB_ERR_ARG, "null argument");
    return read_pair_sets(c, c->mon_pairs * c->S, c->exc_groups * c->S * 2, out);
}

int qnb_set_box(qnb_context* c, const double* boxlength, int32_t qswitch) {
    if (!c) return fail(QNB_ERR_ARG, "null context");
    CU(cudaSetDevice(c->device));
    CU(cudaStreamSynchronize(c->stream));
    if (!boxlength) {
        c->m.box = 0;
        c->m.box_rows = 0;
        c->m.excl = c->d_excl_top;
        use_lrf_tables(c, 0);
    } else {
        for (int k = 0; k < 3; ++k)
            if (!(boxlength[k] > 0.0)) return fail(QNB_ERR_ARG, "box length %d must be positive", k);
        if (c->nqat > 0 && (qswitch < 0 || qswitch >= c->natom))
            return fail(QNB_ERR_ARG, "switching atom %d out of range", qswitch);
        if (c->have_solv) return fail(QNB_ERR_UNSUPPORTED, "solvent restraints are for the sphere");
        c->m.box = 1;
        c->m.box_rows = c->mixed && !c->m.any_atom ? 1 : 0;
        c->m.excl = c->d_excl_none;   // the box lists, lrf_taylor and temperature() test no exclusion
        use_lrf_tables(c, 1);
        c->m.qswitch = qswitch;
        for (int k = 0; k < 3; ++k) {
            c->m.boxl[k] = boxlength[k];
            c->m.inv_boxl[k] = 1.0 / boxlength[k];
            c->m.boxlf[k] = (float)c->m.boxl[k];
            c->m.inv_boxlf[k] = (float)c->m.inv_boxl[k];
        }
    }
    c->lists_built = false;
    c->qp_done = c->qw_done = false;
    ++c->epoch;
    return QNB_OK;
}

}  // extern "C"
