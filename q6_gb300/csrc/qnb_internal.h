// Internal declarations shared by the host layer and the CUDA kernels of the
// qdyn nonbonded engine.  Nothing here is part of the public ABI (qnb.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/qnb.h"

namespace qnb {

constexpr int kMaxSolv = 4;     // atoms per solvent molecule handled on device
constexpr int kMaxStates = 8;   // FEP states
constexpr int kMaxShell = 16;   // water polarisation shells
constexpr int kLrfLen = 43;     // cgp_cent(3) phi0 phi1(3) phi2(9) phi3(27)
constexpr int kLrfMoments = 24; // symmetric moments the LRF accumulation sums per target group
constexpr int kLrfSplitMax = 8; // source ranges of the mixed form's LRF accumulation
constexpr double kFix = 4294967296.0;   // 2^32: fixed-point quantum of forces/energies
constexpr float kFixF = 4294967296.0f;

// energy slots (doubles in FP64 mode, 2^-32 fixed point in mixed mode)
enum {
    E_PP_EL = 0, E_PP_VDW, E_PW_EL, E_PW_VDW, E_WW_EL, E_WW_VDW, E_LRF,
    E_RST_RAD, E_RST_POL, E_RST_FIX, E_RST_SHELL, E_RST_PROT, E_Q0
};
__host__ __device__ constexpr int eq_slot(int s, int k) { return E_Q0 + 6 * s + k; }
// bonded: solute bond, angle, torsion, improper, then the same for solvent;
// then per state the Q bond, angle, torsion, improper
constexpr int E_B0 = E_Q0 + 6 * kMaxStates;
constexpr int E_QB0 = E_B0 + 8;
__host__ __device__ constexpr int qb_slot(int s, int k) { return E_QB0 + 4 * s + k; }
constexpr int E_QR0 = E_QB0 + 4 * kMaxStates;   // per state: EQ(s)%restraint
__host__ __device__ constexpr int qr_slot(int s) { return E_QR0 + s; }
constexpr int kNumE = E_QR0 + kMaxStates;

// list counters (entries at list granularity, plus reference atom-pair counts)
enum { C_WW = 0, C_PW, C_PP, C_QP, C_QW, C_PP14, C_PPG,
       C_RGP, C_RGW, C_RWW, C_RWG, C_RGF,   // longest row seen (mixed-form row lists)
       C_NUM };

constexpr int kMaxGroup = 15;   // atoms per solute charge group handled on device
constexpr int kMaxTypesShared = 32;   // type-pair table staged in shared memory up to this many types

struct alignas(32) QPar {   // one (pair type, state) parameter set: A, B, elec, soft-core alpha
    double A, B, el, sc;
};
struct alignas(16) QParF {
    float A, B, el, sc;
};

// Adjoint factors of one Q pair term E = el/r + A u^2 - B u, u = 1/(r^6 + alpha),
// for the Q atom's charge and code-1 LJ factors a, b:
//   dE/dq = c / r,  dE/da = a2 u^2 + a1 u,  dE/db = b2 u^2 + b1 u.
// Geometric rule: a2 = a_other, b1 = -b_other, a1 = b2 = 0.  Arithmetic rule,
// S = a + a_other: a2 = 12 S^11 b b_other, a1 = -12 S^5 b b_other,
// b2 = S^12 b_other, b1 = -2 S^6 b_other.  The LJ factors are zero where the Q
// side does not use its code-1 factor (1-4 pairs, soft pairs).
struct alignas(16) QAdjF {
    double c, a2, a1, b2, b1, pad;
};
// The same for a static Q pair: Q atom iq and, for Q-Q pairs, jq (jq = -1
// for a Q-bonded solute partner).
struct QQAdj {
    int iq, jq, s, pad;
    QAdjF fi, fj;
};

// Static model on the device.  Passed by value to kernels.
struct DevModel {
    int natom, nat_solute, nwat, sa, ncgp, ncgp_solute, natyps, nqat, S;
    int spc;           // SPC fast path for ww / qw (geometric rule + SPC solvent)
    int use_lrf;
    int any_atom;      // 1: a group pair is inside when any atom pair is (switch atoms off)
    int type_in_entry; // solute row entries carry the partner's LJ type (groups of <= 8 atoms)
    double el14;
    float el14f;       // el14 rounded to FP32 once, for the FP32 pair kernels
    const int* iac;
    const double* crg;
    const int* iqatom;          // -1 or Q index
    const uint8_t* excl;
    const int* gslot;           // [ncgp+1] offsets into gatom
    const int* gatom;           // group member atoms
    const int* gsw;             // [ncgp] switch atoms
    // solute group pairs holding excluded or 1-4 atom pairs: sorted keys
    // g1*ncgp_solute+g2 (g1 <= g2), each with a run of entries
    // (slot in g1) | (slot in g2) << 8 | kind << 16, kind 1 excluded / 3 1-4;
    // inside one group the slots are ordered by atom index
    int nsg;
    const long long* sg_key;
    const int* sg_off;          // [nsg+1]
    const int* sg_ent;
    // per solute group its special group pairs: sgl_ent[sgl_off[g] ..
    // sgl_off[g+1]) = (partner group, sg index), the group itself included
    const int* sgl_off;
    const int2* sgl_ent;
    // per special group pair (lower group gl, upper gu): the 2-bit kinds of
    // every row atom against each partner atom, sgm[sgm_off[sg] + b] for row gl
    // and partner b of gu (for gl == gu the atom itself is kind 1), then
    // sgm[sgm_off[sg] + n(gu) + b] for row gu and partner b of gl
    const int* sgm_off;
    const unsigned* sgm;
    const double2* lj;          // [3][natyps][natyps] (A,B) per LJ code 1..3
    const float2* ljf;
    const float4* ljpair;       // [natyps][natyps]: (A,B) of ljcod code, (A,B) of code 3
    const uint8_t* ljcod;       // [natyps][natyps]
    const uint8_t* ljset;       // [3][natyps][natyps]: |A| or |B| > QREAL_EPS
    int wtype[kMaxSolv];        // solvent template (first molecule) atom types
    unsigned wlj_mask;          // bit a: template atom a has LJ parameters with some solute type
    double wcrg[kMaxSolv];      // and charges
    float wcrgf[kMaxSolv];
    double wwA[kMaxSolv * kMaxSolv], wwB[kMaxSolv * kMaxSolv], wwE[kMaxSolv * kMaxSolv];  // ww_precomp
    float wwAf[kMaxSolv * kMaxSolv], wwBf[kMaxSolv * kMaxSolv], wwEf[kMaxSolv * kMaxSolv];
    const int* iqseq;           // [nqat]
    const QPar* qp_tab;         // [nat_solute][nqat][S]
    const QParF* qp_tabf;
    const QParF* qp_tabft;      // [nqat][nat_solute][S] (the transposed Q kernel's order)
    const QPar* qw_tab;         // [nqat][sa][S]
    const QParF* qw_tabf;
    // adjoint factors with the layouts of qp_tab / qw_tab
    const QAdjF* qp_adj;
    const QAdjF* qw_adj;
    const QQAdj* qq_adj;        // parallel to the static Q-Q / Q-bonded list
    double xpcent[3], xwcent[3];
    float wcoff[3];             // xpcent - xwcent in FP32: packed (xpcent-centred) coordinates to xwcent-centred
    double rexcl_o2;
    // plain solute partners of the mixed form's solute rows: per solute group
    // the partner types that need the general pair path (some non-Q atom of
    // the group has LJ code 2 with them; all bits set when there are more
    // than 128 types), and per atom its code-1 LJ factors in FP32 (geometric
    // rule: A = a_i a_j, B = b_i b_j)
    int geom;
    const ulonglong2* gtmask;           // [ncgp_solute] types 0-63 (x) and 64-127 (y)
    const uint8_t* gallq;               // [ncgp_solute] 1: every atom of the group is a Q atom (no pair row)
    const float2* ljf1;                 // [natom]
    // LRF sources grouped by charge group (mixed form's accumulation):
    // groups with LRF-eligible atoms (non-Q atoms of groups whose distance
    // atom is not excluded), their distance atom | solute flag << 30, and
    // the offsets of their atoms in lrf_gatom (group-major)
    int nlrf_groups;
    const int* lrf_gmeta;       // [nlrf_groups]
    const int* lrf_goff;        // [nlrf_groups + 1]
    const int* lrf_gatom;       // [lrf_goff[nlrf_groups]]
    // periodic box (qnb_set_box): rectangular box lengths, their inverses
    // and the Q-list switching atom (FEP file [PBC] switching_atom)
    int box;
    int qswitch;
    double boxl[3], inv_boxl[3];
    float boxlf[3], inv_boxlf[3];   // FP32 copies (set on the host)
    int box_rows;                   // 1: the mixed form's box path runs on the gather rows
    const int* swat;                // [natom] the reference (switch) atom of the atom's unit
    // FP32 copies are stored relative to xpcent, which bounds their magnitude
    // by the sphere size (FP32 cut-off prefilter and mixed-form pair math)
};

struct QQEntry {   // static Q-Q / Q-bonded-P pair of one state
    int i, j, s, soft;      // atom indices (not Q indices), state, exp-repulsion flag
    double A, B, el, sc;
};


// Geometry of a window's cell grid: cell (ix, iy, iz) of a point p holds
// ix = clamp(trunc((p.x - lo.x) * inv_h), 0, nx - 1), likewise y and z; cell
// index (iz * ny + iy) * nx + ix.  1 / inv_h is at least half the largest
// cut-off plus a margin, so the partners of an atom lie within +-2 cells.
struct CellGrid {
    float lox, loy, loz, inv_h;
    int nx, ny, nz, ncell;
};
// In a periodic box the grid divides each box edge into n cells (n >= 5, so
// the +-2 stencil never meets itself across the boundary): a point's cell is
// trunc(frac(p / L) * n), and the stencil wraps modulo n.
constexpr int kCellCap = 32768;   // cells per window; a larger extent gets larger cells

// Per-context device state of the lists, coordinates and accumulators.
struct DevState {
    double* x;           // [natom*3] coordinates (FP64, as qdyn holds them)
    const double* md_tfree;   // Tfree of the window's last MD temperature() (null before qnb_md_init)
    double* d;           // [natom*3] gradient accumulator (FP64 mode target)
    float4* xq;          // [natom] FP32 (x,y,z,charge) for the mixed form
    float* frow;         // [natom*3] mixed form: row-kernel gradient of each atom's own row (FP32 warp sum)
    float* fq;           // [natom*3] mixed form: Q-environment gradient of each listed qp atom / qw water
    unsigned long long* fix;   // [natom*3] fixed-point gradient (mixed form)
    double* e;           // [kNumE] FP64 energies
    unsigned long long* efix;  // [kNumE] fixed-point energies (mixed form)
    double* lambda;      // [S]
    double* lrf;         // [ncgp*43]
    double* lrf_part;    // mixed form: [kLrfSplitMax][ncgp][kLrfMoments] LRF moments per source range
    int* cnt;            // [C_NUM] list sizes (device-maintained)
    int2* ww; int64_t cap_ww;      // water pairs (iw, jw), iw < jw
    int2* pw; int64_t cap_pw;      // (solute atom, water)
    int2* pp; int64_t cap_pp;      // (i, j | code << 28)
    int2* ppg; int64_t cap_ppg;    // listed solute group pairs (g1 <= g2)
    int* qp;  int64_t cap_qp;      // solute atoms interacting with all Q atoms
    int* qw;  int64_t cap_qw;      // waters interacting with all Q atoms
    // mixed form: gather rows (ELL, fixed capacity per row); row r of list X
    // holds partners at X[r*cap_X .. r*cap_X + cnt_X[r])
    uint2* row_gp; int* cnt_gp; int cap_gp; // solute group -> solute atoms needing the general pair path:
                                            // {j | flags, 2-bit kind per row atom}
    int* row_gf; int* cnt_gf; int cap_gf;   // solute group -> plain solute partners (code 1 with every row atom)
    int* row_gw; int* cnt_gw; int cap_gw;   // solute group -> waters
    int* row_ww; int* cnt_ww; int cap_rww;  // water -> waters
    int* row_wg; int* cnt_wg; int cap_wg;   // water -> solute groups
    // mixed form, switch-atom cut-offs: the cell grid of the row build.  The
    // non-excluded group switch atoms (bin_s) and water oxygens (bin_w) are
    // binned on one uniform grid; cell c holds bin_X[c ? cend_X[c-1] : 0 ..
    // cend_X[c]) in ascending index order, each entry the atom's FP32
    // position with the group or water index in w
    CellGrid* grid; int* cend_s; int* cend_w; float4* bin_s; float4* bin_w; int cap_cells;
    double* x_build;                        // coordinates of the last list build
    QQEntry* qq; int nqq;          // static qq + qqp entries (all states)
    const float4* qqf;   // the entries' (A, B, el, sc) in FP32 (mixed form)
    const float* lambdaf;   // [S] lambda in FP32 (mixed form)
    double* adj;                   // [3][nqat*S] dE_s/dqcrg, dE_s/dqA, dE_s/dqB of this window
    int nqq_qq;                    // first nqq_qq entries are Q-Q (EQ%qq), rest Q-P (EQ%qp)
    // water polarisation
    double* theta;       // [nwat]
    double* rkey;        // [nwat] selection-sort key (theta; 1 - cos theta in the mixed form)
    double* wvec;        // [nwat][8] unit dipole / radial vectors and lengths of the last md call
    int* shell;          // [nwat] shell or -1
    int* rank;           // [nwat]
    int* n_insh;         // [kMaxShell]
    int* shell_list;     // [kMaxShell][nwat] waters per shell
    double* wstate;      // [3*kMaxShell]: theta_corr, avtheta, avn_insh
    double* shell_tsum;  // [kMaxShell] per-step sum of theta per shell (in sorted order)
    double* theta_sorted;   // [kMaxShell][nwat] the shell's thetas by rank
};

// ---- launch wrappers (qnb_kernels.cu) ---------------------------------------
// FP32 decision band of a squared cut-off c: an FP32 distance below lo is
// inside, above hi outside, in between the FP64 distance decides.  Computed
// on the host: a double-to-float conversion in a kernel runs on GB300's
// narrow FP64 pipe, and under register pressure the compiler may redo it
// inside a loop.
struct CutBand {
    float lo, hi;
};
inline CutBand cut_band(double c) {
    float f = (float)c;
    return CutBand{f * 0.9998f, f * 1.0002f};
}
struct Cut {
    double rcq2, rlrf2, rcpp2, rcpw2, rcww2;
    CutBand fq, flrf, fpp, fpw, fww;   // cut_band of each, filled by make_cut
};
inline Cut make_cut(double rcq2, double rlrf2, double rcpp2, double rcpw2, double rcww2) {
    return Cut{rcq2, rlrf2, rcpp2, rcpw2, rcww2, cut_band(rcq2), cut_band(rlrf2), cut_band(rcpp2),
               cut_band(rcpw2), cut_band(rcww2)};
}

// Every launch covers all nwin windows of a context (grid.y = window); s0 is
// window 0's host-side state (capacities are equal across windows) and ds the
// device array of all windows' states.
// Launch geometry chosen by the autotuner (qnb_autotune): blocks per SM of
// the per-step kernels and of the list build, and the Q-kernel chunk size
enum TuneParam { T_ROWS_SOLUTE, T_ROWS_WATER, T_QP, T_QW, T_QCHUNK, T_TAYLOR, T_LRF, T_BUILD, T_NUM };
struct Tune {
    int v[T_NUM];
};
constexpr Tune kTuneDefault = {{16, 16, 8, 8, 8, 16, 3, 16}};

struct Launch {
    const DevModel& m;
    const DevState& s0;
    const DevState* ds;
    int nwin;
    cudaStream_t st;
    const Tune& tu;
};

void launch_pack(const Launch& L);
void launch_reset_counts(const Launch& L, unsigned keep_mask);
void launch_group_centres(const Launch& L);
void launch_build_ww(const Launch& L, const Cut& c);
void launch_build_pw(const Launch& L, const Cut& c);
void launch_build_pp(const Launch& L, const Cut& c);
void launch_build_qp(const Launch& L, const uint8_t* qnear, double rcq2);
void launch_build_qw(const Launch& L, const Cut& c);
int launch_lrf_accumulate(const Launch& L, const Cut& c, int mixed, const int* lrf_src);

int launch_build_rows(const Launch& L, const Cut& c);
// cells per box edge for the periodic row build (0: too few cells, the rows
// take every candidate)
int box_cells(const DevModel& m, const Cut& c, int* n);
// the box half lists for inspection (pp group pairs expanded, pw, ww)
void launch_build_box_pairs(const Launch& L, const Cut& c);
void launch_rows_solute(const Launch& L, int maxg);
void launch_rows_water(const Launch& L);
void launch_ww(const Launch& L, int mixed);
void launch_qw(const Launch& L, int mixed);
void launch_pw(const Launch& L, int mixed);
void launch_pp(const Launch& L, int mixed);
void launch_qp(const Launch& L, int mixed);
void launch_nonbond_qq(const Launch& L, int mixed);
void launch_lrf_taylor(const Launch& L, const int* iwhich, int mixed);
void launch_apply_fixed(const Launch& L, int rows, int qenv);
void launch_clear_fq(const Launch& L);
void launch_solvent_internal(const Launch& L, const int2* ij, const double* par, int n, int mixed);

// kernel classes timed by the optional event profiler
enum { K_WW = 0, K_QW, K_PW, K_PP, K_QP, K_LRF_TAYLOR, K_QQ, K_RESTRAIN, K_WATPOL, K_PACK, K_APPLY,
       K_BUILD, K_LRF_BUILD, K_BONDED, K_MD, K_NUM };

struct SolventDev {
    double fk_wsphere, Dwmz, awmz, rwat, boltz, fkwpol, itdis;
    int wpol, nshell;
    double rout[kMaxShell], dr[kMaxShell], cstb[kMaxShell];
    // FP32 copies for the mixed form's restraint kernels
    float fk_wspheref, Dwmzf, awmzf, fkwpolf, cstbf[kMaxShell];
};
// Tfree < 0: every window's Tfree is read on the device (DevState::md_tfree)
void launch_restrain_solvent(const Launch& L, const SolventDev& p, double Tfree, int mixed, const int* wsw,
                             const uint8_t* heavy_solv);
int launch_watpol(const Launch& L, const SolventDev& p, int istep, int md, int mixed);

void launch_q_adjoint(const Launch& L);

void launch_export_pairs(const Launch& L, int win, int kind, int32_t* di, int32_t* dj, int64_t cap,
                         int* dcount);

// ---- bonded terms (FP64 in both forms) ---------------------------------------
struct BondedDev {
    int nb, nb_sol, na, na_sol, nt, nt_sol, ni, ni_sol;
    const int4* bonds;      // i j code -
    const double2* bondlib; // fk b0
    const int4* angles;     // i j k code
    const double4_16a* anglib;  // fk theta0 ureyfk ureyr0
    const int* tors;        // [5n] i j k l code
    const double4_16a* torlib;  // fk rmult delta 1/paths
    const int* imps;        // [5n]
    const double2* implib;  // fk phi0
    int imp_type, urey;
    int nqb, nqa, nqt, nqi;
    const int2* qbonds; const int* qbond_code;   // [n], [n*S]
    const double4_16a* qbondlib;                     // Dmz amz r0 fk
    const int4* qangles; const int* qangle_code; // i j k -
    const double4_16a* qanglib;
    const int4* qtors; const int* qtor_code;
    const double4_16a* qtorlib;                      // fk rmult delta -
    const int4* qimps; const int* qimp_code;
    const double2* qimplib;
    // Morse couplings per Q angle / torsion / improper: -1, or the Q bond | breaking << 30
    const int* qang_cpl; const int* qtor_cpl; const int* qimp_cpl;
    int nterms;             // classical terms + Q terms x states
};
void launch_bonded(const Launch& L, const BondedDev& b, int mixed);
// p_restrain: the input's restraint sections
struct RestrDev {
    int nseq, npos, ndist, nang, nwall;
    const int4* seq;        // first, last, include-hydrogens, mode
    const double* seq_fk;
    const int2* pos;        // atom, state (-1 all)
    const double* pos_xfk;  // [6n] x0 y0 z0 fkx fky fkz
    const int4* dist;       // i, j, state, -
    const double* dist_p;   // [3n] d1 d2 fk
    const int4* ang;        // i, j, k, state
    const double* ang_p;    // [2n] theta0 (rad) fk
    const int4* wall;       // first, last, include-hydrogens, -
    const double* wall_p;   // [4n] d fk aMorse dMorse
    const double* xtop;     // [natom*3]
    const double* mass;     // [natom]
    const uint8_t* heavy;   // [natom]
};
void launch_restraints(const Launch& L, const RestrDev& r, int mixed);
// offdiag: Hij = A exp(-mu r_kl) per window, out[(w*n + io)*2] = Hij, rkl
struct OffdDev {
    int n;
    const int2* kl;          // atom indices of the two Q atoms
    const double2* Amu;      // A, mu
    double* out;             // [nwin][n][2]
};
void launch_offdiag(const Launch& L, const OffdDev& o);
// listed pair energies (monitor groups, group-contribution exclusions): the
// entries of slot k are [slot_first[k], slot_first[k+1]); each slot's Coulomb
// and LJ sums are written to out[(w*nslots + k)*2 + {0,1}]
struct alignas(16) PairSetEntry {
    int i, j, soft, pad;
    double A, B, el, sc;
};
struct PairSetDev {
    int nslots;
    const PairSetEntry* e;
    const int* slot_first;   // [nslots+1]
    double* out;             // [nwin][nslots][2]
};
void launch_pair_sets(const Launch& L, const PairSetDev& p);
// periodic box: list builds (pp, pw, ww, qp, qw) with minimum-image tests and
// the box energy kernels (nonbond_*_box); FP64 pair arithmetic in the FP64
// form, FP32 in the mixed form
void launch_build_box(const Launch& L, const Cut& c, const uint8_t* qnear, int pairs);
int launch_box_nonbond(const Launch& L, int md, int mixed, const int* iwhich, double rcq2, int pairs);
// fix_shell: flag bit 0 excluded (fk_fix), bit 1 shell (fk_pshell); xtop [natom*3]
void launch_fix_shell(const Launch& L, const uint8_t* flags, const double* xtop, double fk_fix, double fk_pshell,
                      int mixed, int freeze, double* v);

// ---- device-resident MD step (FP64) ----------------------------------------
constexpr int kMaxTg = 4;          // temperature coupling groups
constexpr int kShakeMaxIter = 1000;   // CONST_MAX_ITER, src/globals.f90:520
constexpr int kMaxNh = 10;         // Nose-Hoover chain length (qdyn's default numchain)
struct MdWin {                     // per window, device
    double sfact[kMaxTg];          // Berendsen factors of the next newvel
    double xnh[kMaxNh], vnh[kMaxNh], qnh[kMaxNh];   // Nose-Hoover chain (nh_prop)
    double nh_s;                   // the last nh_prop's velocity scale
    double temp, tfree, ekin;      // last temperature()
    double tg_temp[kMaxTg], tg_tfree[kMaxTg], tg_texcl[kMaxTg];
    unsigned long long shake_iters;   // SHAKE iterations of the last step, summed over molecules
    double min_oldmax, min_scale, min_maxf;   // steepest descent: previous largest force, scale, largest force
    int min_state;                 // last minimisation step: 0 grown, 1 reset, 2 converged
    int pad;
};
struct MdDev {
    int natom, ntg, nmol;
    int thermostat;                // 0 Berendsen, 1 Nose-Hoover, 2 Langevin (qnb_md_set_thermostat / _langevin)
    int vv;                        // velocity Verlet: half-step force updates before and after the move
    int nhchains;
    double nhq;                    // Nose-Hoover mass
    double lan_friction, lan_gkT;  // Langevin: friction, 24 friction Boltz Temp0 / step (uniform draws)
    unsigned long long lan_seed;
    int istep;                     // the step newvel integrates (Langevin random-force counter)
    // put_back_in_box (qnb_set_put_back_in_box): molecules as atom lists
    int pb_nmol, pb_first_mol, pb_last_mol;   // molecules [pb_first_mol, pb_last_mol) are wrapped
    const int* pb_mol_first;       // [nmol+1]
    const int* pb_atoms;
    int pb_rigid;                  // rigid_box_centre: the centre stays at pb_centre
    int pb_nslu;                   // atoms averaged for a floating centre (nat_solute, or natom)
    double pb_centre[3];
    double* pb_boxc;               // [nwin][3] the centre of the last call (boxcentre)
    int tg_first[kMaxTg], tg_last[kMaxTg];
    double tg_ndegf[kMaxTg], tg_ndegfree[kMaxTg], ndegf, ndegfree;
    double dt, tau, temp0, boltz;
    const double* winv;            // [natom] 1/mass
    const double* mass;            // [natom]
    const int* mol_first;          // [nmol+1]
    const int2* con;               // [ncons] atom pairs
    const double* dist2;           // [ncons] squared constraint distances
    uint8_t* ready;                // [nwin][ncons] SHAKE scratch
    int ncons;
    double* v;                     // [nwin][natom*3]
    double* xx;                    // [nwin][natom*3] positions before newvel
    MdWin* win;                    // [nwin]
    int* fail;                     // [nwin] 1 + a molecule whose SHAKE failed, 0 if none (sticky)
};
// a record of one window and step: FP64 energy slots, fixed-point slots, then
// ekin, temp, tfree, SHAKE iterations
constexpr int kMdRec = 2 * kNumE + 4;
void launch_md_newvel(const Launch& L, const MdDev& md);
// nh_prop (chain update, one thread per window) and v *= s of every atom
void launch_md_nh(const Launch& L, const MdDev& md);
// put_back_in_box, src/simprep.f90:4177-4352 (needs DevModel box lengths)
void launch_md_put_back(const Launch& L, const MdDev& md);
// mode 0: constrain x against xx (the step); 1: constrain xx against x
void launch_md_shake(const Launch& L, const MdDev& md, int mode);
void launch_md_velocity(const Launch& L, const MdDev& md);
void launch_md_copy_x(const Launch& L, const MdDev& md, int to_xx);   // xx = x (1) or the x - v dt of initial_constraint (2)
void launch_md_temperature(const Launch& L, const MdDev& md, const uint8_t* excl);
void launch_md_stop_cm(const Launch& L, const MdDev& md);
void launch_md_min_step(const Launch& L, const MdDev& md, double step0, double fcut, double max_move);
void launch_md_record(const Launch& L, const MdDev& md, const double* e_all, const unsigned long long* efix_all,
                      double* rec);
void launch_md_clear_d(const Launch& L, const MdDev& md);   // d = 0, SHAKE count = 0

// records msg as the calling thread's qnb_last_error text; returns code
int set_error(int code, const char* msg);

}  // namespace qnb
