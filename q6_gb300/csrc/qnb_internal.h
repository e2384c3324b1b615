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
constexpr double kFix = 4294967296.0;   // 2^32: fixed-point quantum of forces/energies
constexpr float kFixF = 4294967296.0f;

// energy slots (doubles in FP64 mode, 2^-32 fixed point in mixed mode)
enum {
    E_PP_EL = 0, E_PP_VDW, E_PW_EL, E_PW_VDW, E_WW_EL, E_WW_VDW, E_LRF,
    E_RST_RAD, E_RST_POL, E_Q0
};
__host__ __device__ constexpr int eq_slot(int s, int k) { return E_Q0 + 6 * s + k; }
constexpr int kNumE = E_Q0 + 6 * kMaxStates;

// list counters / status words
enum { C_WW = 0, C_PW, C_PP, C_QP, C_QW, C_PP14, C_NUM };

struct alignas(32) QPar {   // one (pair type, state) parameter set: A, B, elec, soft-core alpha
    double A, B, el, sc;
};
struct alignas(16) QParF {
    float A, B, el, sc;
};

// Static model on the device.  Passed by value to kernels.
struct DevModel {
    int natom, nat_solute, nwat, sa, ncgp, ncgp_solute, natyps, nqat, S;
    int spc;           // SPC fast path for ww / qw (geometric rule + SPC solvent)
    int use_lrf;
    double el14;
    const int* iac;
    const double* crg;
    const int* iqatom;          // -1 or Q index
    const uint8_t* excl;
    const int* gslot;           // [ncgp+1] offsets into gatom
    const int* gatom;           // group member atoms
    const int* gsw;             // [ncgp] switch atoms
    const int* spec_off;        // [nat_solute+1] special partners of i (j > i)
    const int* spec_j;
    const uint8_t* spec_kind;   // 1 excluded, 3 1-4
    const double2* lj;          // [3][natyps][natyps] (A,B) per LJ code 1..3
    const float2* ljf;
    const uint8_t* ljcod;       // [natyps][natyps]
    const uint8_t* ljset;       // [3][natyps][natyps]: |A| or |B| > QREAL_EPS
    int wtype[kMaxSolv];        // solvent template (first molecule) atom types
    double wcrg[kMaxSolv];      // and charges
    float wcrgf[kMaxSolv];
    double wwA[kMaxSolv * kMaxSolv], wwB[kMaxSolv * kMaxSolv], wwE[kMaxSolv * kMaxSolv];  // ww_precomp
    float wwAf[kMaxSolv * kMaxSolv], wwBf[kMaxSolv * kMaxSolv], wwEf[kMaxSolv * kMaxSolv];
    const int* iqseq;           // [nqat]
    const QPar* qp_tab;         // [nat_solute][nqat][S]
    const QParF* qp_tabf;
    const QPar* qw_tab;         // [nqat][sa][S]
    const QParF* qw_tabf;
    double xpcent[3], xwcent[3];
    double rexcl_o2;
};

struct QQEntry {   // static Q-Q / Q-bonded-P pair of one state
    int i, j, s, soft;      // atom indices (not Q indices), state, exp-repulsion flag
    double A, B, el, sc;
};

// Per-context device state of the lists, coordinates and accumulators.
struct DevState {
    double* x;           // [natom*3] coordinates (FP64, as qdyn holds them)
    double* d;           // [natom*3] gradient accumulator (FP64 mode target)
    float4* xq;          // [natom] FP32 (x,y,z,charge) for the mixed form
    unsigned long long* fix;   // [natom*3] fixed-point gradient (mixed form)
    double* e;           // [kNumE] FP64 energies
    unsigned long long* efix;  // [kNumE] fixed-point energies (mixed form)
    double* lambda;      // [S]
    double* lrf;         // [ncgp*43]
    int* cnt;            // [C_NUM] list sizes (device-maintained)
    int2* ww; int64_t cap_ww;      // water pairs (iw, jw), iw < jw
    int2* pw; int64_t cap_pw;      // (solute atom, water)
    int2* pp; int64_t cap_pp;      // (i, j | code << 28)
    int* qp;  int64_t cap_qp;      // solute atoms interacting with all Q atoms
    int* qw;  int64_t cap_qw;      // waters interacting with all Q atoms
    QQEntry* qq; int nqq;          // static qq + qqp entries (all states)
    int nqq_qq;                    // first nqq_qq entries are Q-Q (EQ%qq), rest Q-P (EQ%qp)
    // water polarisation
    double* theta;       // [nwat]
    int* shell;          // [nwat] shell or -1
    int* rank;           // [nwat]
    int* n_insh;         // [kMaxShell]
    double* wstate;      // [3*kMaxShell]: theta_corr, avtheta, avn_insh
};

// ---- launch wrappers (qnb_kernels.cu) ---------------------------------------
struct Cut {
    double rcq2, rlrf2, rcpp2, rcpw2, rcww2;
};

void launch_group_centres(const DevModel& m, DevState& s, cudaStream_t st);
void launch_build_ww(const DevModel& m, DevState& s, const Cut& c, cudaStream_t st);
void launch_build_pw(const DevModel& m, DevState& s, const Cut& c, cudaStream_t st);
void launch_build_pp(const DevModel& m, DevState& s, const Cut& c, cudaStream_t st);
void launch_build_qp_impl(const DevModel& m, DevState& s, const uint8_t* qnear, double rcq2, cudaStream_t st);
void launch_build_qw(const DevModel& m, DevState& s, const Cut& c, cudaStream_t st);
void launch_lrf_accumulate(const DevModel& m, DevState& s, const Cut& c, int mixed, cudaStream_t st);

void launch_pack_mixed(const DevModel& m, DevState& s, cudaStream_t st);
void launch_nonbond(const DevModel& m, DevState& s, int mixed, int md, cudaStream_t st, int* nlaunch);
void launch_nonbond_qq(const DevModel& m, DevState& s, int mixed, cudaStream_t st);
void launch_lrf_taylor_impl(const DevModel& m, DevState& s, const int* iwhich, int mixed, cudaStream_t st);
void launch_apply_fixed(const DevModel& m, DevState& s, cudaStream_t st);

struct SolventDev {
    double fk_wsphere, Dwmz, awmz, rwat, boltz, fkwpol, itdis;
    int wpol, nshell;
    double rout[kMaxShell], dr[kMaxShell], cstb[kMaxShell];
};
void launch_restrain_solvent_impl(const DevModel& m, DevState& s, const SolventDev& p, double Tfree, int mixed,
                                  const int* wsw, const uint8_t* heavy_solv, cudaStream_t st);
void launch_watpol_impl(const DevModel& m, DevState& s, const SolventDev& p, int istep, int md, int mixed,
                        double* shell_tsum, cudaStream_t st, int* nlaunch);

void launch_export_pairs(const DevModel& m, const DevState& s, int kind, int32_t* di, int32_t* dj,
                         int64_t cap, int* dcount, cudaStream_t st);

}  // namespace qnb
