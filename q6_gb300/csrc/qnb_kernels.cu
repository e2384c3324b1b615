// CUDA kernels (sm_103a) of the qdyn nonbonded engine.
//
// Two precision forms share every kernel through a template flag:
//  * FP64 (plain): the reference's arithmetic in double, gradients and
//    energies accumulated with double atomics.
//  * mixed: pair arithmetic in FP32 (rsqrt on the SFU); every per-pair
//    gradient and energy contribution is converted to 64-bit fixed point
//    (quantum 2^-32) and summed with integer atomics, which makes the result
//    independent of list order and thread schedule.  Cut-off tests, group
//    centres, the LRF Taylor terms and the boundary restraints stay FP64.
//
// Pair-list semantics follow Q6 src/nonbondene.f90 (cited per kernel).  A list
// is kept at the granularity the reference tests the cut-off at (charge-group
// pairs, solute atom x water, water pairs) and expanded to atom pairs inside
// the force kernels.
#include <cuda_runtime.h>
#include <math.h>

#include <type_traits>

#include "qnb_internal.h"

namespace qnb {

namespace {

constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int warp_id_global() {
    return (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
}
__device__ __forceinline__ int warps_total() { return (gridDim.x * blockDim.x) >> 5; }

// q_dist4 (src/math.f90:255-262): (b-a).(b-a) summed x,y,z left to right,
// every operation rounded separately (no FMA), so the bits match the oracle.
__device__ __forceinline__ double dist2_exact(double ax, double ay, double az, double bx, double by,
                                              double bz) {
    double dx = __dsub_rn(bx, ax), dy = __dsub_rn(by, ay), dz = __dsub_rn(bz, az);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// warp-aggregated append: returns this lane's first slot (valid when n > 0)
__device__ __forceinline__ int warp_append(int* counter, int n) {
    int lane = threadIdx.x & 31;
    int incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += v;
    }
    int total = __shfl_sync(kFull, incl, 31);
    int base = 0;
    if (lane == 31 && total > 0) base = atomicAdd(counter, total);
    base = __shfl_sync(kFull, base, 31);
    return base + incl - n;
}

// ---- accumulation back-ends -------------------------------------------------
__device__ __forceinline__ unsigned long long to_fix(float v) {
    return (unsigned long long)__float2ll_rn(v * kFixF);
}
__device__ __forceinline__ unsigned long long to_fixd(double v) {
    return (unsigned long long)__double2ll_rn(v * kFix);
}

template <bool MIX>
struct Acc;

template <>
struct Acc<false> {
    double* d;
    double* e;
    __device__ __forceinline__ void grad(int i, double gx, double gy, double gz) const {
        atomicAdd(d + 3 * i, gx);
        atomicAdd(d + 3 * i + 1, gy);
        atomicAdd(d + 3 * i + 2, gz);
    }
    __device__ __forceinline__ void energy(int slot, double v) const { atomicAdd(e + slot, v); }
};

template <>
struct Acc<true> {
    unsigned long long* f;
    unsigned long long* e;
    __device__ __forceinline__ void grad(int i, float gx, float gy, float gz) const {
        atomicAdd(f + 3 * i, to_fix(gx));
        atomicAdd(f + 3 * i + 1, to_fix(gy));
        atomicAdd(f + 3 * i + 2, to_fix(gz));
    }
    __device__ __forceinline__ void gradd(int i, double gx, double gy, double gz) const {
        atomicAdd(f + 3 * i, to_fixd(gx));
        atomicAdd(f + 3 * i + 1, to_fixd(gy));
        atomicAdd(f + 3 * i + 2, to_fixd(gz));
    }
    __device__ __forceinline__ void energy_fix(int slot, unsigned long long v) const {
        atomicAdd(e + slot, v);
    }
};

template <bool MIX>
__device__ __forceinline__ Acc<MIX> make_acc(const DevState& s);
template <>
__device__ __forceinline__ Acc<false> make_acc<false>(const DevState& s) {
    return Acc<false>{s.d, s.e};
}
template <>
__device__ __forceinline__ Acc<true> make_acc<true>(const DevState& s) {
    return Acc<true>{s.fix, s.efix};
}

// warp sums (lane 0 holds the result)
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}
__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
    return v;
}

// Energy accumulator of one thread: FP64 sums in the plain form, exact 64-bit
// fixed-point sums of the per-pair FP32 values in the mixed form.
template <bool MIX>
struct ESum;
template <>
struct ESum<false> {
    double v = 0.0;
    __device__ __forceinline__ void add(double x) { v += x; }
    __device__ __forceinline__ void flush(const Acc<false>& a, int slot) {
        double t = warp_sum(v);
        if ((threadIdx.x & 31) == 0 && t != 0.0) a.energy(slot, t);
    }
};
template <>
struct ESum<true> {
    unsigned long long v = 0ull;
    __device__ __forceinline__ void add(float x) { v += to_fix(x); }
    __device__ __forceinline__ void add(double x) { v += to_fixd(x); }
    __device__ __forceinline__ void flush(const Acc<true>& a, int slot) {
        unsigned long long t = warp_sum(v);
        if ((threadIdx.x & 31) == 0 && t != 0ull) a.energy_fix(slot, t);
    }
};

}  // namespace

// =============================================================================
// List build
// =============================================================================

// cgp_centers, src/nonbondene.f90:43-78: zero the LRF record and set the centre
__global__ void k_group_centres(DevModel m, const double* __restrict__ x, double* __restrict__ lrf) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= m.ncgp) return;
    double cx = 0.0, cy = 0.0, cz = 0.0;
    int a0 = m.gslot[g], a1 = m.gslot[g + 1];
    for (int a = a0; a < a1; ++a) {
        int i = m.gatom[a];
        cx = __dadd_rn(cx, x[3 * i]);
        cy = __dadd_rn(cy, x[3 * i + 1]);
        cz = __dadd_rn(cz, x[3 * i + 2]);
    }
    double n = (double)(a1 - a0);
    double* L = lrf + (size_t)g * kLrfLen;
    L[0] = __ddiv_rn(cx, n);
    L[1] = __ddiv_rn(cy, n);
    L[2] = __ddiv_rn(cz, n);
    for (int k = 3; k < kLrfLen; ++k) L[k] = 0.0;
}

// nbwwlist(_lrf) pair selection, src/nonbondene.f90:4274-4395: water pairs
// with O-O r2 <= Rcww2, neither O excluded.  Each unordered pair is kept once
// (iw < jw), the same set as the reference's parity rule.
__global__ void k_build_ww(DevModel m, const double* __restrict__ x, int2* __restrict__ out,
                           int64_t cap, int* __restrict__ cnt, double rc2) {
    int lane = threadIdx.x & 31;
    for (int iw = warp_id_global(); iw < m.nwat; iw += warps_total()) {
        int io = m.nat_solute + m.sa * iw;
        if (m.excl[io]) continue;
        double xi = x[3 * io], yi = x[3 * io + 1], zi = x[3 * io + 2];
        for (int j0 = iw + 1; j0 < m.nwat; j0 += kWarp) {
            int jw = j0 + lane;
            bool ok = false;
            if (jw < m.nwat) {
                int jo = m.nat_solute + m.sa * jw;
                if (!m.excl[jo]) {
                    double r2 = dist2_exact(xi, yi, zi, x[3 * jo], x[3 * jo + 1], x[3 * jo + 2]);
                    ok = (r2 <= rc2);
                }
            }
            int pos = warp_append(cnt, ok ? 1 : 0);
            if (ok && pos < cap) out[pos] = make_int2(iw, jw);
        }
    }
}

// nbpwlist(_lrf), src/nonbondene.f90:2842-2955: solute group switch atom to
// water O within Rcpw; every non-Q atom of the group pairs with the molecule.
__global__ void k_build_pw(DevModel m, const double* __restrict__ x, int2* __restrict__ out,
                           int64_t cap, int* __restrict__ cnt, double rc2) {
    int lane = threadIdx.x & 31;
    for (int ig = warp_id_global(); ig < m.ncgp_solute; ig += warps_total()) {
        int is = m.gsw[ig];
        if (m.excl[is]) continue;
        int a0 = m.gslot[ig], a1 = m.gslot[ig + 1];
        int nq = 0;
        for (int a = a0; a < a1; ++a) nq += (m.iqatom[m.gatom[a]] < 0);
        if (nq == 0) continue;
        double xi = x[3 * is], yi = x[3 * is + 1], zi = x[3 * is + 2];
        for (int j0 = 0; j0 < m.nwat; j0 += kWarp) {
            int jw = j0 + lane;
            bool ok = false;
            if (jw < m.nwat) {
                int jo = m.nat_solute + m.sa * jw;
                if (!m.excl[jo]) {
                    double r2 = dist2_exact(xi, yi, zi, x[3 * jo], x[3 * jo + 1], x[3 * jo + 2]);
                    ok = (r2 <= rc2);
                }
            }
            int pos = warp_append(cnt, ok ? nq : 0);
            if (ok) {
                for (int a = a0; a < a1; ++a) {
                    int i = m.gatom[a];
                    if (m.iqatom[i] >= 0) continue;
                    if (pos < cap) out[pos] = make_int2(i, jw);
                    ++pos;
                }
            }
        }
    }
}

// classification of one solute atom pair as pp_int_comp does it
// (src/simprep.f90:2992-3053): 0 = excluded, 3 = 1-4, else ljcod
__device__ __forceinline__ int pp_code(const DevModel& m, int i, int j) {
    int lo = i < j ? i : j, hi = i < j ? j : i;
    for (int k = m.spec_off[lo]; k < m.spec_off[lo + 1]; ++k)
        if (m.spec_j[k] == hi) return m.spec_kind[k] == 1 ? 0 : 3;
    return m.ljcod[m.iac[i] * m.natyps + m.iac[j]];
}

// is the pair in the reference's list (pp_map != 0 and precomp%set)?
// precompute_set_values_pp, src/simprep.f90:3321-3350
__device__ __forceinline__ int pp_accept(const DevModel& m, int i, int j) {
    if (m.iqatom[i] >= 0 || m.iqatom[j] >= 0) return 0;
    int code = pp_code(m, i, j);
    if (code == 0) return 0;
    int ti = m.iac[i], tj = m.iac[j];
    bool set = m.ljset[((code - 1) * m.natyps + ti) * m.natyps + tj] ||
               fabs(__dmul_rn(m.crg[i], m.crg[j])) > 1.0e-10;
    return set ? code : 0;
}

// nbpplist(_lrf), src/nonbondene.f90:1777-1908: solute group pairs whose
// switch atoms are within Rcpp, expanded to the accepted atom pairs.
__global__ void k_build_pp(DevModel m, const double* __restrict__ x, int2* __restrict__ out,
                           int64_t cap, int* __restrict__ cnt, int* __restrict__ cnt14, double rc2) {
    int lane = threadIdx.x & 31;
    for (int ig = warp_id_global(); ig < m.ncgp_solute; ig += warps_total()) {
        int is = m.gsw[ig];
        if (m.excl[is]) continue;
        int a0 = m.gslot[ig], a1 = m.gslot[ig + 1];
        double xi = x[3 * is], yi = x[3 * is + 1], zi = x[3 * is + 2];
        for (int j0 = ig; j0 < m.ncgp_solute; j0 += kWarp) {
            int jg = j0 + lane;
            bool ok = false;
            if (jg < m.ncgp_solute) {
                int js = m.gsw[jg];
                if (!m.excl[js]) {
                    double r2 = (jg == ig) ? 0.0
                                           : dist2_exact(xi, yi, zi, x[3 * js], x[3 * js + 1], x[3 * js + 2]);
                    ok = (r2 <= rc2);
                }
            }
            int n = 0, n14 = 0;
            int b0 = 0, b1 = 0;
            if (ok) {
                b0 = m.gslot[jg];
                b1 = m.gslot[jg + 1];
                for (int a = a0; a < a1; ++a)
                    for (int b = b0; b < b1; ++b) {
                        int i = m.gatom[a], j = m.gatom[b];
                        if (jg == ig && i >= j) continue;
                        int c = pp_accept(m, i, j);
                        n += (c != 0);
                        n14 += (c == 3);
                    }
            }
            int pos = warp_append(cnt, n);
            if (__any_sync(kFull, n14 > 0)) warp_append(cnt14, n14);
            if (n > 0) {
                for (int a = a0; a < a1; ++a)
                    for (int b = b0; b < b1; ++b) {
                        int i = m.gatom[a], j = m.gatom[b];
                        if (jg == ig && i >= j) continue;
                        int c = pp_accept(m, i, j);
                        if (c == 0) continue;
                        if (pos < cap) out[pos] = make_int2(i, j | (c << 28));
                        ++pos;
                    }
            }
        }
    }
}

// nbqplist, src/nonbondene.f90:3647-3742: solute groups whose switch atom is
// within Rcq of the solute centre; atoms not bonded/angled to any Q atom.
__global__ void k_build_qp(DevModel m, const double* __restrict__ x, const uint8_t* __restrict__ qnear,
                           int* __restrict__ out, int64_t cap, int* __restrict__ cnt, double rcq2) {
    int ig = blockIdx.x * blockDim.x + threadIdx.x;
    if (ig >= m.ncgp_solute) return;
    int is = m.gsw[ig];
    if (m.excl[is]) return;
    double r2 = dist2_exact(x[3 * is], x[3 * is + 1], x[3 * is + 2], m.xpcent[0], m.xpcent[1], m.xpcent[2]);
    if (r2 > rcq2) return;
    for (int a = m.gslot[ig]; a < m.gslot[ig + 1]; ++a) {
        int i = m.gatom[a];
        if (qnear[i]) continue;
        int pos = atomicAdd(cnt, 1);
        if (pos < cap) out[pos] = i;
    }
}

// nbqwlist, src/nonbondene.f90:3862-3944: waters with O within Rcq of xpcent
__global__ void k_build_qw(DevModel m, const double* __restrict__ x, int* __restrict__ out, int64_t cap,
                           int* __restrict__ cnt, double rcq2) {
    int iw = blockIdx.x * blockDim.x + threadIdx.x;
    if (iw >= m.nwat) return;
    int io = m.nat_solute + m.sa * iw;
    if (m.excl[io]) return;
    double r2 = dist2_exact(x[3 * io], x[3 * io + 1], x[3 * io + 2], m.xpcent[0], m.xpcent[1], m.xpcent[2]);
    if (r2 <= rcq2) {
        int pos = atomicAdd(cnt, 1);
        if (pos < cap) out[pos] = iw;
    }
}

// -----------------------------------------------------------------------------
// LRF: lrf_update(g1, g2) of src/nonbondene.f90:628-725 for every group pair
// the list builders classify as "outside the cut-off but inside RcLRF".
// Gather form: one warp per target group g2 sums the contributions of all its
// far groups g1, so no atomics are needed.
// -----------------------------------------------------------------------------
__device__ __forceinline__ int group_dist_atom(const DevModel& m, int g) {
    // solute groups: switch atom; water groups: the molecule's first atom
    return g < m.ncgp_solute ? m.gsw[g] : m.nat_solute + m.sa * (g - m.ncgp_solute);
}

template <typename T>
__device__ __forceinline__ void lrf_terms(T dx, T dy, T dz, T q, T* acc) {
    T r2 = dx * dx + dy * dy + dz * dz;
    T f0 = q / (r2 * sqrt(r2));
    T f1 = T(3) * f0 / r2;
    T f2 = -f1 / r2;
    T d[3] = {dx, dy, dz};
    acc[0] += f0 * r2;
    acc[1] -= dx * f0;
    acc[2] -= dy * f0;
    acc[3] -= dz * f0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        T t = d[a] * f1;
#pragma unroll
        for (int c = 0; c < 3; ++c) acc[4 + 3 * a + c] += d[c] * t;
    }
    acc[4 + 0] -= f0;
    acc[4 + 4] -= f0;
    acc[4 + 8] -= f0;
    T f25 = T(5) * f2;
#pragma unroll
    for (int n = 0; n < 3; ++n)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            T tk = d[n] * d[j] * f25;
#pragma unroll
            for (int c = 0; c < 3; ++c) acc[13 + 3 * (j + 3 * n) + c] += tk * d[c];
        }
    T u0 = dx * r2 * f2, u1 = dy * r2 * f2, u2 = dz * r2 * f2;
    T* P = acc + 13;   // P[3*m + c] = phi3(m+1) component c
    P[0] -= T(3) * u0; P[1] -= u1; P[2] -= u2;
    P[3] -= u1; P[4] -= u0;
    P[6] -= u2;
    P[8] -= u0;
    P[9] -= u1; P[10] -= u0;
    P[12] -= u0; P[13] -= T(3) * u1; P[14] -= u2;
    P[16] -= u2; P[17] -= u1;
    P[18] -= u2;
    P[20] -= u0;
    P[22] -= u2; P[23] -= u1;
    P[24] -= u0; P[25] -= u1; P[26] -= T(3) * u2;
}

template <bool MIX>
__global__ void __launch_bounds__(128) k_lrf_accumulate(DevModel m, const double* __restrict__ x,
                                                         double* __restrict__ lrf, Cut c) {
    typedef typename std::conditional<MIX, float, double>::type T;
    int lane = threadIdx.x & 31;
    for (int g2 = warp_id_global(); g2 < m.ncgp; g2 += warps_total()) {
        int s2 = group_dist_atom(m, g2);
        if (m.excl[s2]) continue;
        bool sol2 = g2 < m.ncgp_solute;
        double* L = lrf + (size_t)g2 * kLrfLen;
        double cx = L[0], cy = L[1], cz = L[2];
        double xs = x[3 * s2], ys = x[3 * s2 + 1], zs = x[3 * s2 + 2];
        T acc[40];
#pragma unroll
        for (int k = 0; k < 40; ++k) acc[k] = T(0);
        for (int g1 = lane; g1 < m.ncgp; g1 += kWarp) {
            if (g1 == g2) continue;
            int s1 = group_dist_atom(m, g1);
            if (m.excl[s1]) continue;
            bool sol1 = g1 < m.ncgp_solute;
            double rc2 = (sol1 && sol2) ? c.rcpp2 : ((sol1 || sol2) ? c.rcpw2 : c.rcww2);
            double r2 = dist2_exact(xs, ys, zs, x[3 * s1], x[3 * s1 + 1], x[3 * s1 + 2]);
            if (r2 <= rc2 || r2 > c.rlrf2) continue;
            for (int a = m.gslot[g1]; a < m.gslot[g1 + 1]; ++a) {
                int i = m.gatom[a];
                if (m.iqatom[i] >= 0) continue;
                T dx = T(x[3 * i] - cx), dy = T(x[3 * i + 1] - cy), dz = T(x[3 * i + 2] - cz);
                lrf_terms<T>(dx, dy, dz, T(m.crg[i]), acc);
            }
        }
#pragma unroll
        for (int k = 0; k < 40; ++k) {
            double v = warp_sum((double)acc[k]);
            if (lane == 0) L[3 + k] = v;
        }
    }
}

// =============================================================================
// Force / energy kernels
// =============================================================================

__global__ void k_pack_mixed(DevModel m, const double* __restrict__ x, float4* __restrict__ xq) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.natom) return;
    xq[i] = make_float4((float)x[3 * i], (float)x[3 * i + 1], (float)x[3 * i + 2], (float)m.crg[i]);
}

// one plain pair (nbe, src/nonbonded.f90:45-75); returns dv, vec via refs
struct PairD {
    double tx, ty, tz, dv, vel, vdw;
};
__device__ __forceinline__ PairD nbe_d(const double* x, int i, int j, double A, double B, double el,
                                       bool lj) {
    PairD p;
    p.tx = x[3 * j] - x[3 * i];
    p.ty = x[3 * j + 1] - x[3 * i + 1];
    p.tz = x[3 * j + 2] - x[3 * i + 2];
    double r2 = 1.0 / (p.tx * p.tx + p.ty * p.ty + p.tz * p.tz);
    double r = sqrt(r2);
    p.vel = el * r;
    if (lj) {
        double r6 = r2 * r2 * r2;
        double r12 = r6 * r6;
        double va = A * r12, vb = B * r6;
        p.dv = r2 * (-p.vel - 12.0 * va + 6.0 * vb);
        p.vdw = va - vb;
    } else {   // nbe_spc, src/nonbonded.f90:247-267
        p.dv = r2 * (-p.vel);
        p.vdw = 0.0;
    }
    return p;
}
struct PairF {
    float tx, ty, tz, dv, vel, vdw;
};
__device__ __forceinline__ PairF nbe_f(float4 a, float4 b, float A, float B, float el, bool lj) {
    PairF p;
    p.tx = b.x - a.x;
    p.ty = b.y - a.y;
    p.tz = b.z - a.z;
    float rr = p.tx * p.tx + p.ty * p.ty + p.tz * p.tz;
    float ri = rsqrtf(rr);
    float r2 = ri * ri;
    p.vel = el * ri;
    if (lj) {
        float r6 = r2 * r2 * r2;
        float va = A * r6 * r6, vb = B * r6;
        p.dv = r2 * (-p.vel - 12.0f * va + 6.0f * vb);
        p.vdw = va - vb;
    } else {
        p.dv = -r2 * p.vel;
        p.vdw = 0.0f;
    }
    return p;
}

// nonbond_ww_spc / nonbond_ww, src/nonbondene.f90:5886-5975, 5509-5573
template <bool MIX, bool SPC>
__global__ void __launch_bounds__(256) k_ww(DevModel m, DevState s) {
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel, evdw;
    int n = min((int64_t)s.cnt[C_WW], s.cap_ww);
    int sa = m.sa;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int2 e = s.ww[p];
        int i0 = m.nat_solute + sa * e.x, j0 = m.nat_solute + sa * e.y;
        if constexpr (!MIX) {
            double gi[kMaxSolv][3] = {}, gj[kMaxSolv][3] = {};
            for (int la = 0; la < sa; ++la)
                for (int ka = 0; ka < sa; ++ka) {
                    bool lj = !SPC || (la == 0 && ka == 0);
                    int k = la * kMaxSolv + ka;
                    PairD q = nbe_d(s.x, i0 + la, j0 + ka, m.wwA[k], m.wwB[k], m.wwE[k], lj);
                    gi[la][0] -= q.tx * q.dv; gi[la][1] -= q.ty * q.dv; gi[la][2] -= q.tz * q.dv;
                    gj[ka][0] += q.tx * q.dv; gj[ka][1] += q.ty * q.dv; gj[ka][2] += q.tz * q.dv;
                    eel.add(q.vel);
                    evdw.add(q.vdw);
                }
            for (int a = 0; a < sa; ++a) {
                acc.grad(i0 + a, gi[a][0], gi[a][1], gi[a][2]);
                acc.grad(j0 + a, gj[a][0], gj[a][1], gj[a][2]);
            }
        } else {
            float gi[kMaxSolv][3] = {}, gj[kMaxSolv][3] = {};
            float4 xi[kMaxSolv], xj[kMaxSolv];
            for (int a = 0; a < sa; ++a) { xi[a] = s.xq[i0 + a]; xj[a] = s.xq[j0 + a]; }
            for (int la = 0; la < sa; ++la)
                for (int ka = 0; ka < sa; ++ka) {
                    bool lj = !SPC || (la == 0 && ka == 0);
                    int k = la * kMaxSolv + ka;
                    PairF q = nbe_f(xi[la], xj[ka], m.wwAf[k], m.wwBf[k], m.wwEf[k], lj);
                    gi[la][0] -= q.tx * q.dv; gi[la][1] -= q.ty * q.dv; gi[la][2] -= q.tz * q.dv;
                    gj[ka][0] += q.tx * q.dv; gj[ka][1] += q.ty * q.dv; gj[ka][2] += q.tz * q.dv;
                    eel.add(q.vel);
                    evdw.add(q.vdw);
                }
            for (int a = 0; a < sa; ++a) {
                acc.grad(i0 + a, gi[a][0], gi[a][1], gi[a][2]);
                acc.grad(j0 + a, gj[a][0], gj[a][1], gj[a][2]);
            }
        }
    }
    eel.flush(acc, E_WW_EL);
    evdw.flush(acc, E_WW_VDW);
}

// nonbond_pw, src/nonbondene.f90:4856-4916 (pw_precomp, src/simprep.f90:3354-3386)
template <bool MIX>
__global__ void __launch_bounds__(256) k_pw(DevModel m, DevState s) {
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel, evdw;
    int n = min((int64_t)s.cnt[C_PW], s.cap_pw);
    int sa = m.sa;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int2 e = s.pw[p];
        int i = e.x, j0 = m.nat_solute + sa * e.y;
        int ti = m.iac[i];
        if constexpr (!MIX) {
            double g[3] = {0, 0, 0};
            for (int a = 0; a < sa; ++a) {
                int tw = m.wtype[a];
                int code = m.ljcod[ti * m.natyps + tw];
                double2 ab = m.lj[((code - 1) * m.natyps + ti) * m.natyps + tw];
                PairD q = nbe_d(s.x, i, j0 + a, ab.x, ab.y, m.crg[i] * m.wcrg[a], true);
                g[0] -= q.tx * q.dv; g[1] -= q.ty * q.dv; g[2] -= q.tz * q.dv;
                acc.grad(j0 + a, q.tx * q.dv, q.ty * q.dv, q.tz * q.dv);
                eel.add(q.vel);
                evdw.add(q.vdw);
            }
            acc.grad(i, g[0], g[1], g[2]);
        } else {
            float g[3] = {0, 0, 0};
            float4 xi = s.xq[i];
            for (int a = 0; a < sa; ++a) {
                int tw = m.wtype[a];
                int code = m.ljcod[ti * m.natyps + tw];
                float2 ab = m.ljf[((code - 1) * m.natyps + ti) * m.natyps + tw];
                PairF q = nbe_f(xi, s.xq[j0 + a], ab.x, ab.y, xi.w * m.wcrgf[a], true);
                g[0] -= q.tx * q.dv; g[1] -= q.ty * q.dv; g[2] -= q.tz * q.dv;
                acc.grad(j0 + a, q.tx * q.dv, q.ty * q.dv, q.tz * q.dv);
                eel.add(q.vel);
                evdw.add(q.vdw);
            }
            acc.grad(i, g[0], g[1], g[2]);
        }
    }
    eel.flush(acc, E_PW_EL);
    evdw.flush(acc, E_PW_VDW);
}

// nonbond_pp, src/nonbondene.f90:4694-4760 (pp_precomp values)
template <bool MIX>
__global__ void __launch_bounds__(256) k_pp(DevModel m, DevState s) {
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel, evdw;
    int n = min((int64_t)s.cnt[C_PP], s.cap_pp);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int2 e = s.pp[p];
        int i = e.x, j = e.y & 0x0fffffff, code = e.y >> 28;
        int ti = m.iac[i], tj = m.iac[j];
        size_t t = ((size_t)(code - 1) * m.natyps + ti) * m.natyps + tj;
        if constexpr (!MIX) {
            double2 ab = m.lj[t];
            double el = m.crg[i] * m.crg[j];
            if (code == 3) el = el * m.el14;
            PairD q = nbe_d(s.x, i, j, ab.x, ab.y, el, true);
            acc.grad(i, -q.tx * q.dv, -q.ty * q.dv, -q.tz * q.dv);
            acc.grad(j, q.tx * q.dv, q.ty * q.dv, q.tz * q.dv);
            eel.add(q.vel);
            evdw.add(q.vdw);
        } else {
            float2 ab = m.ljf[t];
            float4 xi = s.xq[i], xj = s.xq[j];
            float el = xi.w * xj.w;
            if (code == 3) el *= (float)m.el14;
            PairF q = nbe_f(xi, xj, ab.x, ab.y, el, true);
            acc.grad(i, -q.tx * q.dv, -q.ty * q.dv, -q.tz * q.dv);
            acc.grad(j, q.tx * q.dv, q.ty * q.dv, q.tz * q.dv);
            eel.add(q.vel);
            evdw.add(q.vdw);
        }
    }
    eel.flush(acc, E_PP_EL);
    evdw.flush(acc, E_PP_VDW);
}

// Q-atom x environment.  One thread per environment atom (qp) or molecule
// (qw) loops over the Q atoms; the Q-atom gradients are summed per block in
// shared memory and added once per block.
template <bool MIX>
struct QShared;
template <>
struct QShared<false> {
    double* g;
    __device__ __forceinline__ void add(int iq, double gx, double gy, double gz) {
        atomicAdd(g + 3 * iq, gx);
        atomicAdd(g + 3 * iq + 1, gy);
        atomicAdd(g + 3 * iq + 2, gz);
    }
};
template <>
struct QShared<true> {
    unsigned long long* g;
    __device__ __forceinline__ void add(int iq, float gx, float gy, float gz) {
        atomicAdd(g + 3 * iq, to_fix(gx));
        atomicAdd(g + 3 * iq + 1, to_fix(gy));
        atomicAdd(g + 3 * iq + 2, to_fix(gz));
    }
};

// nbe_qx soft-core pair for one state, src/nonbonded.f90:200-222
__device__ __forceinline__ void nbe_qx_d(double r2, double r, double r6inv_hc_, double A, double B,
                                         double el, double sc, double lam, double& vel, double& vdw,
                                         double& dv) {
    double r6_hc = r6inv_hc_;          // = 1 / dist%r6 = |r|^6
    double r6 = 1.0 / (r6_hc + sc);
    double r12 = r6 * r6;
    vel = el * r;
    double va = A * r12, vb = B * r6;
    vdw = va - vb;
    dv = r2 * (-vel - (12.0 * va - 6.0 * vb) * r6 * r6_hc) * lam;
}
__device__ __forceinline__ void nbe_qx_f(float r2, float r, float r6_hc, float A, float B, float el,
                                         float sc, float lam, float& vel, float& vdw, float& dv) {
    float r6 = 1.0f / (r6_hc + sc);
    float r12 = r6 * r6;
    vel = el * r;
    float va = A * r12, vb = B * r6;
    vdw = va - vb;
    dv = r2 * (-vel - (12.0f * va - 6.0f * vb) * r6 * r6_hc) * lam;
}

constexpr int kMaxQ = 64;

// nonbond_qw_spc / nonbond_qw, src/nonbondene.f90:5658-5767, 5339-5418
template <bool MIX, bool SPC>
__global__ void __launch_bounds__(256) k_qw(DevModel m, DevState s) {
    typedef typename std::conditional<MIX, unsigned long long, double>::type GT;
    __shared__ GT gq[3 * kMaxQ];
    for (int k = threadIdx.x; k < 3 * m.nqat; k += blockDim.x) gq[k] = GT(0);
    __syncthreads();
    QShared<MIX> qs{gq};
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel[kMaxStates], evdw[kMaxStates];
    int n = min((int64_t)s.cnt[C_QW], s.cap_qw);
    int sa = m.sa, S = m.S;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int j0 = m.nat_solute + sa * s.qw[p];
        for (int iq = 0; iq < m.nqat; ++iq) {
            int i = m.iqseq[iq];
            for (int a = 0; a < sa; ++a) {
                int j = j0 + a;
                bool lj = !SPC || a == 0;
                if constexpr (!MIX) {
                    double tx = s.x[3 * j] - s.x[3 * i], ty = s.x[3 * j + 1] - s.x[3 * i + 1],
                           tz = s.x[3 * j + 2] - s.x[3 * i + 2];
                    double r2 = 1.0 / (tx * tx + ty * ty + tz * tz);
                    double r = sqrt(r2);
                    double dvs = 0.0;
                    if (lj) {
                        double r6 = r2 * r2 * r2;
                        double r6hc = 1.0 / r6;
                        for (int st = 0; st < S; ++st) {
                            QPar q = m.qw_tab[(iq * sa + a) * S + st];
                            double vel, vdw, dv;
                            nbe_qx_d(r2, r, r6hc, q.A, q.B, q.el, q.sc, s.lambda[st], vel, vdw, dv);
                            dvs += dv;
                            eel[st].add(vel);
                            evdw[st].add(vdw);
                        }
                    } else {   // nbe_qspc, src/nonbonded.f90:226-243
                        for (int st = 0; st < S; ++st) {
                            QPar q = m.qw_tab[(iq * sa + a) * S + st];
                            double vel = q.el * r;
                            dvs += -r2 * vel * s.lambda[st];
                            eel[st].add(vel);
                        }
                    }
                    qs.add(iq, -tx * dvs, -ty * dvs, -tz * dvs);
                    acc.grad(j, tx * dvs, ty * dvs, tz * dvs);
                } else {
                    float4 xi = s.xq[i], xj = s.xq[j];
                    float tx = xj.x - xi.x, ty = xj.y - xi.y, tz = xj.z - xi.z;
                    float ri = rsqrtf(tx * tx + ty * ty + tz * tz);
                    float r2 = ri * ri;
                    float dvs = 0.0f;
                    if (lj) {
                        float r6 = r2 * r2 * r2;
                        float r6hc = 1.0f / r6;
                        for (int st = 0; st < S; ++st) {
                            QParF q = m.qw_tabf[(iq * sa + a) * S + st];
                            float vel, vdw, dv;
                            nbe_qx_f(r2, ri, r6hc, q.A, q.B, q.el, q.sc, (float)s.lambda[st], vel, vdw, dv);
                            dvs += dv;
                            eel[st].add(vel);
                            evdw[st].add(vdw);
                        }
                    } else {
                        for (int st = 0; st < S; ++st) {
                            QParF q = m.qw_tabf[(iq * sa + a) * S + st];
                            float vel = q.el * ri;
                            dvs += -r2 * vel * (float)s.lambda[st];
                            eel[st].add(vel);
                        }
                    }
                    qs.add(iq, -tx * dvs, -ty * dvs, -tz * dvs);
                    acc.grad(j, tx * dvs, ty * dvs, tz * dvs);
                }
            }
        }
    }
    for (int st = 0; st < S; ++st) {
        eel[st].flush(acc, eq_slot(st, 4));
        evdw[st].flush(acc, eq_slot(st, 5));
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * m.nqat; k += blockDim.x) {
        int i = m.iqseq[k / 3];
        if constexpr (MIX) atomicAdd(s.fix + 3 * i + k % 3, (unsigned long long)gq[k]);
        else atomicAdd(s.d + 3 * i + k % 3, (double)gq[k]);
    }
}

// nonbond_qp, src/nonbondene.f90:5157-5230 (qp_precomp, src/simprep.f90:3112-3148)
template <bool MIX>
__global__ void __launch_bounds__(256) k_qp(DevModel m, DevState s) {
    typedef typename std::conditional<MIX, unsigned long long, double>::type GT;
    __shared__ GT gq[3 * kMaxQ];
    for (int k = threadIdx.x; k < 3 * m.nqat; k += blockDim.x) gq[k] = GT(0);
    __syncthreads();
    QShared<MIX> qs{gq};
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel[kMaxStates], evdw[kMaxStates];
    int n = min((int64_t)s.cnt[C_QP], s.cap_qp);
    int S = m.S;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int j = s.qp[p];
        for (int iq = 0; iq < m.nqat; ++iq) {
            int i = m.iqseq[iq];
            size_t t0 = ((size_t)j * m.nqat + iq) * S;
            if constexpr (!MIX) {
                double tx = s.x[3 * j] - s.x[3 * i], ty = s.x[3 * j + 1] - s.x[3 * i + 1],
                       tz = s.x[3 * j + 2] - s.x[3 * i + 2];
                double r2 = 1.0 / (tx * tx + ty * ty + tz * tz);
                double r = sqrt(r2);
                double r6 = r2 * r2 * r2;
                double r6hc = 1.0 / r6;
                double dvs = 0.0;
                for (int st = 0; st < S; ++st) {
                    QPar q = m.qp_tab[t0 + st];
                    double vel, vdw, dv;
                    nbe_qx_d(r2, r, r6hc, q.A, q.B, q.el, q.sc, s.lambda[st], vel, vdw, dv);
                    dvs += dv;
                    eel[st].add(vel);
                    evdw[st].add(vdw);
                }
                qs.add(iq, -tx * dvs, -ty * dvs, -tz * dvs);
                acc.grad(j, tx * dvs, ty * dvs, tz * dvs);
            } else {
                float4 xi = s.xq[i], xj = s.xq[j];
                float tx = xj.x - xi.x, ty = xj.y - xi.y, tz = xj.z - xi.z;
                float ri = rsqrtf(tx * tx + ty * ty + tz * tz);
                float r2 = ri * ri;
                float r6 = r2 * r2 * r2;
                float r6hc = 1.0f / r6;
                float dvs = 0.0f;
                for (int st = 0; st < S; ++st) {
                    QParF q = m.qp_tabf[t0 + st];
                    float vel, vdw, dv;
                    nbe_qx_f(r2, ri, r6hc, q.A, q.B, q.el, q.sc, (float)s.lambda[st], vel, vdw, dv);
                    dvs += dv;
                    eel[st].add(vel);
                    evdw[st].add(vdw);
                }
                qs.add(iq, -tx * dvs, -ty * dvs, -tz * dvs);
                acc.grad(j, tx * dvs, ty * dvs, tz * dvs);
            }
        }
    }
    for (int st = 0; st < S; ++st) {
        eel[st].flush(acc, eq_slot(st, 2));
        evdw[st].flush(acc, eq_slot(st, 3));
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * m.nqat; k += blockDim.x) {
        int i = m.iqseq[k / 3];
        if constexpr (MIX) atomicAdd(s.fix + 3 * i + k % 3, (unsigned long long)gq[k]);
        else atomicAdd(s.d + 3 * i + k % 3, (double)gq[k]);
    }
}

// nonbond_qq + nonbond_qqp (static lists), src/nonbondene.f90:5013-5153,
// pair kernel nbe_qq, src/nonbonded.f90:111-150.  Always FP64: few pairs.
template <bool MIX>
__global__ void k_qq(DevModel m, DevState s) {
    Acc<MIX> acc = make_acc<MIX>(s);
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= s.nqq) return;
    QQEntry e = s.qq[p];
    double tx = s.x[3 * e.j] - s.x[3 * e.i], ty = s.x[3 * e.j + 1] - s.x[3 * e.i + 1],
           tz = s.x[3 * e.j + 2] - s.x[3 * e.i + 2];
    double r2 = 1.0 / (tx * tx + ty * ty + tz * tz);
    double r = sqrt(r2);
    double r6d = r2 * r2 * r2;
    double r6_hc = 1.0 / r6d;
    double r6 = 1.0 / (r6_hc + e.sc);
    double r12 = r6 * r6;
    double lam = s.lambda[e.s];
    double vel = e.el * r, va, vb, dv;
    if (e.soft) {
        vb = 0.0;
        va = e.A * exp(-e.B / r);
        dv = r2 * (-vel - e.B * va / r) * lam;
    } else {
        va = e.A * r12;
        vb = e.B * r6;
        dv = r2 * (-vel - (12.0 * va - 6.0 * vb) * r6 * r6_hc) * lam;
    }
    int kel = p < s.nqq_qq ? 0 : 2;
    if constexpr (!MIX) {
        acc.grad(e.i, -tx * dv, -ty * dv, -tz * dv);
        acc.grad(e.j, tx * dv, ty * dv, tz * dv);
        acc.energy(eq_slot(e.s, kel), vel);
        acc.energy(eq_slot(e.s, kel + 1), va - vb);
    } else {
        acc.gradd(e.i, -tx * dv, -ty * dv, -tz * dv);
        acc.gradd(e.j, tx * dv, ty * dv, tz * dv);
        acc.energy_fix(eq_slot(e.s, kel), to_fixd(vel));
        acc.energy_fix(eq_slot(e.s, kel + 1), to_fixd(va - vb));
    }
}

// lrf_taylor, src/nonbondene.f90:507-571 (FP64 in both forms)
template <bool MIX>
__global__ void __launch_bounds__(256) k_lrf_taylor(DevModel m, DevState s, const int* __restrict__ iwhich) {
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> elrf;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m.natom; i += gridDim.x * blockDim.x) {
        if (m.excl[i] || m.iqatom[i] >= 0) continue;
        const double* L = s.lrf + (size_t)iwhich[i] * kLrfLen;
        double dx = L[0] - s.x[3 * i], dy = L[1] - s.x[3 * i + 1], dz = L[2] - s.x[3 * i + 2];
        const double* p1 = L + 4;
        const double* p2 = L + 7;    // p2[3a + c]
        const double* p3 = L + 16;   // p3[3m + c]
        double t0 = dx * p2[0] + dy * p2[1] + dz * p2[2];
        double t1 = dx * p2[3] + dy * p2[4] + dz * p2[5];
        double t2 = dx * p2[6] + dy * p2[7] + dz * p2[8];
        double V = L[3] + (dx * p1[0] + dy * p1[1] + dz * p1[2]) + 0.5 * (dx * t0 + dy * t1 + dz * t2);
        elrf.add(0.5 * m.crg[i] * V);
        double df[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const double* q = p3 + 9 * a;
            double u0 = dx * q[0] + dy * q[1] + dz * q[2];
            double u1 = dx * q[3] + dy * q[4] + dz * q[5];
            double u2 = dx * q[6] + dy * q[7] + dz * q[8];
            df[a] = p1[a] + (dx * p2[3 * a] + dy * p2[3 * a + 1] + dz * p2[3 * a + 2]) +
                    0.5 * (dx * u0 + dy * u1 + dz * u2);
        }
        double q = m.crg[i];
        if constexpr (!MIX) acc.grad(i, -df[0] * q, -df[1] * q, -df[2] * q);
        else acc.gradd(i, -df[0] * q, -df[1] * q, -df[2] * q);
    }
    elrf.flush(acc, E_LRF);
}

// mixed form: add the fixed-point gradient into d and clear it
__global__ void k_apply_fixed(int n, unsigned long long* __restrict__ fix, double* __restrict__ d) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        long long v = (long long)fix[k];
        if (v != 0) {
            d[k] += (double)v * (1.0 / kFix);
            fix[k] = 0ull;
        }
    }
}

// =============================================================================
// Spherical-boundary solvent terms (FP64 in both forms)
// =============================================================================

// restrain_solvent, src/nonbondene.f90:6466-6544
template <bool MIX>
__global__ void k_restrain_solvent(DevModel m, DevState s, SolventDev p, double shift,
                                   const int* __restrict__ wsw, const uint8_t* __restrict__ heavy_solv) {
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> er;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < m.nwat; w += gridDim.x * blockDim.x) {
        int isw = wsw[w];
        if (m.excl[isw]) continue;
        int first = m.nat_solute + m.sa * w;
        for (int is = 0; is < m.sa; ++is) {
            int i, idist;
            if (m.sa == 3) {
                if (is > 0) break;
                i = idist = isw;
            } else {
                if (!heavy_solv[is]) continue;
                idist = first;
                i = first + is;
            }
            double vx = s.x[3 * idist] - m.xwcent[0], vy = s.x[3 * idist + 1] - m.xwcent[1],
                   vz = s.x[3 * idist + 2] - m.xwcent[2];
            double b = sqrt(vx * vx + vy * vy + vz * vz);
            double db = b - (p.rwat - shift);
            double erst, dv;
            if (db > 0.0) {
                erst = 0.5 * p.fk_wsphere * (db * db) - p.Dwmz;
                dv = p.fk_wsphere * db / b;
            } else if (b > 0.0) {
                double fexp = exp(p.awmz * db);
                erst = p.Dwmz * (fexp * fexp - 2.0 * fexp);
                dv = -2.0 * p.Dwmz * p.awmz * (fexp - fexp * fexp) / b;
            } else {
                erst = 0.0;
                dv = 0.0;
            }
            if constexpr (!MIX) acc.grad(i, vx * dv, vy * dv, vz * dv);
            else acc.gradd(i, vx * dv, vy * dv, vz * dv);
            er.add(erst);
        }
    }
    er.flush(acc, E_RST_RAD);
}

// watpol step 1 (src/nonbondene.f90:6566-6611): dipole angle theta and shell
__device__ __forceinline__ void water_vectors(const DevModel& m, const double* x, int w, double& rmx,
                                              double& rmy, double& rmz, double& rm, double& rcx, double& rcy,
                                              double& rcz, double& rc) {
    int i = m.nat_solute + m.sa * w;
    double ux = 0, uy = 0, uz = 0;
    if (m.sa == 3) {
        ux = x[3 * (i + 1)] + x[3 * (i + 2)] - 2.0 * x[3 * i];
        uy = x[3 * (i + 1) + 1] + x[3 * (i + 2) + 1] - 2.0 * x[3 * i + 1];
        uz = x[3 * (i + 1) + 2] + x[3 * (i + 2) + 2] - 2.0 * x[3 * i + 2];
        rcx = x[3 * i] - m.xwcent[0];
        rcy = x[3 * i + 1] - m.xwcent[1];
        rcz = x[3 * i + 2] - m.xwcent[2];
    } else {
        double cx = 0, cy = 0, cz = 0;
        for (int k = 0; k < m.sa; ++k) {
            cx += x[3 * (i + k)]; cy += x[3 * (i + k) + 1]; cz += x[3 * (i + k) + 2];
            ux += x[3 * (i + k)] * m.wcrg[k];
            uy += x[3 * (i + k) + 1] * m.wcrg[k];
            uz += x[3 * (i + k) + 2] * m.wcrg[k];
        }
        rcx = cx / m.sa - m.xwcent[0];
        rcy = cy / m.sa - m.xwcent[1];
        rcz = cz / m.sa - m.xwcent[2];
    }
    rm = sqrt(ux * ux + uy * uy + uz * uz);
    rmx = ux / rm; rmy = uy / rm; rmz = uz / rm;
    rc = sqrt(rcx * rcx + rcy * rcy + rcz * rcz);
    rcx /= rc; rcy /= rc; rcz /= rc;
}

__global__ void k_watpol_theta(DevModel m, DevState s, SolventDev p) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= m.nwat) return;
    s.shell[w] = -1;
    s.theta[w] = 0.0;
    int i = m.nat_solute + m.sa * w;
    if (m.excl[i]) return;
    double rmx, rmy, rmz, rm, rcx, rcy, rcz, rc;
    water_vectors(m, s.x, w, rmx, rmy, rmz, rm, rcx, rcy, rcz, rc);
    double scp = rmx * rcx + rmy * rcy + rmz * rcz;
    scp = fmin(1.0, fmax(-1.0, scp));
    s.theta[w] = acos(scp);
    int N = p.nshell;
    if (rc > p.rout[N - 1] - p.dr[N - 1]) {
        int is;
        for (is = N - 1; is >= 1; --is)
            if (rc <= p.rout[is]) break;
        if (is < 0) is = 0;
        s.shell[w] = is;
        atomicAdd(s.n_insh + is, 1);
    }
}

// stable selection order of src/nonbondene.f90:6612-6628: rank = number of
// waters of the same shell with smaller theta, ties broken by water index
__global__ void k_watpol_rank(DevModel m, DevState s) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= m.nwat) return;
    int sh = s.shell[w];
    if (sh < 0) return;
    double t = s.theta[w];
    int r = 0;
    for (int v = 0; v < m.nwat; ++v) {
        if (s.shell[v] != sh) continue;
        double tv = s.theta[v];
        r += (tv < t) || (tv == t && v < w);
    }
    s.rank[w] = r;
}

// theta_corr update every itdis steps, src/nonbondene.f90:6630-6645
__global__ void k_watpol_update(SolventDev p, double* wstate) {
    int is = threadIdx.x;
    if (is >= p.nshell) return;
    double* tc = wstate;
    double* av = wstate + kMaxShell;
    double* an = wstate + 2 * kMaxShell;
    av[is] = av[is] / p.itdis;
    an[is] = an[is] / p.itdis;
    tc[is] = tc[is] + av[is] - acos(p.cstb[is]);
    av[is] = 0.0;
    an[is] = 0.0;
}

// energy and gradient, src/nonbondene.f90:6646-6742
template <bool MIX>
__global__ void k_watpol_force(DevModel m, DevState s, SolventDev p, double* __restrict__ shell_tsum) {
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> ep;
    const double pi = 3.14159265358979323846;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < m.nwat; w += gridDim.x * blockDim.x) {
        int sh = s.shell[w];
        if (sh < 0) continue;
        int n = s.n_insh[sh];
        int il = s.rank[w] + 1;
        double arg = 1.0 + (1.0 - 2.0 * (double)il) / (double)n;
        double t0 = acos(arg);
        t0 = t0 - 3.0 * sin(t0) * p.cstb[sh] / 2.0;
        if (t0 < 0.0) t0 = 0.0;
        if (t0 > pi) t0 = pi;
        double th = s.theta[w];
        atomicAdd(shell_tsum + sh, th);
        double dth = th - t0 + s.wstate[sh];
        ep.add(0.5 * p.fkwpol * dth * dth);
        double dv = p.fkwpol * dth;
        double rmx, rmy, rmz, rm, rcx, rcy, rcz, rc;
        water_vectors(m, s.x, w, rmx, rmy, rmz, rm, rcx, rcy, rcz, rc);
        double scp = rmx * rcx + rmy * rcy + rmz * rcz;
        scp = fmin(1.0, fmax(-1.0, scp));
        double f0 = sin(acos(scp));
        if (fabs(f0) < 1.0e-10) f0 = 1.0e-10;
        f0 = dv * (-1.0 / f0);
        double f1x = (rcx - rmx * scp) * -2.0 / rm, f1y = (rcy - rmy * scp) * -2.0 / rm,
               f1z = (rcz - rmz * scp) * -2.0 / rm;
        double f3x = (rcx - rmx * scp) / rm, f3y = (rcy - rmy * scp) / rm, f3z = (rcz - rmz * scp) / rm;
        double f2x = (rmx - rcx * scp) / rc, f2y = (rmy - rcy * scp) / rc, f2z = (rmz - rcz * scp) / rc;
        int i = m.nat_solute + m.sa * w;
        if constexpr (!MIX) acc.grad(i, (f1x + f2x) * f0, (f1y + f2y) * f0, (f1z + f2z) * f0);
        else acc.gradd(i, (f1x + f2x) * f0, (f1y + f2y) * f0, (f1z + f2z) * f0);
        for (int k = 1; k < m.sa; ++k) {
            if constexpr (!MIX) acc.grad(i + k, f3x * f0, f3y * f0, f3z * f0);
            else acc.gradd(i + k, f3x * f0, f3y * f0, f3z * f0);
        }
    }
    ep.flush(acc, E_RST_POL);
}

// running averages (md only), src/nonbondene.f90:6738-6741
__global__ void k_watpol_average(SolventDev p, DevState s, const double* shell_tsum) {
    int is = threadIdx.x;
    if (is >= p.nshell) return;
    int n = s.n_insh[is];
    if (n == 0) return;
    s.wstate[kMaxShell + is] += shell_tsum[is] / (double)n;
    s.wstate[2 * kMaxShell + is] += (double)n;
}

// =============================================================================
// list export (parity tests): expand to the reference's atom pairs
// =============================================================================
__global__ void k_export(DevModel m, DevState s, int kind, int32_t* __restrict__ oi, int32_t* __restrict__ oj,
                         int64_t cap, int* __restrict__ ocount) {
    int sa = m.sa;
    int n = 0, mult = 1;
    switch (kind) {
        case QNB_LIST_WW: n = min((int64_t)s.cnt[C_WW], s.cap_ww); mult = sa * sa; break;
        case QNB_LIST_PW: n = min((int64_t)s.cnt[C_PW], s.cap_pw); mult = sa; break;
        case QNB_LIST_PP: case QNB_LIST_PP14: n = min((int64_t)s.cnt[C_PP], s.cap_pp); mult = 1; break;
        case QNB_LIST_QP: n = min((int64_t)s.cnt[C_QP], s.cap_qp); mult = m.nqat; break;
        case QNB_LIST_QW: n = min((int64_t)s.cnt[C_QW], s.cap_qw); mult = m.nqat * sa; break;
    }
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int64_t o = (int64_t)p * mult;
        if (kind == QNB_LIST_WW) {
            int2 e = s.ww[p];
            for (int la = 0; la < sa; ++la)
                for (int ka = 0; ka < sa; ++ka, ++o)
                    if (o < cap) { oi[o] = m.nat_solute + sa * e.x + la; oj[o] = m.nat_solute + sa * e.y + ka; }
        } else if (kind == QNB_LIST_PW) {
            int2 e = s.pw[p];
            for (int a = 0; a < sa; ++a, ++o)
                if (o < cap) { oi[o] = e.x; oj[o] = m.nat_solute + sa * e.y + a; }
        } else if (kind == QNB_LIST_PP) {
            int2 e = s.pp[p];
            if (o < cap) { oi[o] = e.x; oj[o] = e.y & 0x0fffffff; }
        } else if (kind == QNB_LIST_PP14) {
            int2 e = s.pp[p];
            if ((e.y >> 28) == 3) {
                int k = atomicAdd(ocount, 1);
                if (k < cap) { oi[k] = e.x; oj[k] = e.y & 0x0fffffff; }
            }
        } else if (kind == QNB_LIST_QP) {
            int j = s.qp[p];
            for (int iq = 0; iq < m.nqat; ++iq, ++o)
                if (o < cap) { oi[o] = iq; oj[o] = j; }
        } else if (kind == QNB_LIST_QW) {
            int w = s.qw[p];
            for (int iq = 0; iq < m.nqat; ++iq)
                for (int a = 0; a < sa; ++a, ++o)
                    if (o < cap) { oi[o] = iq; oj[o] = m.nat_solute + sa * w + a; }
        }
    }
}

// =============================================================================
// launch wrappers
// =============================================================================
namespace {
int g_sms = 0;
int sms() {
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 148;
    }
    return g_sms;
}
int blocks_for(int64_t n, int bs, int per_sm) {
    int64_t b = (n + bs - 1) / bs;
    int64_t lim = (int64_t)sms() * per_sm;
    if (b > lim) b = lim;
    return (int)(b < 1 ? 1 : b);
}
}  // namespace

void launch_group_centres(const DevModel& m, DevState& s, cudaStream_t st) {
    k_group_centres<<<(m.ncgp + 127) / 128, 128, 0, st>>>(m, s.x, s.lrf);
}
void launch_build_ww(const DevModel& m, DevState& s, const Cut& c, cudaStream_t st) {
    if (m.nwat == 0) return;
    k_build_ww<<<blocks_for((int64_t)m.nwat * 32, 256, 8), 256, 0, st>>>(m, s.x, s.ww, s.cap_ww, s.cnt + C_WW,
                                                                          c.rcww2);
}
void launch_build_pw(const DevModel& m, DevState& s, const Cut& c, cudaStream_t st) {
    if (m.nwat == 0 || m.ncgp_solute == 0) return;
    k_build_pw<<<blocks_for((int64_t)m.ncgp_solute * 32, 256, 8), 256, 0, st>>>(m, s.x, s.pw, s.cap_pw,
                                                                                 s.cnt + C_PW, c.rcpw2);
}
void launch_build_pp(const DevModel& m, DevState& s, const Cut& c, cudaStream_t st) {
    if (m.ncgp_solute == 0) return;
    k_build_pp<<<blocks_for((int64_t)m.ncgp_solute * 32, 256, 8), 256, 0, st>>>(
        m, s.x, s.pp, s.cap_pp, s.cnt + C_PP, s.cnt + C_PP14, c.rcpp2);
}
void launch_build_qw(const DevModel& m, DevState& s, const Cut& c, cudaStream_t st) {
    if (m.nwat == 0 || m.nqat == 0) return;
    k_build_qw<<<(m.nwat + 255) / 256, 256, 0, st>>>(m, s.x, s.qw, s.cap_qw, s.cnt + C_QW, c.rcq2);
}
void launch_build_qp_impl(const DevModel& m, DevState& s, const uint8_t* qnear, double rcq2, cudaStream_t st) {
    if (m.ncgp_solute == 0 || m.nqat == 0) return;
    k_build_qp<<<(m.ncgp_solute + 127) / 128, 128, 0, st>>>(m, s.x, qnear, s.qp, s.cap_qp, s.cnt + C_QP, rcq2);
}
void launch_lrf_accumulate(const DevModel& m, DevState& s, const Cut& c, int mixed, cudaStream_t st) {
    int b = blocks_for((int64_t)m.ncgp * 32, 128, 16);
    if (mixed) k_lrf_accumulate<true><<<b, 128, 0, st>>>(m, s.x, s.lrf, c);
    else k_lrf_accumulate<false><<<b, 128, 0, st>>>(m, s.x, s.lrf, c);
}
void launch_pack_mixed(const DevModel& m, DevState& s, cudaStream_t st) {
    k_pack_mixed<<<(m.natom + 255) / 256, 256, 0, st>>>(m, s.x, s.xq);
}

void launch_nonbond(const DevModel& m, DevState& s, int mixed, int md, cudaStream_t st, int* nl) {
    const int bs = 256;
    int bw = blocks_for(s.cap_ww, bs, 8), bp = blocks_for(s.cap_pw, bs, 8), bpp = blocks_for(s.cap_pp, bs, 8);
    int bq = blocks_for(s.cap_qw, bs, 4), bqp = blocks_for(s.cap_qp, bs, 4);
    bool spc = m.spc != 0;
    if (m.natom > m.nat_solute) {
        if (md) {
            if (mixed) { if (spc) k_ww<true, true><<<bw, bs, 0, st>>>(m, s); else k_ww<true, false><<<bw, bs, 0, st>>>(m, s); }
            else { if (spc) k_ww<false, true><<<bw, bs, 0, st>>>(m, s); else k_ww<false, false><<<bw, bs, 0, st>>>(m, s); }
            ++*nl;
        }
        if (m.nqat > 0) {
            if (mixed) { if (spc) k_qw<true, true><<<bq, bs, 0, st>>>(m, s); else k_qw<true, false><<<bq, bs, 0, st>>>(m, s); }
            else { if (spc) k_qw<false, true><<<bq, bs, 0, st>>>(m, s); else k_qw<false, false><<<bq, bs, 0, st>>>(m, s); }
            ++*nl;
        }
        if (md && m.ncgp_solute > 0) {
            if (mixed) k_pw<true><<<bp, bs, 0, st>>>(m, s); else k_pw<false><<<bp, bs, 0, st>>>(m, s);
            ++*nl;
        }
    }
    if (md && m.ncgp_solute > 0) {
        if (mixed) k_pp<true><<<bpp, bs, 0, st>>>(m, s); else k_pp<false><<<bpp, bs, 0, st>>>(m, s);
        ++*nl;
    }
    if (m.nqat > 0 && m.nat_solute > 0) {
        if (mixed) k_qp<true><<<bqp, bs, 0, st>>>(m, s); else k_qp<false><<<bqp, bs, 0, st>>>(m, s);
        ++*nl;
    }
}

void launch_nonbond_qq(const DevModel& m, DevState& s, int mixed, cudaStream_t st) {
    if (s.nqq == 0) return;
    int b = (s.nqq + 127) / 128;
    if (mixed) k_qq<true><<<b, 128, 0, st>>>(m, s); else k_qq<false><<<b, 128, 0, st>>>(m, s);
}

void launch_lrf_taylor_impl(const DevModel& m, DevState& s, const int* iwhich, int mixed, cudaStream_t st) {
    int b = blocks_for(m.natom, 256, 4);
    if (mixed) k_lrf_taylor<true><<<b, 256, 0, st>>>(m, s, iwhich);
    else k_lrf_taylor<false><<<b, 256, 0, st>>>(m, s, iwhich);
}

void launch_apply_fixed(const DevModel& m, DevState& s, cudaStream_t st) {
    int n = 3 * m.natom;
    k_apply_fixed<<<blocks_for(n, 256, 4), 256, 0, st>>>(n, s.fix, s.d);
}

void launch_restrain_solvent_impl(const DevModel& m, DevState& s, const SolventDev& p, double Tfree, int mixed,
                                  const int* wsw, const uint8_t* heavy_solv, cudaStream_t st) {
    if (m.nwat == 0) return;
    double shift = (p.fk_wsphere != 0.0) ? sqrt(p.boltz * Tfree / p.fk_wsphere) : 0.0;
    int b = blocks_for(m.nwat, 256, 4);
    if (mixed) k_restrain_solvent<true><<<b, 256, 0, st>>>(m, s, p, shift, wsw, heavy_solv);
    else k_restrain_solvent<false><<<b, 256, 0, st>>>(m, s, p, shift, wsw, heavy_solv);
}

void launch_watpol_impl(const DevModel& m, DevState& s, const SolventDev& p, int istep, int md, int mixed,
                        double* shell_tsum, cudaStream_t st, int* nl) {
    if (m.nwat == 0 || !p.wpol || p.nshell <= 0) return;
    int bw = (m.nwat + 255) / 256;
    if (md) {
        cudaMemsetAsync(s.n_insh, 0, sizeof(int) * kMaxShell, st);
        k_watpol_theta<<<bw, 256, 0, st>>>(m, s, p);
        k_watpol_rank<<<bw, 256, 0, st>>>(m, s);
        *nl += 2;
    }
    if (istep > 0 && md && (istep % (int)llround(p.itdis)) == 0) {
        k_watpol_update<<<1, kMaxShell, 0, st>>>(p, s.wstate);
        ++*nl;
    }
    cudaMemsetAsync(shell_tsum, 0, sizeof(double) * kMaxShell, st);
    if (mixed) k_watpol_force<true><<<bw, 256, 0, st>>>(m, s, p, shell_tsum);
    else k_watpol_force<false><<<bw, 256, 0, st>>>(m, s, p, shell_tsum);
    ++*nl;
    if (md) {
        k_watpol_average<<<1, kMaxShell, 0, st>>>(p, s, shell_tsum);
        ++*nl;
    }
}

void launch_export_pairs(const DevModel& m, const DevState& s, int kind, int32_t* di, int32_t* dj, int64_t cap,
                         int* dcount, cudaStream_t st) {
    k_export<<<blocks_for(1 << 20, 256, 8), 256, 0, st>>>(m, s, kind, di, dj, cap, dcount);
}

}  // namespace qnb
