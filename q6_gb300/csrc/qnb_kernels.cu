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

// The exact FP64 squared distance of two atoms, out of line: it serves the
// rare candidates whose FP32 distance falls inside a cut-off's rounding band.
// Inline, the compiler may evaluate it speculatively for every candidate, and
// each of its FP64 operations then takes an issue slot of GB300's narrow FP64
// pipe.
__device__ __noinline__ double dist2_exact_atoms(const double* __restrict__ x, int a, int b) {
    return dist2_exact(x[3 * a], x[3 * a + 1], x[3 * a + 2], x[3 * b], x[3 * b + 1], x[3 * b + 2]);
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
// v * 2^32 rounded to the nearest integer (ties to even) as a 64-bit two's
// complement value.  to_fix uses the hardware conversion, which executes on
// the FP64 pipe; to_fix_alu builds the same value from the IEEE-754 fields
// with integer instructions (saturated like cvt.rni.s64.f32, NaN gives 0),
// for kernels whose FP64 pipe is the bottleneck.  Which one pays is measured
// per kernel.
__device__ __forceinline__ unsigned long long to_fix(float v) {
    return (unsigned long long)__float2ll_rn(v * kFixF);
}
__device__ __forceinline__ unsigned long long to_fix_alu(float v) {
    unsigned u = __float_as_uint(v);
    int e = (int)((u >> 23) & 0xffu);
    unsigned m = (u & 0x7fffffu) | 0x800000u;
    int sh = e - 118;                     // v * 2^32 = m * 2^(e - 127 - 23 + 32)
    int ls = min(max(sh, 0), 39);
    int k = min(max(-sh, 0), 31);
    unsigned q = m >> k;
    unsigned rem = m & ((1u << k) - 1u), half = (1u << k) >> 1;
    q += (unsigned)((k > 0) & ((rem > half) | ((rem == half) & (q & 1u))));
    unsigned long long r = sh >= 0 ? ((unsigned long long)m << ls) : (unsigned long long)q;
    if (e == 0) r = 0ull;                 // zero and subnormals: |v * 2^32| < 2^-94
    bool sat = sh > 39;                   // |v| >= 2^31, infinities, NaN
    if (sat) r = (e == 255 && (u & 0x7fffffu)) ? 0ull : 0x7fffffffffffffffull;
    unsigned long long neg = (sat && r) ? 0x8000000000000000ull : 0ull - r;
    return (u >> 31) ? neg : r;
}
// The double form is built from the IEEE-754 fields with integer
// instructions, saturated like cvt.rni.s64.f64 (NaN gives 0): GB300 executes
// DMUL and double-to-int64 conversions on its FP64 pipe (1/64 of the FP32
// rate), which the FP64 kernels of the mixed form (LRF Taylor, Q-Q, solvent
// restraints) already keep busy.
__device__ __forceinline__ unsigned long long to_fixd(double v) {
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    int e = (int)((u >> 52) & 0x7ffull);
    unsigned long long m = (u & 0xfffffffffffffull) | 0x10000000000000ull;
    int sh = e - 1043;                    // v * 2^32 = m * 2^(e - 1023 - 52 + 32)
    int ls = min(max(sh, 0), 10);
    int k = min(max(-sh, 0), 63);
    unsigned long long q = m >> k;
    unsigned long long rem = m & ((1ull << k) - 1ull), half = (1ull << k) >> 1;
    q += (unsigned long long)((k > 0) & ((rem > half) | ((rem == half) & (q & 1ull))));
    unsigned long long r = sh >= 0 ? (m << ls) : q;
    if (e == 0) r = 0ull;
    bool sat = sh > 10;
    if (sat) r = (e == 2047 && (u & 0xfffffffffffffull)) ? 0ull : 0x7fffffffffffffffull;
    unsigned long long neg = (sat && r) ? 0x8000000000000000ull : 0ull - r;
    return (u >> 63) ? neg : r;
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
    __device__ __forceinline__ void grad_alu(int i, float gx, float gy, float gz) const {
        atomicAdd(f + 3 * i, to_fix_alu(gx));
        atomicAdd(f + 3 * i + 1, to_fix_alu(gy));
        atomicAdd(f + 3 * i + 2, to_fix_alu(gz));
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
__device__ __forceinline__ float warp_sum(float v) {
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
    __device__ __forceinline__ void add_alu(float x) { v += to_fix_alu(x); }
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
__global__ void k_group_centres(DevModel m, const DevState* __restrict__ states) {
    const double* __restrict__ x = states[blockIdx.y].x;
    double* __restrict__ lrf = states[blockIdx.y].lrf;
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

// FP32 coordinates relative to xpcent, charge in w (cut-off prefilter and
// mixed-form pair math)
__global__ void k_pack(DevModel m, const DevState* __restrict__ states) {
    const double* __restrict__ x = states[blockIdx.y].x;
    float4* __restrict__ xq = states[blockIdx.y].xq;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.natom) return;
    xq[i] = make_float4((float)(x[3 * i] - m.xpcent[0]), (float)(x[3 * i + 1] - m.xpcent[1]),
                        (float)(x[3 * i + 2] - m.xpcent[2]), (float)m.crg[i]);
}

__device__ __forceinline__ float r2_f(float4 a, float4 b) {
    float dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    return dx * dx + dy * dy + dz * dz;
}

// Exact cut-off decision r2 <= rc2.  The FP32 distance of centred
// coordinates (|x| within the sphere, relative error far below 1e-5 of r2)
// decides away from the boundary; within 2e-4 of it the FP64 distance in the
// reference's operation order decides, so the outcome is the FP64 one.  The
// FP32 band is built once per kernel: a double-to-float conversion per test
// would execute on the FP64 pipe.
struct Band {
    float lo, hi;   // r2f < lo: inside; r2f > hi: outside
    double c;       // the FP64 threshold
};
__device__ __forceinline__ Band band(double c, CutBand b) { return Band{b.lo, b.hi, c}; }
__device__ __forceinline__ Band band(double c) {
    float f = (float)c;
    return Band{f * 0.9998f, f * 1.0002f, c};
}
__device__ __forceinline__ bool within(float r2f, const Band& rc, const double* __restrict__ x, int a, int b) {
    if (r2f < rc.lo) return true;
    if (r2f > rc.hi) return false;
    return dist2_exact_atoms(x, a, b) <= rc.c;
}

// Any-atom group tests (iuse_switch_atom = 0): nbpplis2(_lrf) and
// nbpwlis2(_lrf), src/nonbondene.f90:1451-1468, 2565-2577.  A solute group
// pair is inside when any of its atom pairs (Q and excluded atoms included)
// is within the cut-off; a group and a water when any atom of the group is
// within the cut-off of the water's first atom.
__device__ __forceinline__ bool gg_inside_any(const DevModel& m, const double* __restrict__ x,
                                              const float4* __restrict__ xq, int g1, int g2, const Band& rc2) {
    int b0 = m.gslot[g2], b1 = m.gslot[g2 + 1];
    for (int a = m.gslot[g1]; a < m.gslot[g1 + 1]; ++a) {
        int i = m.gatom[a];
        float4 xi = xq[i];
        for (int b = b0; b < b1; ++b) {
            int j = m.gatom[b];
            if (within(r2_f(xi, xq[j]), rc2, x, i, j)) return true;
        }
    }
    return false;
}
__device__ __forceinline__ bool gw_inside_any(const DevModel& m, const double* __restrict__ x,
                                              const float4* __restrict__ xq, int g, int o, const Band& rc2) {
    float4 xo = xq[o];
    for (int a = m.gslot[g]; a < m.gslot[g + 1]; ++a) {
        int i = m.gatom[a];
        if (within(r2_f(xq[i], xo), rc2, x, i, o)) return true;
    }
    return false;
}
// solute group pair g1 != g2 inside the cut-off, in either mode
__device__ __forceinline__ bool gg_inside(const DevModel& m, const double* __restrict__ x,
                                          const float4* __restrict__ xq, int g1, int g2, const Band& rc2) {
    if (m.any_atom) return gg_inside_any(m, x, xq, g1, g2, rc2);
    int s1 = m.gsw[g1], s2 = m.gsw[g2];
    return within(r2_f(xq[s1], xq[s2]), rc2, x, s1, s2);
}
// solute group g and the water whose first atom is o, in either mode
__device__ __forceinline__ bool gw_inside(const DevModel& m, const double* __restrict__ x,
                                          const float4* __restrict__ xq, int g, int o, const Band& rc2) {
    if (m.any_atom) return gw_inside_any(m, x, xq, g, o, rc2);
    int s = m.gsw[g];
    return within(r2_f(xq[s], xq[o]), rc2, x, s, o);
}

// nbwwlist(_lrf) pair selection, src/nonbondene.f90:4274-4395: water pairs
// with O-O r2 <= Rcww2, neither O excluded.  Each unordered pair is kept once
// (iw < jw), the same set as the reference's parity rule.  A warp owns rows
// r and nwat-1-r so every warp scans about nwat candidates.
__global__ void k_build_ww(DevModel m, const DevState* __restrict__ states, double rc2d) {
    const Band rc2 = band(rc2d);
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const float4* __restrict__ xq = s.xq;
    int2* __restrict__ out = s.ww;
    int64_t cap = s.cap_ww;
    int* cnt = s.cnt + C_WW;
    int lane = threadIdx.x & 31;
    int half = (m.nwat + 1) / 2;
    for (int w = warp_id_global(); w < half; w += warps_total()) {
        for (int pass = 0; pass < 2; ++pass) {
            int iw = pass == 0 ? w : m.nwat - 1 - w;
            if (pass == 1 && iw == w) break;
            int io = m.nat_solute + m.sa * iw;
            if (m.excl[io]) continue;
            float4 xi = xq[io];
            for (int j0 = iw + 1; j0 < m.nwat; j0 += kWarp) {
                int jw = j0 + lane;
                bool ok = false;
                if (jw < m.nwat) {
                    int jo = m.nat_solute + m.sa * jw;
                    if (!m.excl[jo]) ok = within(r2_f(xi, xq[jo]), rc2, x, io, jo);
                }
                int pos = warp_append(cnt, ok ? 1 : 0);
                if (ok && pos < cap) out[pos] = make_int2(iw, jw);
            }
        }
    }
}

// nbpwlist(_lrf), src/nonbondene.f90:2842-2955: solute group switch atom to
// water O within Rcpw (nbpwlis2(_lrf), 2137-2242, 2493-2618: any atom of the
// group); every non-Q atom of the group pairs with the molecule.
__global__ void k_build_pw(DevModel m, const DevState* __restrict__ states, double rc2d) {
    const Band rc2 = band(rc2d);
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const float4* __restrict__ xq = s.xq;
    int2* __restrict__ out = s.pw;
    int64_t cap = s.cap_pw;
    int* cnt = s.cnt + C_PW;
    int lane = threadIdx.x & 31;
    for (int ig = warp_id_global(); ig < m.ncgp_solute; ig += warps_total()) {
        int is = m.gsw[ig];
        if (m.excl[is]) continue;
        int a0 = m.gslot[ig], a1 = m.gslot[ig + 1];
        int nq = 0;
        for (int a = a0; a < a1; ++a) nq += (m.iqatom[m.gatom[a]] < 0);
        if (nq == 0) continue;
        for (int j0 = 0; j0 < m.nwat; j0 += kWarp) {
            int jw = j0 + lane;
            bool ok = false;
            if (jw < m.nwat) {
                int jo = m.nat_solute + m.sa * jw;
                if (!m.excl[jo]) ok = gw_inside(m, x, xq, ig, jo, rc2);
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

// special (excluded / 1-4) status of one atom pair of a solute group pair
__device__ __forceinline__ int sg_find(const DevModel& m, long long key) {
    int lo = 0, hi = m.nsg - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        long long k = m.sg_key[mid];
        if (k == key) return mid;
        if (k < key) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}
__device__ __forceinline__ int sg_kind(const DevModel& m, int sgi, int sa, int sb) {
    if (sgi < 0) return 0;
    int want = sa | (sb << 8);
    for (int k = m.sg_off[sgi]; k < m.sg_off[sgi + 1]; ++k) {
        int e = m.sg_ent[k];
        if ((e & 0xffff) == want) return e >> 16;
    }
    return 0;
}

// reference list membership and LJ code of atom pair (i, j) of a solute group
// pair: pp_int_comp + precompute_set_values_pp, src/simprep.f90:2952-3065,
// 3321-3350 (0 = not listed, 3 = 1-4, else ljcod)
__device__ __forceinline__ int pp_accept(const DevModel& m, int i, int j, int kind) {
    if (kind == 1) return 0;
    int code = kind == 3 ? 3 : m.ljcod[m.iac[i] * m.natyps + m.iac[j]];
    int ti = m.iac[i], tj = m.iac[j];
    bool set = m.ljset[((code - 1) * m.natyps + ti) * m.natyps + tj] ||
               fabs(__dmul_rn(m.crg[i], m.crg[j])) > 1.0e-10;
    return set ? code : 0;
}

// nbpplist(_lrf) group selection, src/nonbondene.f90:1777-1908: solute group
// pairs whose switch atoms are within Rcpp, or any atom pairs for
// nbpplis2(_lrf), 950-1086, 1369-1516 (g1 <= g2; a group with itself is
// always listed).  Rows are paired like k_build_ww for balance.
__global__ void k_build_pp_groups(DevModel m, const DevState* __restrict__ states, double rc2d) {
    const Band rc2 = band(rc2d);
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const float4* __restrict__ xq = s.xq;
    int2* __restrict__ out = s.ppg;
    int64_t cap = s.cap_ppg;
    int* cnt = s.cnt + C_PPG;
    int lane = threadIdx.x & 31;
    int G = m.ncgp_solute, half = (G + 1) / 2;
    for (int w = warp_id_global(); w < half; w += warps_total()) {
        for (int pass = 0; pass < 2; ++pass) {
            int g1 = pass == 0 ? w : G - 1 - w;
            if (pass == 1 && g1 == w) break;
            int s1 = m.gsw[g1];
            if (m.excl[s1]) continue;
            for (int j0 = g1; j0 < G; j0 += kWarp) {
                int g2 = j0 + lane;
                bool ok = false;
                if (g2 < G) {
                    int s2 = m.gsw[g2];
                    if (!m.excl[s2]) ok = (g2 == g1) || gg_inside(m, x, xq, g1, g2, rc2);
                }
                int pos = warp_append(cnt, ok ? 1 : 0);
                if (ok && pos < cap) out[pos] = make_int2(g1, g2);
            }
        }
    }
}

// expands listed solute group pairs into the reference's atom pairs
// (i, j | code << 28); one thread per group pair
__global__ void k_expand_pp(DevModel m, const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.y];
    const int2* __restrict__ groups = s.ppg;
    const int* ngroups = s.cnt + C_PPG;
    int64_t gcap = s.cap_ppg;
    int2* __restrict__ out = s.pp;
    int64_t cap = s.cap_pp;
    int* cnt = s.cnt + C_PP;
    int* cnt14 = s.cnt + C_PP14;
    int n = min((int64_t)*ngroups, gcap);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int2 g = groups[p];
        int a0 = m.gslot[g.x], a1 = m.gslot[g.x + 1], b0 = m.gslot[g.y], b1 = m.gslot[g.y + 1];
        int sgi = m.nsg ? sg_find(m, (long long)g.x * m.ncgp_solute + g.y) : -1;
        int na = 0, n14 = 0;
        for (int pass = 0; pass < 2; ++pass) {
            int pos = 0;
            if (pass == 1) {
                if (na == 0) break;
                pos = atomicAdd(cnt, na);
                if (n14) atomicAdd(cnt14, n14);
            }
            for (int a = a0; a < a1; ++a) {
                int i = m.gatom[a];
                if (m.iqatom[i] >= 0) continue;
                for (int b = b0; b < b1; ++b) {
                    int j = m.gatom[b];
                    if (m.iqatom[j] >= 0) continue;
                    int sa = a - a0, sb = b - b0;
                    if (g.x == g.y) {
                        if (i >= j) continue;
                    }
                    int code = pp_accept(m, i, j, sg_kind(m, sgi, sa, sb));
                    if (!code) continue;
                    if (pass == 0) {
                        ++na;
                        n14 += (code == 3);
                    } else {
                        if (pos < cap) out[pos] = make_int2(i, j | (code << 28));
                        ++pos;
                    }
                }
            }
        }
    }
}

// Exclusive prefix sum of v over the block (blockDim.x a multiple of 32, at
// most 1024); *total receives the block sum.  Used for ordered appends.
__device__ __forceinline__ int block_excl_scan(int v, int* total) {
    __shared__ int wsum[32];
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    __syncthreads();   // wsum reuse across calls
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nw ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += t;
        }
        if (lane < nw) wsum[lane] = w;   // inclusive over warps
    }
    __syncthreads();
    *total = wsum[nw - 1];
    return (warp ? wsum[warp - 1] : 0) + incl - v;
}

// nbqplist, src/nonbondene.f90:3647-3742: solute groups whose switch atom is
// within Rcq of the solute centre (nbqplis2, 3408-3519: any atom of the
// group); atoms not bonded/angled to any Q atom.  One block per window
// appends in group order, so the list order is deterministic.
__global__ void __launch_bounds__(1024) k_build_qp(DevModel m, const DevState* __restrict__ states,
                                                   const uint8_t* __restrict__ qnear, double rcq2) {
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    int* __restrict__ out = s.qp;
    const int64_t cap = s.cap_qp;
    int base = 0;
    for (int g0 = 0; g0 < m.ncgp_solute; g0 += blockDim.x) {
        int ig = g0 + threadIdx.x, na = 0;
        if (ig < m.ncgp_solute && !m.excl[m.gsw[ig]]) {
            bool inside = false;
            if (m.any_atom) {   // nbqplis2, src/nonbondene.f90:3477-3487
                for (int a = m.gslot[ig]; a < m.gslot[ig + 1] && !inside; ++a) {
                    int i = m.gatom[a];
                    inside = dist2_exact(x[3 * i], x[3 * i + 1], x[3 * i + 2], m.xpcent[0], m.xpcent[1],
                                         m.xpcent[2]) <= rcq2;
                }
            } else {
                int is = m.gsw[ig];
                inside = dist2_exact(x[3 * is], x[3 * is + 1], x[3 * is + 2], m.xpcent[0], m.xpcent[1],
                                     m.xpcent[2]) <= rcq2;
            }
            if (inside)
                for (int a = m.gslot[ig]; a < m.gslot[ig + 1]; ++a) na += !qnear[m.gatom[a]];
        }
        int tot;
        int pos = base + block_excl_scan(na, &tot);
        if (na)
            for (int a = m.gslot[ig]; a < m.gslot[ig + 1]; ++a) {
                int i = m.gatom[a];
                if (qnear[i]) continue;
                if (pos < cap) out[pos] = i;
                ++pos;
            }
        base += tot;
    }
    if (threadIdx.x == 0) s.cnt[C_QP] = base;
}

// nbqwlist, src/nonbondene.f90:3862-3944: waters with O within Rcq of xpcent,
// appended in water order by one block per window
__global__ void __launch_bounds__(1024) k_build_qw(DevModel m, const DevState* __restrict__ states, double rcq2) {
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    int* __restrict__ out = s.qw;
    const int64_t cap = s.cap_qw;
    int base = 0;
    for (int w0 = 0; w0 < m.nwat; w0 += blockDim.x) {
        int iw = w0 + threadIdx.x;
        bool ok = false;
        if (iw < m.nwat) {
            int io = m.nat_solute + m.sa * iw;
            ok = !m.excl[io] && dist2_exact(x[3 * io], x[3 * io + 1], x[3 * io + 2], m.xpcent[0], m.xpcent[1],
                                            m.xpcent[2]) <= rcq2;
        }
        int tot;
        int pos = base + block_excl_scan(ok ? 1 : 0, &tot);
        if (ok && pos < cap) out[pos] = iw;
        base += tot;
    }
    if (threadIdx.x == 0) s.cnt[C_QW] = base;
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

// lrf_update's sums (src/nonbondene.f90:628-725) regrouped by symmetry: per
// source atom (dr from the target centre, charge q)
//   m[0]      phi0 += f0 r2
//   m[1..3]   phi1 -= dr f0
//   m[4..9]   S2(ab)  += f1 dr_a dr_b        (a <= b; phi2(a)_b = S2(ab) - [a==b] F0)
//   m[10]     F0      += f0
//   m[11..20] S3(abc) += 5 f2 dr_a dr_b dr_c (a <= b <= c)
//   m[21..23] U(c)    += f2 r2 dr_c
// with f0 = q/r^3, f1 = 3 f0/r^2, f2 = -f1/r^2.  lrf_expand rebuilds the 40
// reference coefficients, including its diagonal corrections of phi3.
constexpr int kLrfMom = kLrfMoments;
template <typename T>
__device__ __forceinline__ void lrf_terms(T dx, T dy, T dz, T q, T* m) {
    T r2 = dx * dx + dy * dy + dz * dz;
    T ri2, f0;
    if constexpr (std::is_same<T, float>::value) {
        float ri = rsqrtf(r2);
        ri2 = ri * ri;
        f0 = q * ri * ri2;
    } else {
        ri2 = 1.0 / r2;
        f0 = q / (r2 * sqrt(r2));
    }
    T f1 = T(3) * f0 * ri2;
    T f2 = -f1 * ri2;
    m[0] += f0 * r2;
    m[1] -= dx * f0;
    m[2] -= dy * f0;
    m[3] -= dz * f0;
    T ax = dx * f1, ay = dy * f1, az = dz * f1;
    m[4] += ax * dx; m[5] += ax * dy; m[6] += ax * dz;
    m[7] += ay * dy; m[8] += ay * dz; m[9] += az * dz;
    m[10] += f0;
    T g = T(5) * f2;
    T gxx = g * dx * dx, gyy = g * dy * dy, gzz = g * dz * dz, gxy = g * dx * dy, gxz = g * dx * dz,
      gyz = g * dy * dz;
    m[11] += gxx * dx;   // xxx
    m[12] += gxx * dy;   // xxy
    m[13] += gxx * dz;   // xxz
    m[14] += gyy * dx;   // xyy
    m[15] += gxy * dz;   // xyz
    m[16] += gzz * dx;   // xzz
    m[17] += gyy * dy;   // yyy
    m[18] += gyy * dz;   // yyz
    m[19] += gzz * dy;   // yzz
    m[20] += gzz * dz;   // zzz
    T h = f2 * r2;
    m[21] += h * dx;
    m[22] += h * dy;
    m[23] += h * dz;
}

// 40 reference coefficients (phi0, phi1(3), phi2(3x3), phi3(9x3)) from the moments
__device__ __forceinline__ void lrf_expand(const double* m, double* L) {
    // S3 index of the sorted triple (a<=b<=c)
    auto s3 = [&](int a, int b, int c) -> double {
        int t;
        if (a > b) { t = a; a = b; b = t; }
        if (b > c) { t = b; b = c; c = t; }
        if (a > b) { t = a; a = b; b = t; }
        const int idx[3][3][3] = {{{11, 12, 13}, {12, 14, 15}, {13, 15, 16}},
                                  {{12, 14, 15}, {14, 17, 18}, {15, 18, 19}},
                                  {{13, 15, 16}, {15, 18, 19}, {16, 19, 20}}};
        return m[idx[a][b][c]];
    };
    const int i2[3][3] = {{4, 5, 6}, {5, 7, 8}, {6, 8, 9}};
    L[0] = m[0];
    L[1] = m[1];
    L[2] = m[2];
    L[3] = m[3];
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) L[4 + 3 * a + c] = m[i2[a][c]] - (a == c ? m[10] : 0.0);
    for (int n = 0; n < 3; ++n)
        for (int j = 0; j < 3; ++j)
            for (int c = 0; c < 3; ++c) L[13 + 3 * (j + 3 * n) + c] = s3(n, j, c);
    const double* U = m + 21;
    double* P = L + 13;
    P[0] -= 3.0 * U[0]; P[1] -= U[1]; P[2] -= U[2];
    P[3] -= U[1]; P[4] -= U[0];
    P[6] -= U[2];
    P[8] -= U[0];
    P[9] -= U[1]; P[10] -= U[0];
    P[12] -= U[0]; P[13] -= 3.0 * U[1]; P[14] -= U[2];
    P[16] -= U[2]; P[17] -= U[1];
    P[18] -= U[2];
    P[20] -= U[0];
    P[22] -= U[2]; P[23] -= U[1];
    P[24] -= U[0]; P[25] -= U[1]; P[26] -= 3.0 * U[2];
}

// The mixed form's LRF sums with 20 moments: the sums m[10] and m[21..23] of
// lrf_terms follow from the others, F0 = tr S2 / 3 (f1 r2 = 3 f0) and
// U(c) = (S3(xxc) + S3(yyc) + S3(zzc)) / 5 (dr_x^2 + dr_y^2 + dr_z^2 = r2), so
// they are formed in FP64 from the totals instead of summed per atom.
//   n[0] phi0, n[1..3] phi1, n[4..9] S2, n[10..19] S3 (the order of lrf_terms)
constexpr int kLrfMom20 = 20;
__device__ __forceinline__ void lrf_terms20(float dx, float dy, float dz, float q, float* n) {
    const float r2 = dx * dx + dy * dy + dz * dz;
    const float ri = rsqrtf(r2), ri2 = ri * ri;
    const float qri = q * ri;
    const float f0 = qri * ri2;
    const float f1 = 3.f * f0 * ri2;
    const float g = -5.f * f1 * ri2;   // 5 f2
    n[0] += qri;                        // f0 r2
    n[1] -= dx * f0;
    n[2] -= dy * f0;
    n[3] -= dz * f0;
    const float ax = dx * f1, ay = dy * f1, az = dz * f1;
    n[4] += ax * dx; n[5] += ax * dy; n[6] += ax * dz;
    n[7] += ay * dy; n[8] += ay * dz; n[9] += az * dz;
    const float gx = g * dx, gy = g * dy, gz = g * dz;
    const float gxx = gx * dx, gyy = gy * dy, gzz = gz * dz, gxy = gx * dy;
    n[10] += gxx * dx;   // xxx
    n[11] += gxx * dy;   // xxy
    n[12] += gxx * dz;   // xxz
    n[13] += gyy * dx;   // xyy
    n[14] += gxy * dz;   // xyz
    n[15] += gzz * dx;   // xzz
    n[16] += gyy * dy;   // yyy
    n[17] += gyy * dz;   // yyz
    n[18] += gzz * dy;   // yzz
    n[19] += gzz * dz;   // zzz
}
// the 24 moments of lrf_expand from the 20 (FP64)
__device__ __forceinline__ void lrf_moments24(const double* n, double* m) {
    for (int k = 0; k < 10; ++k) m[k] = n[k];
    m[10] = (n[4] + n[7] + n[9]) / 3.0;
    for (int k = 0; k < 10; ++k) m[11 + k] = n[10 + k];
    m[21] = (n[10] + n[13] + n[15]) / 5.0;   // xxx + xyy + xzz
    m[22] = (n[11] + n[16] + n[18]) / 5.0;   // xxy + yyy + yzz
    m[23] = (n[12] + n[17] + n[19]) / 5.0;   // xxz + yyz + zzz
}

// LRF classification of a group pair: true when rc2 < r2 <= rlrf2 in FP64
__device__ __forceinline__ bool lrf_pair(float r2f, const Band& rc, const Band& rl, const double* __restrict__ x,
                                         int a, int b) {
    if (r2f > rc.hi && r2f < rl.lo) return true;
    if (r2f < rc.lo || r2f > rl.hi) return false;
    double r2 = dist2_exact_atoms(x, a, b);
    return r2 > rc.c && r2 <= rl.c;
}

// One warp per target group g2 sums the far-field contributions of every
// non-Q atom whose group is classified "LRF" against g2; the 40 coefficients
// are then reduced across the warp.  The warps of a block take consecutive
// targets and stream the source atoms through shared memory together: each
// atom (position, charge, its group's distance atom) is loaded from global
// memory once per block instead of once per target.  Mixed form: FP32 terms
// (rsqrt on the SFU); FP64 form: FP64 terms.
constexpr int kLrfBlock = 256;
template <bool MIX>
__global__ void __launch_bounds__(kLrfBlock) k_lrf_accumulate(DevModel m, const DevState* __restrict__ states, Cut c,
                                                              const int* __restrict__ lrf_src) {
    typedef typename std::conditional<MIX, float, double>::type T;
    const Band bpp = band(c.rcpp2, c.fpp), bpw = band(c.rcpw2, c.fpw), bww = band(c.rcww2, c.fww),
               blrf = band(c.rlrf2, c.flrf);
    __shared__ float4 s_xs[kLrfBlock];                  // distance atom of the source's group
    __shared__ int s_src[kLrfBlock];                    // lrf_src entry (-1: not a source)
    __shared__ T s_xi[4 * kLrfBlock];                   // source x, y, z (centred in FP32), charge
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const float4* __restrict__ xq = s.xq;
    double* __restrict__ lrf = s.lrf;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = kLrfBlock / 32;
    for (int gbase = blockIdx.x * nw; gbase < m.ncgp; gbase += gridDim.x * nw) {   // block-uniform
        const int g2 = gbase + warp;
        int s2 = 0;
        bool act = g2 < m.ncgp;
        if (act) {
            s2 = group_dist_atom(m, g2);
            act = !m.excl[s2];
        }
        const bool sol2 = act && g2 < m.ncgp_solute;
        const Band rc_s = sol2 ? bpp : bpw, rc_w = sol2 ? bpw : bww;
        double cx = 0.0, cy = 0.0, cz = 0.0;
        float4 x2 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (act) {
            const double* L = lrf + (size_t)g2 * kLrfLen;
            cx = L[0]; cy = L[1]; cz = L[2];
            x2 = xq[s2];
        }
        const T ccx = MIX ? T(cx - m.xpcent[0]) : T(cx), ccy = MIX ? T(cy - m.xpcent[1]) : T(cy),
                ccz = MIX ? T(cz - m.xpcent[2]) : T(cz);
        T mom[kLrfMom];
#pragma unroll
        for (int k = 0; k < kLrfMom; ++k) mom[k] = T(0);
        for (int i0 = 0; i0 < m.natom; i0 += kLrfBlock) {
            __syncthreads();
            {
                int i = i0 + threadIdx.x, t = threadIdx.x;
                int src = i < m.natom ? lrf_src[i] : -1;
                s_src[t] = src;
                if (src >= 0) {
                    s_xs[t] = xq[src & 0x3fffffff];
                    if constexpr (MIX) {
                        float4 xi = xq[i];
                        s_xi[4 * t] = xi.x; s_xi[4 * t + 1] = xi.y; s_xi[4 * t + 2] = xi.z; s_xi[4 * t + 3] = xi.w;
                    } else {
                        s_xi[4 * t] = x[3 * i]; s_xi[4 * t + 1] = x[3 * i + 1]; s_xi[4 * t + 2] = x[3 * i + 2];
                        s_xi[4 * t + 3] = m.crg[i];
                    }
                }
            }
            __syncthreads();
            if (!act) continue;
            const int n = min(kLrfBlock, m.natom - i0);
            for (int k = lane; k < n; k += kWarp) {
                int src = s_src[k];   // distance atom of i's group | solute flag << 30
                if (src < 0) continue;
                int s1 = src & 0x3fffffff;
                if (s1 == s2) continue;   // same group
                const Band& rc2 = (src >> 30) ? rc_s : rc_w;
                if (!lrf_pair(r2_f(x2, s_xs[k]), rc2, blrf, x, s2, s1)) continue;
                lrf_terms<T>(s_xi[4 * k] - ccx, s_xi[4 * k + 1] - ccy, s_xi[4 * k + 2] - ccz, s_xi[4 * k + 3], mom);
            }
        }
        if (!act) continue;
        double tot[kLrfMom];
#pragma unroll
        for (int k = 0; k < kLrfMom; ++k) {
            T v = mom[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
            tot[k] = (double)v;
        }
        if (lane == 0) lrf_expand(tot, lrf + (size_t)g2 * kLrfLen + 3);
    }
}

// Mixed form, two target groups per warp: every lane applies the source atom
// it loaded to both targets, so the shared-memory loads and the loop
// overhead of a source atom are paid once for two targets (the kernel is
// issue-bound: about 90 instructions per target and source with one target
// per warp).  Sums and their order per target are those of k_lrf_accumulate.
constexpr int kLrfPair = 2;
__global__ void __launch_bounds__(kLrfBlock) k_lrf_accumulate2(DevModel m, const DevState* __restrict__ states, Cut c,
                                                               const int* __restrict__ lrf_src) {
    const Band bpp = band(c.rcpp2, c.fpp), bpw = band(c.rcpw2, c.fpw), bww = band(c.rcww2, c.fww),
               blrf = band(c.rlrf2, c.flrf);
    __shared__ float4 s_xs[kLrfBlock];
    __shared__ int s_src[kLrfBlock];
    __shared__ float4 s_xi[kLrfBlock];
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const float4* __restrict__ xq = s.xq;
    double* __restrict__ lrf = s.lrf;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = kLrfBlock / 32;
    const int per_block = nw * kLrfPair;
    for (int gbase = blockIdx.x * per_block; gbase < m.ncgp; gbase += gridDim.x * per_block) {   // block-uniform
        int g2[kLrfPair], s2[kLrfPair];
        bool act[kLrfPair];
        Band rc_s[kLrfPair], rc_w[kLrfPair];
        float4 x2[kLrfPair];
        float ccx[kLrfPair], ccy[kLrfPair], ccz[kLrfPair];
        float mom[kLrfPair][kLrfMom];
#pragma unroll
        for (int t = 0; t < kLrfPair; ++t) {
            g2[t] = gbase + kLrfPair * warp + t;
            s2[t] = 0;
            act[t] = g2[t] < m.ncgp;
            if (act[t]) {
                s2[t] = group_dist_atom(m, g2[t]);
                act[t] = !m.excl[s2[t]];
            }
            const bool sol2 = act[t] && g2[t] < m.ncgp_solute;
            rc_s[t] = sol2 ? bpp : bpw;
            rc_w[t] = sol2 ? bpw : bww;
            double cx = 0.0, cy = 0.0, cz = 0.0;
            x2[t] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (act[t]) {
                const double* L = lrf + (size_t)g2[t] * kLrfLen;
                cx = L[0]; cy = L[1]; cz = L[2];
                x2[t] = xq[s2[t]];
            }
            ccx[t] = (float)(cx - m.xpcent[0]);
            ccy[t] = (float)(cy - m.xpcent[1]);
            ccz[t] = (float)(cz - m.xpcent[2]);
#pragma unroll
            for (int k = 0; k < kLrfMom; ++k) mom[t][k] = 0.f;
        }
        const bool any = act[0] || act[1];
        for (int i0 = 0; i0 < m.natom; i0 += kLrfBlock) {
            __syncthreads();
            {
                int i = i0 + threadIdx.x, t = threadIdx.x;
                int src = i < m.natom ? lrf_src[i] : -1;
                s_src[t] = src;
                if (src >= 0) {
                    s_xs[t] = xq[src & 0x3fffffff];
                    s_xi[t] = xq[i];
                }
            }
            __syncthreads();
            if (!any) continue;
            const int n = min(kLrfBlock, m.natom - i0);
            for (int k = lane; k < n; k += kWarp) {
                int src = s_src[k];   // distance atom of i's group | solute flag << 30
                if (src < 0) continue;
                const int s1 = src & 0x3fffffff;
                const bool sol1 = (src >> 30) != 0;
                const float4 xs = s_xs[k], xi = s_xi[k];
#pragma unroll
                for (int t = 0; t < kLrfPair; ++t) {
                    if (!act[t] || s1 == s2[t]) continue;
                    const Band& rc2 = sol1 ? rc_s[t] : rc_w[t];
                    if (!lrf_pair(r2_f(x2[t], xs), rc2, blrf, x, s2[t], s1)) continue;
                    lrf_terms<float>(xi.x - ccx[t], xi.y - ccy[t], xi.z - ccz[t], xi.w, mom[t]);
                }
            }
        }
#pragma unroll
        for (int t = 0; t < kLrfPair; ++t) {
            if (!act[t]) continue;   // warp-uniform
            double tot[kLrfMom];
#pragma unroll
            for (int k = 0; k < kLrfMom; ++k) {
                float v = mom[t][k];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
                tot[k] = (double)v;
            }
            if (lane == 0) lrf_expand(tot, lrf + (size_t)g2[t] * kLrfLen + 3);
        }
    }
}

// lattice shift and minimum-image distance of two atoms (periodic box)
__device__ __forceinline__ void box_shift(const DevModel& m, const double* __restrict__ x, int a, int b,
                                          double& sx, double& sy, double& sz) {
    sx = m.boxl[0] * round((x[3 * a] - x[3 * b]) * m.inv_boxl[0]);
    sy = m.boxl[1] * round((x[3 * a + 1] - x[3 * b + 1]) * m.inv_boxl[1]);
    sz = m.boxl[2] * round((x[3 * a + 2] - x[3 * b + 2]) * m.inv_boxl[2]);
}
// q_dist4(shift, boxlength*q_nint(shift*inv_boxl)) of atoms a and b
__device__ __forceinline__ double box_d2(const DevModel& m, const double* __restrict__ x, int a, int b) {
    double r2 = 0.0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        double d = x[3 * a + c] - x[3 * b + c];
        double t = m.boxl[c] * round(d * m.inv_boxl[c]) - d;
        r2 += t * t;
    }
    return r2;
}
// ---- box LRF (the LRF branch of nbpplist_box_lrf, nbpwlist_box_lrf and
// nbwwlist_box_lrf, src/nonbondene.f90:1910-2055, 2957-3085, 4397-4515, and
// the shift of lrf_update, 636-643).  A unit pair is classified by the
// minimum-image distance of its switch atoms; the source's atoms enter the
// target's moments at x_i - shift, shift = boxlength * nint((x_switch(source)
// - centre(target)) / boxlength).  In FP32 a lattice index whose fraction lies
// within 1e-4 of one half (where FP32 and FP64 could round apart) is
// recomputed in FP64 from the atoms, as are distances within the decision
// bands.
__device__ __forceinline__ bool near_half(float t) {
    float a = fabsf(t);
    return fabsf(a - truncf(a) - 0.5f) < 1e-4f;
}
__device__ __noinline__ bool lrf_pair_box_exact(const DevModel& m, const double* __restrict__ x, int a, int b,
                                                double rc2, double rl2) {
    const double r2 = box_d2(m, x, a, b);
    return r2 > rc2 && r2 <= rl2;
}
// target switch atom a, source switch atom b (packed positions)
__device__ __forceinline__ bool lrf_pair_box(const DevModel& m, float4 pa, float4 pb, const Band& rc, const Band& rl,
                                             const double* __restrict__ x, int a, int b) {
    const float dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
    const float tx = dx * m.inv_boxlf[0], ty = dy * m.inv_boxlf[1], tz = dz * m.inv_boxlf[2];
    if (near_half(tx) || near_half(ty) || near_half(tz)) return lrf_pair_box_exact(m, x, a, b, rc.c, rl.c);
    const float ex = m.boxlf[0] * roundf(tx) - dx, ey = m.boxlf[1] * roundf(ty) - dy, ez = m.boxlf[2] * roundf(tz) - dz;
    const float r2f = ex * ex + ey * ey + ez * ez;
    if (r2f > rc.hi && r2f < rl.lo) return true;
    if (r2f < rc.lo || r2f > rl.hi) return false;
    return lrf_pair_box_exact(m, x, a, b, rc.c, rl.c);
}
// lattice shift of source switch atom b against the target centre (FP64 centre
// cd, packed FP32 centre cf)
__device__ __noinline__ float3 lrf_shift_exact(const DevModel& m, const double* __restrict__ x, int b,
                                                const double* __restrict__ cd) {
    float3 r;
    r.x = (float)(m.boxl[0] * round((x[3 * b] - cd[0]) * m.inv_boxl[0]));
    r.y = (float)(m.boxl[1] * round((x[3 * b + 1] - cd[1]) * m.inv_boxl[1]));
    r.z = (float)(m.boxl[2] * round((x[3 * b + 2] - cd[2]) * m.inv_boxl[2]));
    return r;
}
__device__ __forceinline__ float3 lrf_shift(const DevModel& m, float4 pb, float cx, float cy, float cz,
                                            const double* __restrict__ x, int b, const double* __restrict__ cd) {
    const float tx = (pb.x - cx) * m.inv_boxlf[0], ty = (pb.y - cy) * m.inv_boxlf[1], tz = (pb.z - cz) * m.inv_boxlf[2];
    if (near_half(tx) || near_half(ty) || near_half(tz)) return lrf_shift_exact(m, x, b, cd);
    return make_float3(m.boxlf[0] * roundf(tx), m.boxlf[1] * roundf(ty), m.boxlf[2] * roundf(tz));
}

// Mixed form, N-body layout: one thread per target group.  The blocks stage
// the LRF source groups (the eligible atoms of each charge group, in group
// order: lrf_gmeta / lrf_goff / lrf_gatom) in shared memory, kLrfGT groups
// per tile, and every thread reads them as broadcasts.  The group-pair
// classification runs once per (target, source group); the source group's
// atoms then add their terms.  Each thread's 20 moment sums (lrf_terms20) run
// in FP32 over at most kLrfFold source groups and are then folded into a
// double-float accumulator with Knuth's TwoSum (s = a + b, bb = s - a,
// e = (a - (s - bb)) + (b - bb)), so the FP32 rounding of the sums is kept
// to short runs.  The source groups are split into nsplit ranges
// (blockIdx.z, the split fixed by the topology) whose moments
// k_lrf_combine adds in range order: each target's order of terms is fixed,
// so its coefficients do not depend on the launch or the number of windows.
constexpr int kLrfNB = 64;     // targets per block
constexpr int kLrfGT = 64;     // source groups per staged tile
constexpr int kLrfFold = 8;    // source groups per FP32 partial sum

__device__ __forceinline__ void two_sum_fold(float& hi, float& lo, float& p) {
    float s = __fadd_rn(hi, p);
    float bb = __fsub_rn(s, hi);
    float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, e);
    p = 0.f;
}

// The 20 moments of lrf_terms20 in packed FP32x2 arithmetic: the source
// atom's (x, y) and (z, q) arrive as register pairs from the staged float4,
// and the 20 sums are held as 10 pairs, so 10 FFMA2 replace 20 FFMA.  Each
// sum gets the same products in the same order as in lrf_terms20.  Slots
// (lrf_slot):
// (n1,n2) (n3,n0) (n4,n5) (n6,n9) (n7,n8) (n10,n11) (n12,n19) (n13,n16)
// (n14,n17) (n15,n18).
__host__ __device__ constexpr int lrf_slot(int k) {
    constexpr int t[kLrfMom20] = {1, 2, 3, 0, 4, 5, 6, 9, 7, 8, 10, 11, 12, 19, 13, 16, 14, 17, 15, 18};
    return t[k];
}
__device__ __forceinline__ void lrf_terms20x2(float4 xi, float2 oxy, float2 ozq, float2* n) {
    const float2 dxy = __fadd2_rn(make_float2(xi.x, xi.y), oxy);   // (dx, dy)
    const float2 dzq = __fadd2_rn(make_float2(xi.z, xi.w), ozq);   // (dz, q)
    const float dx = dxy.x, dy = dxy.y, dz = dzq.x, q = dzq.y;
    const float r2 = dx * dx + dy * dy + dz * dz;
    const float ri = rsqrtf(r2), ri2 = ri * ri;
    const float qri = q * ri;
    const float f0 = qri * ri2;
    const float f1 = 3.f * f0 * ri2;
    const float g = -5.f * f1 * ri2;
    n[0] = __ffma2_rn(dxy, make_float2(-f0, -f0), n[0]);                 // n1 -= dx f0, n2 -= dy f0
    n[1] = __ffma2_rn(dzq, make_float2(-f0, ri), n[1]);                  // n3 -= dz f0, n0 += q ri
    const float2 axy = __fmul2_rn(dxy, make_float2(f1, f1));             // (ax, ay)
    const float az = dz * f1;
    n[2] = __ffma2_rn(make_float2(axy.x, axy.x), dxy, n[2]);            // n4 += ax dx, n5 += ax dy
    n[3] = __ffma2_rn(make_float2(axy.x, az), make_float2(dz, dz), n[3]);  // n6 += ax dz, n9 += az dz
    n[4] = __ffma2_rn(make_float2(axy.y, axy.y), make_float2(dy, dz), n[4]);   // n7 += ay dy, n8 += ay dz
    const float2 gxy = __fmul2_rn(dxy, make_float2(g, g));               // (gx, gy)
    const float gz = g * dz;
    const float2 gxxyy = __fmul2_rn(gxy, dxy);                           // (gxx, gyy)
    const float gzz = gz * dz, gxy_ = gxy.x * dy;
    n[5] = __ffma2_rn(make_float2(gxxyy.x, gxxyy.x), dxy, n[5]);         // n10 += gxx dx, n11 += gxx dy
    n[6] = __ffma2_rn(make_float2(gxxyy.x, gzz), make_float2(dz, dz), n[6]);   // n12 += gxx dz, n19 += gzz dz
    n[7] = __ffma2_rn(make_float2(gxxyy.y, gxxyy.y), dxy, n[7]);         // n13 += gyy dx, n16 += gyy dy
    n[8] = __ffma2_rn(make_float2(gxy_, gxxyy.y), make_float2(dz, dz), n[8]);  // n14 += gxy dz, n17 += gyy dz
    n[9] = __ffma2_rn(make_float2(gzz, gzz), dxy, n[9]);                 // n15 += gzz dx, n18 += gzz dy
}
template <bool BOX>
__global__ void __launch_bounds__(kLrfNB, 10) k_lrf_nbody(DevModel m, const DevState* __restrict__ states, Cut c,
                                                          int nsplit) {
    const Band bpp = band(c.rcpp2, c.fpp), bpw = band(c.rcpw2, c.fpw), bww = band(c.rcww2, c.fww),
               blrf = band(c.rlrf2, c.flrf);
    __shared__ int s_meta[kLrfGT];
    __shared__ int s_off[kLrfGT + 1];
    __shared__ float4 s_xs[kLrfGT];
    __shared__ float4 s_xi[kLrfGT * kMaxGroup];
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const float4* __restrict__ xq = s.xq;
    double* __restrict__ lrf = s.lrf;
    const int g2 = blockIdx.x * kLrfNB + threadIdx.x;
    int s2 = -1;
    bool act = g2 < m.ncgp;
    if (act) {
        s2 = group_dist_atom(m, g2);
        act = !m.excl[s2];
    }
    const bool sol2 = g2 < m.ncgp_solute;
    const Band rc_s = sol2 ? bpp : bpw, rc_w = sol2 ? bpw : bww;
    float ccx = 0.f, ccy = 0.f, ccz = 0.f;
    float4 x2 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (act) {
        const double* L = lrf + (size_t)g2 * kLrfLen;
        ccx = (float)(L[0] - m.xpcent[0]);
        ccy = (float)(L[1] - m.xpcent[1]);
        ccz = (float)(L[2] - m.xpcent[2]);
        x2 = xq[s2];
    }
    constexpr int NS = kLrfMom20 / 2;   // packed slots (lrf_slot)
    float2 part[NS], hi[NS], lo[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) part[k] = hi[k] = lo[k] = make_float2(0.f, 0.f);
    const float2 oxy0 = make_float2(-ccx, -ccy), ozq0 = make_float2(-ccz, 0.f);
    // this block's range of source groups (blockIdx.z of nsplit)
    const int gbeg = (int)((int64_t)m.nlrf_groups * blockIdx.z / nsplit);
    const int gend = (int)((int64_t)m.nlrf_groups * (blockIdx.z + 1) / nsplit);
    for (int t0 = gbeg; t0 < gend; t0 += kLrfGT) {   // block-uniform
        const int ng = min(kLrfGT, gend - t0);
        const int a_base = m.lrf_goff[t0];
        const int na = m.lrf_goff[t0 + ng] - a_base;   // <= kLrfGT * kMaxGroup
        __syncthreads();   // the previous tile is consumed
        for (int k = threadIdx.x; k < ng; k += kLrfNB) {
            int meta = m.lrf_gmeta[t0 + k];
            s_meta[k] = meta;
            s_xs[k] = xq[meta & 0x3fffffff];
            s_off[k] = m.lrf_goff[t0 + k] - a_base;
        }
        if (threadIdx.x == 0) s_off[ng] = na;
        for (int k = threadIdx.x; k < na; k += kLrfNB) s_xi[k] = xq[m.lrf_gatom[a_base + k]];
        __syncthreads();
        if (!act) continue;
        for (int gi = 0; gi < ng; ++gi) {
            const int meta = s_meta[gi], s1 = meta & 0x3fffffff;
            const Band& rc2 = (meta >> 30) ? rc_s : rc_w;
            if (BOX) {
                if (s1 != s2 && lrf_pair_box(m, x2, s_xs[gi], rc2, blrf, x, s2, s1)) {
                    const float3 sh = lrf_shift(m, s_xs[gi], ccx, ccy, ccz, x, s1, lrf + (size_t)g2 * kLrfLen);
                    const float2 oxy = make_float2(-(ccx + sh.x), -(ccy + sh.y)), ozq = make_float2(-(ccz + sh.z), 0.f);
                    const int k1 = s_off[gi + 1];
                    for (int k = s_off[gi]; k < k1; ++k) lrf_terms20x2(s_xi[k], oxy, ozq, part);
                }
            } else if (s1 != s2 && lrf_pair(r2_f(x2, s_xs[gi]), rc2, blrf, x, s2, s1)) {
                const int k1 = s_off[gi + 1];
                for (int k = s_off[gi]; k < k1; ++k) lrf_terms20x2(s_xi[k], oxy0, ozq0, part);
            }
            if ((gi + 1) % kLrfFold == 0 || gi == ng - 1) {
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    two_sum_fold(hi[k].x, lo[k].x, part[k].x);
                    two_sum_fold(hi[k].y, lo[k].y, part[k].y);
                }
            }
        }
    }
    if (!act) return;
    double tot[kLrfMom20];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
        tot[lrf_slot(2 * k)] = (double)hi[k].x + (double)lo[k].x;
        tot[lrf_slot(2 * k + 1)] = (double)hi[k].y + (double)lo[k].y;
    }
    double* out = s.lrf_part + ((size_t)blockIdx.z * m.ncgp + g2) * kLrfMom20;
#pragma unroll
    for (int k = 0; k < kLrfMom20; ++k) out[k] = tot[k];
}

// The source ranges' moments of each target summed in range order, then
// expanded into the record.
__global__ void k_lrf_combine(DevModel m, const DevState* __restrict__ states, int nsplit) {
    const DevState& s = states[blockIdx.y];
    const int g2 = blockIdx.x * blockDim.x + threadIdx.x;
    if (g2 >= m.ncgp || m.excl[group_dist_atom(m, g2)]) return;
    double tot[kLrfMom20];
#pragma unroll
    for (int k = 0; k < kLrfMom20; ++k) tot[k] = 0.0;
    for (int z = 0; z < nsplit; ++z) {
        const double* p = s.lrf_part + ((size_t)z * m.ncgp + g2) * kLrfMom20;
#pragma unroll
        for (int k = 0; k < kLrfMom20; ++k) tot[k] += p[k];
    }
    double m24[kLrfMom];
    lrf_moments24(tot, m24);
    lrf_expand(m24, s.lrf + (size_t)g2 * kLrfLen + 3);
}

// Unstaged variant: one warp per target group reads the source atoms straight
// from global memory (lanes stride over the atoms, so loads are coalesced).
template <bool MIX, bool BOX>
__global__ void __launch_bounds__(128) k_lrf_accumulate_direct(DevModel m, const DevState* __restrict__ states, Cut c,
                                                         const int* __restrict__ lrf_src) {
    const Band bpp = band(c.rcpp2, c.fpp), bpw = band(c.rcpw2, c.fpw), bww = band(c.rcww2, c.fww),
               blrf = band(c.rlrf2, c.flrf);
    typedef typename std::conditional<MIX, float, double>::type T;
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const float4* __restrict__ xq = s.xq;
    double* __restrict__ lrf = s.lrf;
    int lane = threadIdx.x & 31;
    for (int g2 = warp_id_global(); g2 < m.ncgp; g2 += warps_total()) {
        int s2 = group_dist_atom(m, g2);
        if (m.excl[s2]) continue;
        bool sol2 = g2 < m.ncgp_solute;
        double* L = lrf + (size_t)g2 * kLrfLen;
        double cx = L[0], cy = L[1], cz = L[2];
        float4 x2 = xq[s2];
        float cxf = (float)(cx - m.xpcent[0]), cyf = (float)(cy - m.xpcent[1]), czf = (float)(cz - m.xpcent[2]);
        const Band rc_s = sol2 ? bpp : bpw, rc_w = sol2 ? bpw : bww;
        T mom[kLrfMom];
#pragma unroll
        for (int k = 0; k < kLrfMom; ++k) mom[k] = T(0);
        for (int i = lane; i < m.natom; i += kWarp) {
            int src = lrf_src[i];   // distance atom of i's group | solute flag << 30, -1 if never a source
            if (src < 0) continue;
            int s1 = src & 0x3fffffff;
            if (s1 == s2) continue;   // same group
            const Band& rc2 = (src >> 30) ? rc_s : rc_w;
            if constexpr (BOX) {   // FP64 minimum image and lattice shift (the FP64 form)
                static_assert(!MIX, "the mixed form's box LRF is k_lrf_nbody<true>");
                if (!lrf_pair_box_exact(m, x, s2, s1, rc2.c, blrf.c)) continue;
                double sx = m.boxl[0] * round((x[3 * s1] - cx) * m.inv_boxl[0]);
                double sy = m.boxl[1] * round((x[3 * s1 + 1] - cy) * m.inv_boxl[1]);
                double sz = m.boxl[2] * round((x[3 * s1 + 2] - cz) * m.inv_boxl[2]);
                lrf_terms<double>(x[3 * i] - cx - sx, x[3 * i + 1] - cy - sy, x[3 * i + 2] - cz - sz, m.crg[i], mom);
                continue;
            }
            if (!lrf_pair(r2_f(x2, xq[s1]), rc2, blrf, x, s2, s1)) continue;
            if constexpr (MIX) {
                float4 xi = xq[i];
                lrf_terms<float>(xi.x - cxf, xi.y - cyf, xi.z - czf, xi.w, mom);
            } else {
                lrf_terms<double>(x[3 * i] - cx, x[3 * i + 1] - cy, x[3 * i + 2] - cz, m.crg[i], mom);
            }
        }
        double tot[kLrfMom];
#pragma unroll
        for (int k = 0; k < kLrfMom; ++k) {
            T v = mom[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
            tot[k] = (double)v;
        }
        if (lane == 0) lrf_expand(tot, L + 3);
    }
}

// Any-atom mode (nbpplis2_lrf / nbpwlis2_lrf, src/nonbondene.f90:1369-1516,
// 2493-2618): a pair of groups that involves a solute group is "LRF" when no
// atom pair is inside the cut-off and the r2 of the last atom pair examined,
// (last atom of one group, last atom of the other; a water's first atom), is
// within RcLRF.  Water pairs keep the O-O test.  One warp per target group g2;
// lanes stride over the source groups, so each group pair is classified once.
__device__ __forceinline__ int group_last_atom(const DevModel& m, int g) {
    return g < m.ncgp_solute ? m.gatom[m.gslot[g + 1] - 1] : m.nat_solute + m.sa * (g - m.ncgp_solute);
}
template <bool MIX>
__global__ void __launch_bounds__(128) k_lrf_accumulate_any(DevModel m, const DevState* __restrict__ states, Cut c) {
    const Band bpp = band(c.rcpp2, c.fpp), bpw = band(c.rcpw2, c.fpw), bww = band(c.rcww2, c.fww),
               blrf = band(c.rlrf2, c.flrf);
    typedef typename std::conditional<MIX, float, double>::type T;
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const float4* __restrict__ xq = s.xq;
    double* __restrict__ lrf = s.lrf;
    int lane = threadIdx.x & 31;
    for (int g2 = warp_id_global(); g2 < m.ncgp; g2 += warps_total()) {
        int s2 = group_dist_atom(m, g2);
        if (m.excl[s2]) continue;
        bool sol2 = g2 < m.ncgp_solute;
        int l2 = group_last_atom(m, g2);
        double* L = lrf + (size_t)g2 * kLrfLen;
        double cx = L[0], cy = L[1], cz = L[2];
        float cxf = (float)(cx - m.xpcent[0]), cyf = (float)(cy - m.xpcent[1]), czf = (float)(cz - m.xpcent[2]);
        T mom[kLrfMom];
#pragma unroll
        for (int k = 0; k < kLrfMom; ++k) mom[k] = T(0);
        for (int g1 = lane; g1 < m.ncgp; g1 += kWarp) {
            if (g1 == g2) continue;
            int s1 = group_dist_atom(m, g1);
            if (m.excl[s1]) continue;
            bool sol1 = g1 < m.ncgp_solute;
            bool far;
            if (sol1 && sol2) {
                far = !gg_inside_any(m, x, xq, g1, g2, bpp);
            } else if (sol1 || sol2) {
                far = !gw_inside_any(m, x, xq, sol1 ? g1 : g2, sol1 ? s2 : s1, bpw);
            } else {
                far = lrf_pair(r2_f(xq[s2], xq[s1]), bww, blrf, x, s2, s1);
            }
            if (far && (sol1 || sol2)) {
                int l1 = group_last_atom(m, g1);
                far = within(r2_f(xq[l1], xq[l2]), blrf, x, l1, l2);
            }
            if (!far) continue;
            for (int a = m.gslot[g1]; a < m.gslot[g1 + 1]; ++a) {
                int i = m.gatom[a];
                if (m.iqatom[i] >= 0) continue;
                if constexpr (MIX) {
                    float4 xi = xq[i];
                    lrf_terms<float>(xi.x - cxf, xi.y - cyf, xi.z - czf, xi.w, mom);
                } else {
                    lrf_terms<double>(x[3 * i] - cx, x[3 * i + 1] - cy, x[3 * i + 2] - cz, m.crg[i], mom);
                }
            }
        }
        double tot[kLrfMom];
#pragma unroll
        for (int k = 0; k < kLrfMom; ++k) {
            T v = mom[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
            tot[k] = (double)v;
        }
        if (lane == 0) lrf_expand(tot, L + 3);
    }
}

// Periodic box with the switch-atom flag off (nbpplis2_box_lrf /
// nbpwlis2_box_lrf, src/nonbondene.f90:1220-1367, 2359-2491; water pairs
// nbwwlist_box_lrf 4397-4515): a unit pair with a solute group is "LRF" when
// none of its minimum-image atom pairs (a water by its first atom; Q and
// excluded atoms included) lies within the pair's cut-off and one lies within
// RcLRF; water pairs take the first-atom test.  lrf_update (628-725) shifts
// the source by boxlength * nint((x_switch(source) - centre(target)) /
// boxlength).  FP64 geometry and terms in both forms (this topology option
// is off the benchmark path).  One warp per target group, lanes over the
// source groups; the moments are summed in a fixed lane order.
__device__ __forceinline__ void unit_pair_min_box(const DevModel& m, const double* __restrict__ x, int g1, int g2,
                                                  double rc2, double rl2, bool& inside, bool& lrf) {
    // a water is tested by its molecule's first atom
    const bool w1 = g1 >= m.ncgp_solute, w2 = g2 >= m.ncgp_solute;
    const int a0 = w1 ? 0 : m.gslot[g1], a1 = w1 ? 1 : m.gslot[g1 + 1];
    const int b0 = w2 ? 0 : m.gslot[g2], b1 = w2 ? 1 : m.gslot[g2 + 1];
    inside = lrf = false;
    for (int a = a0; a < a1 && !inside; ++a) {
        const int i = w1 ? group_dist_atom(m, g1) : m.gatom[a];
        for (int b = b0; b < b1 && !inside; ++b) {
            const double r2 = box_d2(m, x, i, w2 ? group_dist_atom(m, g2) : m.gatom[b]);
            if (r2 <= rc2) inside = true;
            else if (r2 <= rl2) lrf = true;
        }
    }
}
__global__ void __launch_bounds__(128) k_lrf_accumulate_any_box(DevModel m, const DevState* __restrict__ states,
                                                               Cut c) {
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    double* __restrict__ lrf = s.lrf;
    const int lane = threadIdx.x & 31;
    for (int g2 = warp_id_global(); g2 < m.ncgp; g2 += warps_total()) {
        const bool sol2 = g2 < m.ncgp_solute;
        double* L = lrf + (size_t)g2 * kLrfLen;
        const double cx = L[0], cy = L[1], cz = L[2];
        double mom[kLrfMom];
#pragma unroll
        for (int k = 0; k < kLrfMom; ++k) mom[k] = 0.0;
        for (int g1 = lane; g1 < m.ncgp; g1 += kWarp) {
            if (g1 == g2) continue;
            const bool sol1 = g1 < m.ncgp_solute;
            const double rc2 = sol1 && sol2 ? c.rcpp2 : (sol1 || sol2 ? c.rcpw2 : c.rcww2);
            bool inside, far;
            unit_pair_min_box(m, x, g1, g2, rc2, c.rlrf2, inside, far);
            if (inside || !far) continue;
            const int s1 = group_dist_atom(m, g1);
            const double sx = m.boxl[0] * round((x[3 * s1] - cx) * m.inv_boxl[0]);
            const double sy = m.boxl[1] * round((x[3 * s1 + 1] - cy) * m.inv_boxl[1]);
            const double sz = m.boxl[2] * round((x[3 * s1 + 2] - cz) * m.inv_boxl[2]);
            for (int a = m.gslot[g1]; a < m.gslot[g1 + 1]; ++a) {
                const int i = m.gatom[a];
                if (m.iqatom[i] >= 0) continue;
                lrf_terms<double>(x[3 * i] - cx - sx, x[3 * i + 1] - cy - sy, x[3 * i + 2] - cz - sz, m.crg[i], mom);
            }
        }
        double tot[kLrfMom];
#pragma unroll
        for (int k = 0; k < kLrfMom; ++k) {
            double v = mom[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(kFull, v, o);
            tot[k] = v;
        }
        if (lane == 0) lrf_expand(tot, L + 3);
    }
}

// =============================================================================
// Force / energy kernels
// =============================================================================


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
__global__ void __launch_bounds__(256) k_ww(DevModel m, const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.y];
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
__global__ void __launch_bounds__(256) k_pw(DevModel m, const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.y];
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
__global__ void __launch_bounds__(256) k_pp(DevModel m, const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.y];
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
            if (code == 3) el *= m.el14f;
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

// nbe_qx soft-core pair for one state, src/nonbonded.f90:200-222
__device__ __forceinline__ void nbe_qx_d(double r2, double r, double r6_hc, double A, double B, double el,
                                         double sc, double lam, double& vel, double& vdw, double& dv) {
    double r6 = 1.0 / (r6_hc + sc);
    double r12 = r6 * r6;
    vel = el * r;
    double va = A * r12, vb = B * r6;
    vdw = va - vb;
    dv = r2 * (-vel - (12.0 * va - 6.0 * vb) * r6 * r6_hc) * lam;
}
__device__ __forceinline__ void nbe_qx_f(float r2, float r, float r6_hc, float A, float B, float el, float sc,
                                         float lam, float& vel, float& vdw, float& dv) {
    float r6 = __fdividef(1.0f, r6_hc + sc);
    float r12 = r6 * r6;
    vel = el * r;
    float va = A * r12, vb = B * r6;
    vdw = va - vb;
    dv = r2 * (-vel - (12.0f * va - 6.0f * vb) * r6 * r6_hc) * lam;
}

constexpr int kMaxQ = 64;
constexpr int kQBlock = 256;   // threads per block of the Q kernels

// Q-atom gradients: every lane keeps its Q atoms' sums in registers; at the
// end the warps of a block combine them in shared memory and the block adds
// them once (fixed point in the mixed form).
template <bool MIX>
__device__ __forceinline__ void flush_q_grad(const DevModel& m, const DevState& s,
                                             const unsigned long long (&gqx)[2][3], const double (&gqd)[2][3]) {
    typedef typename std::conditional<MIX, unsigned long long, double>::type GT;
    __shared__ GT red[3 * kMaxQ];
    for (int k = threadIdx.x; k < 3 * m.nqat; k += blockDim.x) red[k] = GT(0);
    __syncthreads();
    int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < kMaxQ / 32; ++k) {
        int iq = k * 32 + lane;
        if (iq >= m.nqat) break;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            if constexpr (MIX) atomicAdd(&red[3 * iq + c], gqx[k][c]);
            else atomicAdd(&red[3 * iq + c], gqd[k][c]);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * m.nqat; k += blockDim.x) {
        int i = m.iqseq[k / 3];
        if constexpr (MIX) atomicAdd(s.fix + 3 * i + k % 3, (unsigned long long)red[k]);
        else atomicAdd(s.d + 3 * i + k % 3, (double)red[k]);
    }
}

// Per-lane Q-atom x environment-atom interaction for all states (soft-core
// LJ + Coulomb when lj, Coulomb only otherwise): returns the lambda-weighted
// dv sum over states and adds the per-state energies to pel/pvdw.
template <bool MIX, int SMAX>
struct QPairT;
template <int SMAX>
struct QPairT<false, SMAX> {
    __device__ __forceinline__ static double run(const QPar* P, const double* lam, int S, bool lj, double r2, double r,
                                                 double* pel, double* pvdw) {
        double dvs = 0.0;
        if (lj) {
            double r6hc = 1.0 / (r2 * r2 * r2);
#pragma unroll
            for (int st = 0; st < SMAX; ++st) {
                if (st >= S) break;
                QPar q = P[st];
                double vel, vdw, dv;
                nbe_qx_d(r2, r, r6hc, q.A, q.B, q.el, q.sc, lam[st], vel, vdw, dv);
                dvs += dv;
                pel[st] += vel;
                pvdw[st] += vdw;
            }
        } else {   // nbe_qspc, src/nonbonded.f90:226-243
#pragma unroll
            for (int st = 0; st < SMAX; ++st) {
                if (st >= S) break;
                double vel = P[st].el * r;
                dvs += -r2 * vel * lam[st];
                pel[st] += vel;
            }
        }
        return dvs;
    }
};
template <int SMAX>
struct QPairT<true, SMAX> {
    __device__ __forceinline__ static float run(const QParF* P, const float* lam, int S, bool lj, float r2, float r,
                                                float* pel, float* pvdw) {
        float dvs = 0.0f;
        if (lj) {
            float r6hc = __fdividef(1.0f, r2 * r2 * r2);
#pragma unroll
            for (int st = 0; st < SMAX; ++st) {
                if (st >= S) break;
                QParF q = P[st];
                float vel, vdw, dv;
                nbe_qx_f(r2, r, r6hc, q.A, q.B, q.el, q.sc, lam[st], vel, vdw, dv);
                dvs += dv;
                pel[st] += vel;
                pvdw[st] += vdw;
            }
        } else {
#pragma unroll
            for (int st = 0; st < SMAX; ++st) {
                if (st >= S) break;
                float vel = P[st].el * r;
                dvs += -r2 * vel * lam[st];
                pel[st] += vel;
            }
        }
        return dvs;
    }
};

// nonbond_qw_spc / nonbond_qw (src/nonbondene.f90:5658-5767, 5339-5418) and
// nonbond_qp (src/nonbondene.f90:5157-5230): one warp per listed environment
// unit (a water molecule, or one solute atom), lane = Q atom.  A warp takes
// fixed chunks of qchunk consecutive units (autotuned); the per-state energies of a
// chunk are summed in registers and converted once per chunk, so the fixed-
// point totals do not depend on the grid.  An environment atom's gradient is
// summed over the Q atoms in FP32 in a fixed shuffle order, then converted.

template <bool MIX, bool SPC, bool WATER, int SMAX>
__global__ void __launch_bounds__(kQBlock, 3) k_qenv(DevModel m, const DevState* __restrict__ states, int qchunk) {
    typedef typename std::conditional<MIX, float, double>::type T;
    const DevState& s = states[blockIdx.y];
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel[SMAX], evdw[SMAX];
    float gqf[2][3] = {};              // this chunk's Q-atom gradient (mixed form)
    unsigned long long gqx[2][3] = {}; // converted once per chunk: the sum over chunks is exact
    double gqd[2][3] = {};
    T lam[SMAX];
#pragma unroll
    for (int st = 0; st < SMAX; ++st) lam[st] = st < m.S ? (T)s.lambda[st] : T(0);
    int lane = threadIdx.x & 31;
    int n = WATER ? min((int64_t)s.cnt[C_QW], s.cap_qw) : min((int64_t)s.cnt[C_QP], s.cap_qp);
    int S = m.S;
    const int na = WATER ? m.sa : 1;
    const int nchunk = (n + qchunk - 1) / qchunk;
    for (int ch = warp_id_global(); ch < nchunk; ch += warps_total()) {
      T pel[SMAX], pvdw[SMAX];
#pragma unroll
      for (int st = 0; st < SMAX; ++st) pel[st] = pvdw[st] = T(0);
      const int pend = min(n, (ch + 1) * qchunk);
      for (int p = ch * qchunk; p < pend; ++p) {
        int j0 = WATER ? m.nat_solute + m.sa * s.qw[p] : s.qp[p];
        for (int a = 0; a < na; ++a) {
            int j = j0 + a;
            bool lj = !WATER || !SPC || a == 0;
            T gj[3] = {T(0), T(0), T(0)};
#pragma unroll
            for (int k = 0; k < kMaxQ / 32; ++k) {
                int iq = k * 32 + lane;
                if (iq >= m.nqat) break;
                int i = m.iqseq[iq];
                T tx, ty, tz, r2, r;
                if constexpr (MIX) {
                    float4 xi = s.xq[i], xj = s.xq[j];
                    tx = xj.x - xi.x;
                    ty = xj.y - xi.y;
                    tz = xj.z - xi.z;
                    r = rsqrtf(tx * tx + ty * ty + tz * tz);
                    r2 = r * r;
                } else {
                    tx = s.x[3 * j] - s.x[3 * i];
                    ty = s.x[3 * j + 1] - s.x[3 * i + 1];
                    tz = s.x[3 * j + 2] - s.x[3 * i + 2];
                    r2 = 1.0 / (tx * tx + ty * ty + tz * tz);
                    r = sqrt(r2);
                }
                T dvs;
                if constexpr (MIX) {
                    const QParF* P = WATER ? m.qw_tabf + (iq * m.sa + a) * S : m.qp_tabf + ((size_t)j * m.nqat + iq) * S;
                    dvs = QPairT<true, SMAX>::run(P, lam, S, lj, r2, r, pel, pvdw);
                    gqf[k][0] -= tx * dvs; gqf[k][1] -= ty * dvs; gqf[k][2] -= tz * dvs;
                } else {
                    const QPar* P = WATER ? m.qw_tab + (iq * m.sa + a) * S : m.qp_tab + ((size_t)j * m.nqat + iq) * S;
                    dvs = QPairT<false, SMAX>::run(P, lam, S, lj, r2, r, pel, pvdw);
                    gqd[k][0] -= tx * dvs; gqd[k][1] -= ty * dvs; gqd[k][2] -= tz * dvs;
                }
                gj[0] += tx * dvs;
                gj[1] += ty * dvs;
                gj[2] += tz * dvs;
            }
            // environment atom gradient: sum over the warp's Q atoms.  Each
            // atom is in one unit of the list, so the mixed form stores its
            // FP32 sum (k_apply_fixed adds it) instead of a converted atomic
            T v0 = warp_sum(gj[0]), v1 = warp_sum(gj[1]), v2 = warp_sum(gj[2]);
            if (lane == 0) {
                if constexpr (MIX) {
                    s.fq[3 * j] = v0;
                    s.fq[3 * j + 1] = v1;
                    s.fq[3 * j + 2] = v2;
                } else {
                    acc.grad(j, v0, v1, v2);
                }
            }
        }
      }
#pragma unroll
      for (int st = 0; st < SMAX; ++st) {
          if (st >= S) break;
          if constexpr (MIX) {
              eel[st].add_alu(pel[st]);
              evdw[st].add_alu(pvdw[st]);
          } else {
              eel[st].add(pel[st]);
              evdw[st].add(pvdw[st]);
          }
      }
      if constexpr (MIX) {
#pragma unroll
          for (int k = 0; k < kMaxQ / 32; ++k) {
              if (k * 32 >= m.nqat) break;   // warp-uniform
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                  gqx[k][c] += to_fix_alu(gqf[k][c]);
                  gqf[k][c] = 0.f;
              }
          }
      }
    }
    const int kel = WATER ? 4 : 2;
#pragma unroll
    for (int st = 0; st < SMAX; ++st) {
        if (st >= S) break;
        eel[st].flush(acc, eq_slot(st, kel));
        evdw[st].flush(acc, eq_slot(st, kel + 1));
    }
    flush_q_grad<MIX>(m, s, gqx, gqd);
}

// ---------------------------------------------------------------------------
// Adjoint of the Q-atom energies with respect to the Q parameters: for every
// Q atom iq and state s, dE_s/dqcrg(iq,s), dE_s/dqA(iq,s) and dE_s/dqB(iq,s),
// where qA/qB are the Q atom's code-1 LJ factors (A_pair = qA * a_j,
// B_pair = qB * b_j, geometric rule).  The pair terms are recomputed from the
// lists: E_s = sum el/r + A/(r^6+alpha)^2 - B/(r^6+alpha) (nbe_qx,
// src/nonbonded.f90:200-222), so
//   dE/dqcrg += c_j / r,  dE/dqA += a_j / (r^6+alpha)^2,  dE/dqB -= b_j / (r^6+alpha).
// One warp per environment unit, lane = Q atom, sums in FP64 registers.
// ---------------------------------------------------------------------------
// Mixed form, transposed: lane = environment unit (a listed solute atom or
// water), each warp taking a fixed chunk of 32 consecutive units, and a loop
// over the Q atoms with their coordinates in shared memory.  An environment
// atom's gradient stays in its lane (stored once, no reduction); a Q atom's
// gradient is a fixed-order warp sum per Q atom and chunk, added to the
// block's fixed-point total; each unit's per-state energies are converted
// once.  The sums do not depend on the grid.  qw's parameters are the same
// for all lanes (broadcast); qp's come from the [Q atom][solute atom] table,
// so lanes holding consecutive solute atoms read consecutive entries.
// periodic box, mixed form's FP32 pair geometry: packed coordinates
// (xpcent-centred) and an FP32 lattice shift of a against b (boxlength *
// nint((a - b) / boxlength)); a pair vector is shift - (x_i - x_j)
__device__ __forceinline__ float3 box_shift_f(const DevModel& m, float4 a, float4 b) {
    return make_float3((float)m.boxl[0] * roundf((a.x - b.x) * (float)m.inv_boxl[0]),
                       (float)m.boxl[1] * roundf((a.y - b.y) * (float)m.inv_boxl[1]),
                       (float)m.boxl[2] * roundf((a.z - b.z) * (float)m.inv_boxl[2]));
}

// Sums each of N (16 or 32) values over the 32 lanes of a warp at once: a
// butterfly whose step with lane bit o halves the vector, every lane keeping
// the half its bit o selects and adding the partner's copy of it, until one
// value is left; the remaining lane bits are summed as in warp_sum.  With
// N = 32 lane v ends with the sum of value v, with N = 16 lanes 2v and 2v + 1
// do.  Each sum pairs the lanes as warp_sum does (lane i with i + 16, then
// with i + 8, ...), so it is the same FP32 value warp_sum gives, for N - 1
// shuffles and additions instead of 5 N.
template <int N>
__device__ __forceinline__ float reduce_scatter(float (&g)[N], int lane) {
    static_assert(N == 16 || N == 32, "16 or 32 values");
    int o = 16;
#pragma unroll
    for (int len = N; len > 1; o >>= 1, len >>= 1) {
        const bool up = lane & o;
#pragma unroll
        for (int i = 0; i < len / 2; ++i) {
            const float keep = up ? g[i + len / 2] : g[i];
            const float send = up ? g[i] : g[i + len / 2];
            g[i] = keep + __shfl_xor_sync(kFull, send, o);
        }
    }
    float v = g[0];
#pragma unroll
    for (; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}
constexpr int kQRed = 5;   // Q atoms per transposed reduction (15 of its 16 values)

//
// BOX (nonbond_qp_box, src/nonbondene.f90:5234-5335; nonbond_qw_box /
// nonbond_qw_spc_box, 5422-5505, 5771-5881): each unit is taken at the image
// next to qswitch, shifted by the lattice vector of qswitch against the
// water's first atom (qw) or against the first atom of the solute atom's
// group within Rcq of qswitch (qp, nbqp_cgp; iwhich, rq2); the pair vector
// is shift - (x_q - x_j).
template <bool SPC, bool WATER, int SMAX, bool BOX = false>
__global__ void __launch_bounds__(kQBlock) k_qenv_lanes(DevModel m, const DevState* __restrict__ states,
                                                        const int* __restrict__ iwhich = nullptr, float rq2 = 0.f) {
    const DevState& s = states[blockIdx.y];
    __shared__ unsigned long long red[3 * kMaxQ];
    __shared__ float4 sq[kMaxQ];
    for (int k = threadIdx.x; k < 3 * m.nqat; k += blockDim.x) red[k] = 0ull;
    for (int k = threadIdx.x; k < m.nqat; k += blockDim.x) sq[k] = s.xq[m.iqseq[k]];
    __syncthreads();
    Acc<true> acc = make_acc<true>(s);
    ESum<true> eel[SMAX], evdw[SMAX];
    float lam[SMAX];
#pragma unroll
    for (int st = 0; st < SMAX; ++st) lam[st] = st < m.S ? (float)s.lambda[st] : 0.f;
    const int lane = threadIdx.x & 31, S = m.S, nq = m.nqat;
    const int n = WATER ? min((int64_t)s.cnt[C_QW], s.cap_qw) : min((int64_t)s.cnt[C_QP], s.cap_qp);
    constexpr int NA = WATER ? kMaxSolv : 1;
    const int na = WATER ? m.sa : 1;
    for (int c0 = warp_id_global() * kWarp; c0 < n; c0 += warps_total() * kWarp) {
        const int p = c0 + lane;
        const bool act = p < n;
        const int j0 = act ? (WATER ? m.nat_solute + m.sa * s.qw[p] : s.qp[p]) : 0;
        float4 xj[NA];
        float gj[NA][3];
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            gj[a][0] = gj[a][1] = gj[a][2] = 0.f;
            xj[a] = (act && a < na) ? s.xq[j0 + a] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        float3 sh = make_float3(0.f, 0.f, 0.f);   // the unit's lattice shift (BOX)
        if (BOX && act) {
            const float4 xs = s.xq[m.qswitch];
            if (WATER) {
                sh = box_shift_f(m, xs, xj[0]);
            } else {
                const int grp = iwhich[j0];
                int ref = m.gatom[m.gslot[grp]];
                for (int b = m.gslot[grp]; b < m.gslot[grp + 1]; ++b) {
                    const float4 xb = s.xq[m.gatom[b]];
                    const float3 t3 = box_shift_f(m, xb, xs);
                    const float dx = t3.x - (xb.x - xs.x), dy = t3.y - (xb.y - xs.y), dz = t3.z - (xb.z - xs.z);
                    if (dx * dx + dy * dy + dz * dz <= rq2) {
                        ref = m.gatom[b];
                        break;
                    }
                }
                sh = box_shift_f(m, xs, s.xq[ref]);
            }
        }
        float pel[SMAX], pvdw[SMAX];
#pragma unroll
        for (int st = 0; st < SMAX; ++st) pel[st] = pvdw[st] = 0.f;
        // Q atoms in blocks of kQRed: their 3 kQRed gradient components are
        // summed over the warp in one transposed butterfly (reduce_scatter)
        for (int q0 = 0; q0 < nq; q0 += kQRed) {
            float g[16];
#pragma unroll
            for (int v = 0; v < 16; ++v) g[v] = 0.f;
#pragma unroll
            for (int b = 0; b < kQRed; ++b) {
                const int iq = q0 + b;
                if (iq >= nq) break;   // warp-uniform
                const float4 xi = sq[iq];
                float gx = 0.f, gy = 0.f, gz = 0.f;
                if (act) {
#pragma unroll
                    for (int a = 0; a < NA; ++a) {
                        if (a >= na) break;
                        const bool lj = !WATER || !SPC || a == 0;
                        float tx, ty, tz;
                        if (BOX) {
                            tx = sh.x - (xi.x - xj[a].x), ty = sh.y - (xi.y - xj[a].y), tz = sh.z - (xi.z - xj[a].z);
                        } else {
                            tx = xj[a].x - xi.x, ty = xj[a].y - xi.y, tz = xj[a].z - xi.z;
                        }
                        float r = rsqrtf(tx * tx + ty * ty + tz * tz), r2 = r * r;
                        const QParF* P = WATER ? m.qw_tabf + (iq * m.sa + a) * S
                                               : m.qp_tabft + ((size_t)iq * m.nat_solute + j0) * S;
                        float dvs = QPairT<true, SMAX>::run(P, lam, S, lj, r2, r, pel, pvdw);
                        gx -= tx * dvs; gy -= ty * dvs; gz -= tz * dvs;
                        gj[a][0] += tx * dvs; gj[a][1] += ty * dvs; gj[a][2] += tz * dvs;
                    }
                }
                g[3 * b] = gx;
                g[3 * b + 1] = gy;
                g[3 * b + 2] = gz;
            }
            const float v = reduce_scatter<16>(g, lane);
            const int idx = lane >> 1;   // the component this lane pair holds
            if (!(lane & 1) && idx < 3 * kQRed && 3 * q0 + idx < 3 * nq) atomicAdd(&red[3 * q0 + idx], to_fix_alu(v));
        }
        if (act) {
#pragma unroll
            for (int a = 0; a < NA; ++a) {
                if (a >= na) break;
                s.fq[3 * (j0 + a)] = gj[a][0];
                s.fq[3 * (j0 + a) + 1] = gj[a][1];
                s.fq[3 * (j0 + a) + 2] = gj[a][2];
            }
#pragma unroll
            for (int st = 0; st < SMAX; ++st) {
                if (st >= S) break;
                eel[st].add_alu(pel[st]);
                evdw[st].add_alu(pvdw[st]);
            }
        }
    }
    const int kel = WATER ? 4 : 2;
#pragma unroll
    for (int st = 0; st < SMAX; ++st) {
        if (st >= S) break;
        eel[st].flush(acc, eq_slot(st, kel));
        evdw[st].flush(acc, eq_slot(st, kel + 1));
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * nq; k += blockDim.x) {
        unsigned long long v = red[k];
        if (v) atomicAdd(s.fix + 3 * m.iqseq[k / 3] + k % 3, v);
    }
}

// Adjoint of the Q-environment terms in FP64 in both precision forms: the
// adjoint is an occasional call for parameter fitting, and FP64 geometry keeps
// its gradients to the FP64 reference's rounding.
template <bool SPC, bool WATER, int SMAX>
__global__ void __launch_bounds__(kQBlock) k_qadj_env(DevModel m, const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.y];
    double aq[2][SMAX] = {}, aa[2][SMAX] = {}, ab[2][SMAX] = {};
    int lane = threadIdx.x & 31;
    int n = WATER ? min((int64_t)s.cnt[C_QW], s.cap_qw) : min((int64_t)s.cnt[C_QP], s.cap_qp);
    const int S = m.S, na = WATER ? m.sa : 1;
    for (int p = warp_id_global(); p < n; p += warps_total()) {
        int j0 = WATER ? m.nat_solute + m.sa * s.qw[p] : s.qp[p];
        for (int a = 0; a < na; ++a) {
            int j = j0 + a;
            bool lj = !WATER || !SPC || a == 0;
#pragma unroll
            for (int k = 0; k < kMaxQ / 32; ++k) {
                int iq = k * 32 + lane;
                if (iq >= m.nqat) break;
                int i = m.iqseq[iq];
                double tx = s.x[3 * j] - s.x[3 * i], ty = s.x[3 * j + 1] - s.x[3 * i + 1],
                       tz = s.x[3 * j + 2] - s.x[3 * i + 2];
                double d2 = tx * tx + ty * ty + tz * tz;
                double r = 1.0 / sqrt(d2), r6 = d2 * d2 * d2;
                size_t t0 = WATER ? (size_t)(iq * m.sa + a) * S : ((size_t)j * m.nqat + iq) * S;
                const QAdjF* F = (WATER ? m.qw_adj : m.qp_adj) + t0;
                const QPar* P = (WATER ? m.qw_tab : m.qp_tab) + t0;
#pragma unroll
                for (int st = 0; st < SMAX; ++st) {
                    if (st >= S) break;
                    const QAdjF& f = F[st];
                    aq[k][st] += f.c * r;
                    if (lj) {
                        double u = 1.0 / (r6 + P[st].sc);
                        aa[k][st] += (f.a2 * u + f.a1) * u;
                        ab[k][st] += (f.b2 * u + f.b1) * u;
                    }
                }
            }
        }
    }
    // block sums in shared memory, one atomic per value and block
    __shared__ double red[3 * kMaxQ * kMaxStates];
    for (int k = threadIdx.x; k < 3 * m.nqat * S; k += blockDim.x) red[k] = 0.0;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kMaxQ / 32; ++k) {
        int iq = k * 32 + lane;
        if (iq >= m.nqat) break;
#pragma unroll
        for (int st = 0; st < SMAX; ++st) {
            if (st >= S) break;
            int o = iq + m.nqat * st;
            atomicAdd(&red[o], aq[k][st]);
            atomicAdd(&red[m.nqat * S + o], aa[k][st]);
            atomicAdd(&red[2 * m.nqat * S + o], ab[k][st]);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 3 * m.nqat * S; k += blockDim.x)
        if (red[k] != 0.0) atomicAdd(s.adj + k, red[k]);
}

// static Q-Q and Q-bonded pairs (nbqq / nbqqp lists)
__global__ void k_qadj_qq(DevModel m, const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.y];
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= s.nqq) return;
    QQEntry e = s.qq[p];
    QQAdj f = m.qq_adj[p];
    double tx = s.x[3 * e.j] - s.x[3 * e.i], ty = s.x[3 * e.j + 1] - s.x[3 * e.i + 1],
           tz = s.x[3 * e.j + 2] - s.x[3 * e.i + 2];
    double d2 = tx * tx + ty * ty + tz * tz;
    double r = 1.0 / sqrt(d2), r6 = d2 * d2 * d2;
    double u = 1.0 / (r6 + e.sc);
    int nqs = m.nqat * m.S;
    int oi = f.iq + m.nqat * f.s;
    atomicAdd(s.adj + oi, f.fi.c * r);
    if (!e.soft) {
        atomicAdd(s.adj + nqs + oi, (f.fi.a2 * u + f.fi.a1) * u);
        atomicAdd(s.adj + 2 * nqs + oi, (f.fi.b2 * u + f.fi.b1) * u);
    }
    if (f.jq >= 0) {
        int oj = f.jq + m.nqat * f.s;
        atomicAdd(s.adj + oj, f.fj.c * r);
        if (!e.soft) {
            atomicAdd(s.adj + nqs + oj, (f.fj.a2 * u + f.fj.a1) * u);
            atomicAdd(s.adj + 2 * nqs + oj, (f.fj.b2 * u + f.fj.b1) * u);
        }
    }
}

// nonbond_qq + nonbond_qqp (static lists), src/nonbondene.f90:5013-5153,
// pair kernel nbe_qq, src/nonbonded.f90:111-150.  The FP64 form computes in
// FP64; the mixed form in FP32 like the other pair kernels (the FP64 pipe runs
// at 1/64 of the FP32 rate), with the entries' parameters and lambda kept in
// FP32 copies.  Every pair touches a Q atom and one of a few energy slots, so the Q atoms'
// gradients and the energies are summed in shared memory per block (fixed
// point in the mixed form) and added once per block: global atomics on those
// few addresses serialise.
template <bool MIX>
__global__ void __launch_bounds__(256) k_qq(DevModel m, const DevState* __restrict__ states) {
    typedef typename std::conditional<MIX, unsigned long long, double>::type GT;
    __shared__ GT red[3 * kMaxQ];
    __shared__ GT rede[kNumE];
    const DevState& s = states[blockIdx.y];
    Acc<MIX> acc = make_acc<MIX>(s);
    for (int k = threadIdx.x; k < 3 * m.nqat; k += blockDim.x) red[k] = GT(0);
    for (int k = threadIdx.x; k < kNumE; k += blockDim.x) rede[k] = GT(0);
    __syncthreads();
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < s.nqq) {
    QQEntry e = s.qq[p];
    const int kel = p < s.nqq_qq ? 0 : 2;
    const int at[2] = {e.i, e.j};
    if constexpr (MIX) {   // FP32 pair arithmetic, fixed-point sums
        const float4 pf = s.qqf[p];   // A, B, el, sc
        float4 xi = s.xq[e.i], xj = s.xq[e.j];
        float tx = xj.x - xi.x, ty = xj.y - xi.y, tz = xj.z - xi.z;
        float d2 = tx * tx + ty * ty + tz * tz;
        float r = rsqrtf(d2), r2 = r * r;   // r = 1/distance as in nbe_qq
        float r6_hc = __fdividef(1.0f, r2 * r2 * r2);
        float r6 = __fdividef(1.0f, r6_hc + pf.w);
        float lam = s.lambdaf[e.s];
        float vel = pf.z * r, va, vb, dv;
        if (e.soft) {
            vb = 0.0f;
            float dist = d2 * r;
            va = pf.x * expf(-pf.y * dist);
            dv = r2 * (-vel - pf.y * va * dist) * lam;
        } else {
            va = pf.x * r6 * r6;
            vb = pf.y * r6;
            dv = r2 * (-vel - (12.0f * va - 6.0f * vb) * r6 * r6_hc) * lam;
        }
        const float g[2][3] = {{-tx * dv, -ty * dv, -tz * dv}, {tx * dv, ty * dv, tz * dv}};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            int iq = m.iqatom[at[h]];
            if (iq >= 0) {
#pragma unroll
                for (int c = 0; c < 3; ++c) atomicAdd(&red[3 * iq + c], to_fix_alu(g[h][c]));
            } else {
                acc.grad(at[h], g[h][0], g[h][1], g[h][2]);
            }
        }
        atomicAdd(&rede[eq_slot(e.s, kel)], to_fix_alu(vel));
        atomicAdd(&rede[eq_slot(e.s, kel + 1)], to_fix_alu(va - vb));
    } else {
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
        const double g[2][3] = {{-tx * dv, -ty * dv, -tz * dv}, {tx * dv, ty * dv, tz * dv}};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            int iq = m.iqatom[at[h]];
            if (iq >= 0) {
#pragma unroll
                for (int c = 0; c < 3; ++c) atomicAdd(&red[3 * iq + c], g[h][c]);
            } else {
                acc.grad(at[h], g[h][0], g[h][1], g[h][2]);
            }
        }
        atomicAdd(&rede[eq_slot(e.s, kel)], vel);
        atomicAdd(&rede[eq_slot(e.s, kel + 1)], va - vb);
    }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kNumE; k += blockDim.x) {
        GT v = rede[k];
        if (v != GT(0)) {
            if constexpr (MIX) acc.energy_fix(k, v);
            else acc.energy(k, v);
        }
    }
    for (int k = threadIdx.x; k < 3 * m.nqat; k += blockDim.x) {
        GT v = red[k];
        if (v != GT(0)) {
            int i = m.iqseq[k / 3];
            if constexpr (MIX) atomicAdd(s.fix + 3 * i + k % 3, v);
            else atomicAdd(s.d + 3 * i + k % 3, v);
        }
    }
}

// lrf_taylor, src/nonbondene.f90:507-571 (FP64 in both forms)
template <bool MIX>
__global__ void __launch_bounds__(256) k_lrf_taylor(DevModel m, const DevState* __restrict__ states, const int* __restrict__ iwhich) {
    const DevState& s = states[blockIdx.y];
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> elrf;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m.natom; i += gridDim.x * blockDim.x) {
        if (m.excl[i] || m.iqatom[i] >= 0 || iwhich[i] < 0) continue;   // (an atom in no group: no record)
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
// d += fixed-point gradient (cleared for the next evaluation), plus the rows'
// and the Q-environment FP32 gradients when those kernels ran in this
// evaluation: they rewrite every atom they own each time, and atoms they do
// not own stay 0 (fq is cleared when the Q lists are rebuilt)
__global__ void k_apply_fixed(int n, const DevState* __restrict__ states, int rows, int qenv) {
    unsigned long long* __restrict__ fix = states[blockIdx.y].fix;
    const float* __restrict__ frow = states[blockIdx.y].frow;
    const float* __restrict__ fq = states[blockIdx.y].fq;
    double* __restrict__ d = states[blockIdx.y].d;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        long long v = (long long)fix[k];
        // a row atom's gradient (its row's FP32 sum) is converted once to 64-bit
        // fixed point and joins the atom's other fixed-point contributions as
        // an integer (exact, order-free); the conversion is done here rather
        // than in the row kernels, whose main loops it slowed by 15-24 %
        if (rows) v += (long long)to_fix(frow[k]);
        double add = (double)v * (1.0 / kFix);
        if (qenv) add += (double)fq[k];
        if (add != 0.0) d[k] += add;
        if (v != 0) fix[k] = 0ull;
    }
}

// =============================================================================
// Spherical-boundary solvent terms (FP64 in both forms)
// =============================================================================

// restrain_solvent, src/nonbondene.f90:6466-6544
template <bool MIX>
__global__ void k_restrain_solvent(DevModel m, const DevState* __restrict__ states, SolventDev p, double shift,
                                   const int* __restrict__ wsw, const uint8_t* __restrict__ heavy_solv, int tdev) {
    const DevState& s = states[blockIdx.y];
    if (tdev)   // the window's Tfree from its last MD temperature(), as the host computes the shift
        shift = (p.fk_wsphere != 0.0) ? sqrt(p.boltz * *s.md_tfree / p.fk_wsphere) : 0.0;
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> er;
    const float r0f = (float)(p.rwat - shift);
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
            if constexpr (MIX) {   // FP32 arithmetic; the two branches meet with equal value and slope at db = 0
                float4 xa = s.xq[idist];
                float ux = xa.x + m.wcoff[0], uy = xa.y + m.wcoff[1], uz = xa.z + m.wcoff[2];
                float bf = sqrtf(ux * ux + uy * uy + uz * uz);
                float dbf = bf - r0f;
                float ef, dvf;
                if (dbf > 0.f) {
                    ef = 0.5f * p.fk_wspheref * (dbf * dbf) - p.Dwmzf;
                    dvf = p.fk_wspheref * dbf / bf;
                } else if (bf > 0.f) {
                    float fexp = expf(p.awmzf * dbf);
                    ef = p.Dwmzf * (fexp * fexp - 2.f * fexp);
                    dvf = -2.f * p.Dwmzf * p.awmzf * (fexp - fexp * fexp) / bf;
                } else {
                    ef = 0.f;
                    dvf = 0.f;
                }
                acc.grad_alu(i, ux * dvf, uy * dvf, uz * dvf);
                er.add_alu(ef);
                continue;
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

// SPC water vectors in FP32 from the packed (xpcent-centred) coordinates:
// dipole direction H1 + H2 - 2 O and radial vector O - xwcent, with lengths
__device__ __forceinline__ void water_vectors_f(const DevModel& m, const float4* __restrict__ xq, int w, float& rmx,
                                                float& rmy, float& rmz, float& rm, float& rcx, float& rcy,
                                                float& rcz, float& rc) {
    int i = m.nat_solute + 3 * w;
    float4 o = xq[i], h1 = xq[i + 1], h2 = xq[i + 2];
    float ux = h1.x + h2.x - 2.f * o.x, uy = h1.y + h2.y - 2.f * o.y, uz = h1.z + h2.z - 2.f * o.z;
    rcx = o.x + m.wcoff[0];
    rcy = o.y + m.wcoff[1];
    rcz = o.z + m.wcoff[2];
    rm = sqrtf(ux * ux + uy * uy + uz * uz);
    rmx = ux / rm; rmy = uy / rm; rmz = uz / rm;
    rc = sqrtf(rcx * rcx + rcy * rcy + rcz * rcz);
    rcx /= rc; rcy /= rc; rcz /= rc;
}

// Shell of a water from its radial distance rc: the outer shells beyond
// rout[N-1] - dr[N-1] (src/nonbondene.f90:6590-6606).  `rcd` is exact FP64.
__device__ __forceinline__ int watpol_shell(const SolventDev& p, double rcd) {
    int N = p.nshell;
    if (!(rcd > p.rout[N - 1] - p.dr[N - 1])) return -1;
    int is;
    for (is = N - 1; is >= 1; --is)
        if (rcd <= p.rout[is]) break;
    return is < 0 ? 0 : is;
}

// Mixed form (SPC): the selection order is decided in FP64, on the key
// 1 - cos(theta) from FP64 dot products (one square root and one division
// instead of the reference's six divisions and an arc cosine; it orders like
// theta), because swapping two waters' targets changes their forces by
// fkwpol * dtheta0.  The unit vectors for the forces are FP32 from the same
// FP64 differences, theta is an FP32 atan2 of the FP64 cross and dot products
// (below), and the shell of every
// water is decided exactly: the FP32 distance decides away from the shell
// radii, the FP64 distance within 2e-4 of one.
template <bool MIX>
__global__ void k_watpol_theta(DevModel m, const DevState* __restrict__ states, SolventDev p) {
    const DevState& s = states[blockIdx.y];
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= m.nwat) return;
    s.shell[w] = -1;
    s.theta[w] = 0.0;
    s.rkey[w] = 0.0;
    int i = m.nat_solute + m.sa * w;
    if (m.excl[i]) return;
    double* v = s.wvec + 8 * (size_t)w;   // reused by k_watpol_force in the same call
    double rcd;
    if (MIX && m.sa == 3) {
        const double* x = s.x;
        double ux = x[3 * (i + 1)] + x[3 * (i + 2)] - 2.0 * x[3 * i];
        double uy = x[3 * (i + 1) + 1] + x[3 * (i + 2) + 1] - 2.0 * x[3 * i + 1];
        double uz = x[3 * (i + 1) + 2] + x[3 * (i + 2) + 2] - 2.0 * x[3 * i + 2];
        double qx = x[3 * i] - m.xwcent[0], qy = x[3 * i + 1] - m.xwcent[1], qz = x[3 * i + 2] - m.xwcent[2];
        double uu = ux * ux + uy * uy + uz * uz, rr = qx * qx + qy * qy + qz * qz, ur = ux * qx + uy * qy + uz * qz;
        double scp64 = fmin(1.0, fmax(-1.0, ur / sqrt(uu * rr)));
        s.rkey[w] = 1.0 - scp64;
        float rm = sqrtf((float)uu), rc = sqrtf((float)rr);
        float rmx = (float)ux / rm, rmy = (float)uy / rm, rmz = (float)uz / rm;
        float rcx = (float)qx / rc, rcy = (float)qy / rc, rcz = (float)qz / rc;
        // theta from atan2(|u x q|, u.q) of FP64 products: well conditioned at 0
        // and pi, where the arc cosine of a rounded cosine is not (an FP32
        // cosine of 1 gives theta 0 for a water a few 1e-5 rad off the radius,
        // and the force's 1/sin(theta) then meets an O(theta) vector difference)
        double cx = uy * qz - uz * qy, cy = uz * qx - ux * qz, cz = ux * qy - uy * qx;
        s.theta[w] = (double)atan2f(sqrtf((float)(cx * cx + cy * cy + cz * cz)), (float)ur);
        v[0] = rmx; v[1] = rmy; v[2] = rmz; v[3] = rm;
        v[4] = rcx; v[5] = rcy; v[6] = rcz; v[7] = rc;
        bool near = false;
        for (int k = 0; k < p.nshell; ++k) {
            float t = (float)p.rout[k];
            near |= fabsf(rc - t) <= 2e-4f * t;
        }
        {
            float t = (float)(p.rout[p.nshell - 1] - p.dr[p.nshell - 1]);
            near |= fabsf(rc - t) <= 2e-4f * t;
        }
        if (near) {   // the reference's FP64 distance
            rcd = sqrt(rr);
        } else {
            rcd = (double)rc;
        }
    } else {
        double rmx, rmy, rmz, rm, rcx, rcy, rcz, rc;
        water_vectors(m, s.x, w, rmx, rmy, rmz, rm, rcx, rcy, rcz, rc);
        double scp = rmx * rcx + rmy * rcy + rmz * rcz;
        scp = fmin(1.0, fmax(-1.0, scp));
        s.theta[w] = acos(scp);
        s.rkey[w] = s.theta[w];
        v[0] = rmx; v[1] = rmy; v[2] = rmz; v[3] = rm;
        v[4] = rcx; v[5] = rcy; v[6] = rcz; v[7] = rc;
        rcd = rc;
    }
    int is = watpol_shell(p, rcd);
    if (is >= 0) {
        s.shell[w] = is;
        int k = atomicAdd(s.n_insh + is, 1);
        s.shell_list[(size_t)is * m.nwat + k] = w;
    }
}

// stable selection order of src/nonbondene.f90:6612-6628: rank = number of
// waters of the same shell with a smaller key, ties broken by water index
// (the reference scans the shell in water order and keeps the first minimum).
// kRankParts blocks per shell: each stages the whole shell's keys in shared
// memory and ranks its share of the waters, one warp per water with the
// lanes splitting the comparisons.
constexpr int kRankBlock = 256;
constexpr int kRankParts = 4;
__global__ void __launch_bounds__(kRankBlock) k_watpol_rank(DevModel m, const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.y];
    // the keys (theta, or 1 - cos theta in the mixed form) are >= 0, so the
    // bit patterns of the doubles order like the values;
    // integer compares keep the sort off the (narrow) FP64 pipe
    __shared__ long long th[1024];
    __shared__ int ww[1024];
    const int sh = blockIdx.x / kRankParts, part = blockIdx.x % kRankParts, n = s.n_insh[sh];
    const int* L = s.shell_list + (size_t)sh * m.nwat;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int base = 0; base < n; base += 1024) {
        int cn = min(1024, n - base);
        __syncthreads();
        for (int k = threadIdx.x; k < cn; k += blockDim.x) {
            ww[k] = L[base + k];
            th[k] = __double_as_longlong(s.rkey[ww[k]]);
        }
        __syncthreads();
        for (int k = part * nw + warp; k < n; k += kRankParts * nw) {
            int w;
            long long t;
            if (k >= base && k < base + cn) {
                w = ww[k - base];
                t = th[k - base];
            } else {
                w = L[k];
                t = __double_as_longlong(s.rkey[w]);
            }
            int r = 0;
            for (int v = lane; v < cn; v += kWarp) r += (th[v] < t) || (th[v] == t && ww[v] < w);
            r = __reduce_add_sync(kFull, r);
            if (lane == 0) {
                if (base == 0) s.rank[w] = r;
                else s.rank[w] += r;
            }
        }
    }
}

__global__ void k_watpol_reset(const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.x];
    if (threadIdx.x < kMaxShell) {
        s.n_insh[threadIdx.x] = 0;
        s.shell_tsum[threadIdx.x] = 0.0;
    }
}

// theta_corr update every itdis steps, src/nonbondene.f90:6630-6645
__global__ void k_watpol_update(SolventDev p, const DevState* __restrict__ states) {
    double* wstate = states[blockIdx.y].wstate;
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

// energy and gradient, src/nonbondene.f90:6646-6742.  STORED: the vectors and
// theta of this call's k_watpol_theta are current (md); otherwise they are
// recomputed from the coordinates, as the reference does in every call.
template <bool MIX, bool STORED>
__global__ void k_watpol_force(DevModel m, const DevState* __restrict__ states, SolventDev p) {
    const DevState& s = states[blockIdx.y];
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> ep;
    const double pi = 3.14159265358979323846;
    for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < m.nwat; w += gridDim.x * blockDim.x) {
        int sh = s.shell[w];
        if (sh < 0) continue;
        int n = s.n_insh[sh];
        int il = s.rank[w] + 1;
        if constexpr (MIX) {
            if (m.sa == 3) {   // FP32 arithmetic (the theta kernel's FP32 vectors when STORED)
                const float pif = 3.14159265f;
                float arg = 1.f + (1.f - 2.f * (float)il) / (float)n;
                float t0 = acosf(arg);
                t0 = t0 - 3.f * sinf(t0) * p.cstbf[sh] / 2.f;
                t0 = fminf(fmaxf(t0, 0.f), pif);
                float th = (float)s.theta[w];
                float dth = th - t0 + (float)s.wstate[sh];
                ep.add_alu(0.5f * p.fkwpolf * dth * dth);
                float dv = p.fkwpolf * dth;
                float rmx, rmy, rmz, rm, rcx, rcy, rcz, rc;
                if constexpr (STORED) {
                    const double* v = s.wvec + 8 * (size_t)w;
                    rmx = (float)v[0]; rmy = (float)v[1]; rmz = (float)v[2]; rm = (float)v[3];
                    rcx = (float)v[4]; rcy = (float)v[5]; rcz = (float)v[6]; rc = (float)v[7];
                } else {
                    water_vectors_f(m, s.xq, w, rmx, rmy, rmz, rm, rcx, rcy, rcz, rc);
                }
                float scp = fminf(1.f, fmaxf(-1.f, rmx * rcx + rmy * rcy + rmz * rcz));
                float f0 = STORED ? sinf(th) : sinf(acosf(scp));
                if (fabsf(f0) < 1.0e-10f) f0 = 1.0e-10f;
                f0 = dv * (-1.f / f0);
                float f3x = (rcx - rmx * scp) / rm, f3y = (rcy - rmy * scp) / rm, f3z = (rcz - rmz * scp) / rm;
                float f2x = (rmx - rcx * scp) / rc, f2y = (rmy - rcy * scp) / rc, f2z = (rmz - rcz * scp) / rc;
                int i = m.nat_solute + 3 * w;
                acc.grad_alu(i, (-2.f * f3x + f2x) * f0, (-2.f * f3y + f2y) * f0, (-2.f * f3z + f2z) * f0);
                acc.grad_alu(i + 1, f3x * f0, f3y * f0, f3z * f0);
                acc.grad_alu(i + 2, f3x * f0, f3y * f0, f3z * f0);
                continue;
            }
        }
        double arg = 1.0 + (1.0 - 2.0 * (double)il) / (double)n;
        double t0 = acos(arg);
        t0 = t0 - 3.0 * sin(t0) * p.cstb[sh] / 2.0;
        if (t0 < 0.0) t0 = 0.0;
        if (t0 > pi) t0 = pi;
        double th = s.theta[w];
        double dth = th - t0 + s.wstate[sh];
        ep.add(0.5 * p.fkwpol * dth * dth);
        double dv = p.fkwpol * dth;
        double rmx, rmy, rmz, rm, rcx, rcy, rcz, rc, f0;
        if constexpr (STORED) {
            const double* v = s.wvec + 8 * (size_t)w;
            rmx = v[0]; rmy = v[1]; rmz = v[2]; rm = v[3];
            rcx = v[4]; rcy = v[5]; rcz = v[6]; rc = v[7];
        } else {
            water_vectors(m, s.x, w, rmx, rmy, rmz, rm, rcx, rcy, rcz, rc);
        }
        double scp = rmx * rcx + rmy * rcy + rmz * rcz;
        scp = fmin(1.0, fmax(-1.0, scp));
        // theta = acos(scp) of this same scp when STORED
        f0 = STORED ? sin(th) : sin(acos(scp));
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
// running averages (md only), src/nonbondene.f90:6738-6741.  The shell's
// theta sum (6652-6666) is taken over the thetas placed at their ranks, by one
// warp per shell in a fixed order: deterministic whatever order the shell
// list was filled in.
__global__ void __launch_bounds__(512) k_watpol_average(DevModel m, SolventDev p, const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.y];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int sh = 0; sh < p.nshell; ++sh) {
        const int n = s.n_insh[sh];
        const int* L = s.shell_list + (size_t)sh * m.nwat;
        double* sorted = s.theta_sorted + (size_t)sh * m.nwat;
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            int w = L[k];
            sorted[s.rank[w]] = s.theta[w];
        }
    }
    __syncthreads();
    for (int sh = warp; sh < p.nshell; sh += nw) {
        const int n = s.n_insh[sh];
        const double* sorted = s.theta_sorted + (size_t)sh * m.nwat;
        double t = 0.0;
        for (int k = lane; k < n; k += kWarp) t += sorted[k];
        t = warp_sum(t);
        if (lane == 0 && n > 0) {
            s.wstate[kMaxShell + sh] += t / (double)n;
            s.wstate[2 * kMaxShell + sh] += (double)n;
        }
    }
}

// =============================================================================
// list export (parity tests): expand to the reference's atom pairs
// =============================================================================
__global__ void k_export(DevModel m, const DevState* __restrict__ states, int win, int kind,
                         int32_t* __restrict__ oi, int32_t* __restrict__ oj, int64_t cap, int* __restrict__ ocount) {
    const DevState& s = states[win];
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
// Mixed form: gather rows.  Every solute charge group and every water owns a
// row of partners; a warp walks one row and accumulates the gradient of the
// row's own atoms only, so each pair is evaluated once from each side (twice
// in FP32) and no per-pair atomics are needed.  Energies are counted once.
// =============================================================================

// appends this lane's candidate to row `row` (one warp owns the row)
__device__ __forceinline__ int row_append(int* __restrict__ row, int cap, int count, bool ok, int value) {
    unsigned b = __ballot_sync(kFull, ok);
    int lane = threadIdx.x & 31;
    if (ok) {
        int pos = count + __popc(b & ((1u << lane) - 1u));
        if (pos < cap) row[pos] = value;
    }
    return count + __popc(b);
}

// minimum-image test of a unit pair's reference atoms (a, b) against a
// cut-off band: FP32 from the packed positions unless a lattice index lies
// near one half or the distance inside the band, FP64 (box_d2) otherwise
__device__ __noinline__ bool within_box_exact(const DevModel& m, const double* __restrict__ x, int a, int b,
                                              double c) {
    return box_d2(m, x, a, b) <= c;
}
__device__ __forceinline__ bool within_box(const DevModel& m, float4 pa, float4 pb, const Band& rc,
                                           const double* __restrict__ x, int a, int b) {
    const float dx = pa.x - pb.x, dy = pa.y - pb.y, dz = pa.z - pb.z;
    const float tx = dx * m.inv_boxlf[0], ty = dy * m.inv_boxlf[1], tz = dz * m.inv_boxlf[2];
    if (near_half(tx) || near_half(ty) || near_half(tz)) return within_box_exact(m, x, a, b, rc.c);
    const float ex = m.boxlf[0] * roundf(tx) - dx, ey = m.boxlf[1] * roundf(ty) - dy, ez = m.boxlf[2] * roundf(tz) - dz;
    const float r2f = ex * ex + ey * ey + ez * ez;
    if (r2f < rc.lo) return true;
    if (r2f > rc.hi) return false;
    return within_box_exact(m, x, a, b, rc.c);
}

// partner atom j needs the general pair path against some row atom (its LJ
// code with a row atom's type is not 1); the row mask covers 128 types, and
// with more every partner takes the general path
__device__ __forceinline__ bool type_special(const DevModel& m, ulonglong2 tmask, int j) {
    if (m.natyps > 128) return true;
    const int t = m.iac[j];
    return t < 64 ? ((tmask.x >> t) & 1ull) : ((tmask.y >> (t - 64)) & 1ull);
}

// ---- cell grid of the row build -------------------------------------------
// The reference bins atoms for its neighbour search in populate_grids
// (src/nonbondene.f90:6264-6460, under USE_GRID).  Here one block per window
// bins the distance atoms of the switch-atom tests (each non-excluded solute
// group's switch atom, each non-excluded water's oxygen) on a uniform grid:
// cells of at least half the largest cut-off, counted with atomics, ranges
// from a block scan, entries scattered and then sorted by index inside each
// cell, so the grid's contents do not depend on the atomics' order.
__device__ __forceinline__ int cell_coord(float p, float lo, float inv_h, int n) {
    // clamped in FP32 first: a NaN or far-away coordinate lands in an edge cell
    return (int)fminf(fmaxf((p - lo) * inv_h, 0.0f), (float)(n - 1));
}
__device__ __forceinline__ int3 cell_of(const CellGrid& G, float4 p) {
    return make_int3(cell_coord(p.x, G.lox, G.inv_h, G.nx), cell_coord(p.y, G.loy, G.inv_h, G.ny),
                     cell_coord(p.z, G.loz, G.inv_h, G.nz));
}
__device__ __forceinline__ int cell_index(const CellGrid& G, int3 c) { return (c.z * G.ny + c.y) * G.nx + c.x; }
// periodic box: the cell of a point's fractional position (clamped in FP32: a
// NaN lands in cell 0)
__device__ __forceinline__ int pcell_coord(float p, float inv_l, int n) {
    float f = p * inv_l;
    f -= floorf(f);
    return (int)fminf(fmaxf(f * (float)n, 0.0f), (float)(n - 1));
}
template <bool BOX>
__device__ __forceinline__ int3 cell_at(const DevModel& m, const CellGrid& G, float4 p) {
    if (BOX)
        return make_int3(pcell_coord(p.x, m.inv_boxlf[0], G.nx), pcell_coord(p.y, m.inv_boxlf[1], G.ny),
                         pcell_coord(p.z, m.inv_boxlf[2], G.nz));
    return cell_of(G, p);
}

// distance atom of binned item t: solute groups first, then waters
__device__ __forceinline__ int bin_atom(const DevModel& m, int t) {
    return t < m.ncgp_solute ? m.gsw[t] : m.nat_solute + m.sa * (t - m.ncgp_solute);
}

__global__ void __launch_bounds__(1024) k_bin_cells(DevModel m, const DevState* __restrict__ states, float inv_h0,
                                                    int3 boxn) {
    const DevState& s = states[blockIdx.x];
    const float4* __restrict__ xq = s.xq;
    const int ng = m.ncgp_solute, n = ng + m.nwat;
    __shared__ float red[6][32];
    __shared__ CellGrid G;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        int a = bin_atom(m, t);
        if (m.excl[a]) continue;
        float4 p = xq[a];
        lo[0] = fminf(lo[0], p.x); lo[1] = fminf(lo[1], p.y); lo[2] = fminf(lo[2], p.z);
        hi[0] = fmaxf(hi[0], p.x); hi[1] = fmaxf(hi[1], p.y); hi[2] = fmaxf(hi[2], p.z);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(kFull, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(kFull, hi[k], o));
        }
    if (lane == 0)
        for (int k = 0; k < 3; ++k) red[k][warp] = lo[k], red[3 + k][warp] = hi[k];
    __syncthreads();
    if (threadIdx.x == 0 && boxn.x > 0) {   // periodic box: n cells per edge, set on the host
        G = CellGrid{0.f, 0.f, 0.f, 0.f, boxn.x, boxn.y, boxn.z, boxn.x * boxn.y * boxn.z};
        *s.grid = G;
    } else if (threadIdx.x == 0) {
        for (int w = 1; w < nw; ++w)
            for (int k = 0; k < 3; ++k) red[k][0] = fminf(red[k][0], red[k][w]), red[3 + k][0] = fmaxf(red[3 + k][0], red[3 + k][w]);
        float l[3], e[3];
        for (int k = 0; k < 3; ++k) {
            bool any = red[k][0] <= red[3 + k][0];   // false when nothing is binned (or NaN)
            l[k] = any ? red[k][0] : 0.0f;
            e[k] = any ? fminf(red[3 + k][0] - red[k][0], 1.0e6f) : 0.0f;
        }
        // larger cells keep the +-2 stencil sufficient: shrink inv_h until the grid fits
        float ih = inv_h0;
        int dim[3];
        for (int it = 0; it < 256; ++it) {
            for (int k = 0; k < 3; ++k) dim[k] = (int)(e[k] * ih) + 1;
            if ((long long)dim[0] * dim[1] * dim[2] <= s.cap_cells) break;
            ih *= 0.9f;
        }
        if ((long long)dim[0] * dim[1] * dim[2] > s.cap_cells) ih = 0.0f, dim[0] = dim[1] = dim[2] = 1;   // one cell
        G = CellGrid{l[0], l[1], l[2], ih, dim[0], dim[1], dim[2], dim[0] * dim[1] * dim[2]};
        *s.grid = G;
    }
    __syncthreads();
    const CellGrid g = G;
    for (int c = threadIdx.x; c < g.ncell; c += blockDim.x) s.cend_s[c] = 0, s.cend_w[c] = 0;
    __syncthreads();
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        int a = bin_atom(m, t);
        if (m.excl[a]) continue;
        const int3 cc = boxn.x > 0 ? cell_at<true>(m, g, xq[a]) : cell_of(g, xq[a]);
        atomicAdd((t < ng ? s.cend_s : s.cend_w) + cell_index(g, cc), 1);
    }
    __syncthreads();
    // exclusive scan of the counts, in place, both grids
    int carry_s = 0, carry_w = 0;
    for (int c0 = 0; c0 < g.ncell; c0 += blockDim.x) {
        int c = c0 + threadIdx.x, tot;
        int vs = c < g.ncell ? s.cend_s[c] : 0;
        int es = block_excl_scan(vs, &tot);
        if (c < g.ncell) s.cend_s[c] = carry_s + es;
        carry_s += tot;
        int vw = c < g.ncell ? s.cend_w[c] : 0;
        int ew = block_excl_scan(vw, &tot);
        if (c < g.ncell) s.cend_w[c] = carry_w + ew;
        carry_w += tot;
    }
    __syncthreads();
    // scatter: each append advances the cell's start to its end
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        int a = bin_atom(m, t);
        if (m.excl[a]) continue;
        float4 p = xq[a];
        int c = cell_index(g, boxn.x > 0 ? cell_at<true>(m, g, p) : cell_of(g, p));
        bool sol = t < ng;
        int pos = atomicAdd((sol ? s.cend_s : s.cend_w) + c, 1);
        p.w = __int_as_float(sol ? t : t - ng);
        (sol ? s.bin_s : s.bin_w)[pos] = p;
    }
    __syncthreads();
    // ascending index inside each cell (insertion sort; a cell holds a few entries)
    for (int c = threadIdx.x; c < 2 * g.ncell; c += blockDim.x) {
        bool sol = c < g.ncell;
        int cc = sol ? c : c - g.ncell;
        const int* ce = sol ? s.cend_s : s.cend_w;
        float4* b = sol ? s.bin_s : s.bin_w;
        int b0 = cc ? ce[cc - 1] : 0, b1 = ce[cc];
        for (int i = b0 + 1; i < b1; ++i) {
            float4 v = b[i];
            int key = __float_as_int(v.w), j = i - 1;
            while (j >= b0 && __float_as_int(b[j].w) > key) {
                b[j + 1] = b[j];
                --j;
            }
            b[j + 1] = v;
        }
    }
}

// The +-2 cell stencil of a row as 25 runs of consecutive cells along x
// (one per (dy, dz)), each a contiguous range of the bin.  Lane r < 25 holds
// run r's first entry (st) and the number of entries in runs before it
// (pre); lanes 25..31 hold empty runs.  The warp then walks the runs as one
// index space 0..total-1, 32 candidates at a time.
struct Runs {
    int st, pre, total;
};
// In a periodic box y and z wrap modulo n, and an x-run that crosses the
// boundary is split: seg 0 holds the part inside [0, nx), seg 1 the part
// wrapped to the other side (empty for runs that do not cross).
template <bool BOX>
__device__ __forceinline__ Runs stencil_runs(const int* __restrict__ cend, const CellGrid& G, int3 c, int seg = 0) {
    const int lane = threadIdx.x & 31;
    int st = 0, len = 0;
    if (lane < 25) {
        int y = c.y + lane % 5 - 2, z = c.z + lane / 5 - 2;
        int x0 = max(c.x - 2, 0), x1 = min(c.x + 2, G.nx - 1);
        if (BOX) {
            y = (y + G.ny) % G.ny;
            z = (z + G.nz) % G.nz;
            if (seg == 1) {   // the wrapped part, if any (nx >= 5: at most one side wraps)
                if (c.x - 2 < 0) x0 = c.x - 2 + G.nx, x1 = G.nx - 1;
                else if (c.x + 2 >= G.nx) x0 = 0, x1 = c.x + 2 - G.nx;
                else x0 = 1, x1 = 0;   // empty
            }
        }
        if (y >= 0 && y < G.ny && z >= 0 && z < G.nz && x0 <= x1) {
            int c0 = (z * G.ny + y) * G.nx + x0;
            st = c0 ? cend[c0 - 1] : 0;
            len = cend[c0 + x1 - x0] - st;
        }
    }
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int v = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += v;
    }
    return Runs{st, incl - len, __shfl_sync(kFull, incl, 31)};
}
// bin position of candidate t (all lanes call it; t >= total gives an unused value)
__device__ __forceinline__ int run_item(const Runs& R, int t) {
    int r = 0;   // the last run with pre <= t; empty runs and lanes past 24 are skipped
#pragma unroll
    for (int step = 16; step; step >>= 1) {
        int pv = __shfl_sync(kFull, R.pre, r + step);
        if (pv <= t) r += step;
    }
    return __shfl_sync(kFull, R.st, r) + t - __shfl_sync(kFull, R.pre, r);
}

// nbpplist/nbpwlist/nbwwlist selections (src/nonbondene.f90:1777-1908,
// 2842-2955, 4274-4395) stored from both sides.  Rows 0..ncgp_solute-1 are
// solute groups, the next nwat rows waters; one warp per row.  CELLS: the
// candidates are the entries of the row's +-2 cell stencil (switch-atom
// tests); otherwise every group and water is a candidate (any-atom tests).
// The inside tests are the same in both: the FP32 distance of the packed
// positions, the FP64 distance within the decision band.
template <bool CELLS, bool BOX>
__global__ void k_build_rows(DevModel m, const DevState* __restrict__ states, Cut c) {
    constexpr int NSEG = CELLS && BOX ? 2 : 1;   // a periodic stencil's wrapped x-runs come second
    const Band bpp = band(c.rcpp2, c.fpp), bpw = band(c.rcpw2, c.fpw), bww = band(c.rcww2, c.fww);
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const float4* __restrict__ xq = s.xq;
    int nrows = m.ncgp_solute + m.nwat;
    int lane = threadIdx.x & 31;
    CellGrid G;
    if (CELLS) G = *s.grid;
    for (int r = warp_id_global(); r < nrows; r += warps_total()) {
        if (r < m.ncgp_solute) {
            int g = r, is = m.gsw[g];
            int npp = 0, npf = 0, npw = 0;
            if (!m.excl[is] && !m.gallq[g]) {   // a Q-only group's row stays empty
                const float4 xs = xq[is];
                Runs R{0, 0, 0};
                const int3 cs = CELLS ? cell_at<BOX>(m, G, xs) : make_int3(0, 0, 0);
                const ulonglong2 tmask = m.gtmask[g];
                const int n1 = m.gslot[g + 1] - m.gslot[g];
                uint2* rp = s.row_gp + (size_t)g * s.cap_gp;
                int* rf = s.row_gf + (size_t)g * s.cap_gf;
                // the row's special group pairs, one per lane (found by shuffles;
                // a row with more than 32 falls back to the binary search)
                const int sl0 = m.sgl_off[g], nsl = m.sgl_off[g + 1] - sl0;
                const int2 my_sg = lane < nsl ? m.sgl_ent[sl0 + lane] : make_int2(-1, -1);
                for (int seg = 0; seg < NSEG; ++seg) {
                if (CELLS) R = stencil_runs<BOX>(s.cend_s, G, cs, seg);
                const int ncand = CELLS ? R.total : m.ncgp_solute;
                for (int j0 = 0; j0 < ncand; j0 += kWarp) {
                    const int t = j0 + lane;
                    const int bi = CELLS ? run_item(R, t) : 0;
                    bool ok = false;
                    int g2 = -1, b0 = 0, n2 = 0, ns = 0, nf = 0, sgi = -1;
                    if (t < ncand) {
                        if (CELLS) {
                            float4 it = s.bin_s[bi];
                            g2 = __float_as_int(it.w);
                            ok = g2 == g || (BOX ? within_box(m, xs, it, bpp, x, is, m.gsw[g2])
                                                 : within(r2_f(xs, it), bpp, x, is, m.gsw[g2]));
                        } else if (BOX) {
                            g2 = t;
                            ok = g2 == g || within_box(m, xs, xq[m.gsw[g2]], bpp, x, is, m.gsw[g2]);
                        } else {
                            g2 = t;
                            if (!m.excl[m.gsw[g2]]) ok = g2 == g || gg_inside(m, x, xq, g, g2, bpp);
                        }
                    }
                    if (nsl <= kWarp) {
                        for (int c = 0; c < nsl; ++c) {   // warp-uniform
                            const int eg = __shfl_sync(kFull, my_sg.x, c), es = __shfl_sync(kFull, my_sg.y, c);
                            if (eg == g2) sgi = es;
                        }
                    }
                    if (t < ncand) {
                        if (ok) {
                            b0 = m.gslot[g2];
                            n2 = m.gslot[g2 + 1] - b0;
                            if (nsl > kWarp)
                                sgi = sg_find(m, g <= g2 ? (long long)g * m.ncgp_solute + g2
                                                         : (long long)g2 * m.ncgp_solute + g);
                            // the general path: the group itself, group pairs with
                            // excluded / 1-4 atom pairs, and partner types with LJ
                            // code 2 against a row atom; plain code-1 partners otherwise
                            const bool all_special = g2 == g || sgi >= 0;
                            for (int b = 0; b < n2; ++b) {
                                int j = m.gatom[b0 + b];
                                if (m.iqatom[j] >= 0) continue;
                                if (all_special || type_special(m, tmask, j)) ++ns;
                                else ++nf;
                            }
                        }
                    }
                    // row-local offsets of both lists: one inclusive warp scan of the
                    // packed counts (each below 2^15 per lane, at most 15 * 32 per warp)
                    int incl = ns | (nf << 16);
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        int v = __shfl_up_sync(kFull, incl, o);
                        if (lane >= o) incl += v;
                    }
                    int total = __shfl_sync(kFull, incl, 31);
                    if (ns + nf > 0) {
                        int ps = npp + (incl & 0xffff) - ns, pf = npf + (incl >> 16) - nf;
                        const bool lower = g <= g2;
                        const bool all_special = g2 == g || sgi >= 0;
                        unsigned flags = (g < g2 ? 1u : 0u) | (g == g2 ? 2u : 0u);
                        for (int b = 0; b < n2; ++b) {
                            int j = m.gatom[b0 + b];
                            if (m.iqatom[j] >= 0) continue;
                            if (!all_special && !type_special(m, tmask, j)) {
                                if (pf < s.cap_gf) rf[pf] = j;
                                ++pf;
                                continue;
                            }
                            // 2-bit kind per row atom against partner atom b (the
                            // host's table of the group pair; none: every kind 0)
                            unsigned mask = g == g2 ? 1u << (2 * b) : 0u;   // the atom itself
                            if (sgi >= 0) mask = m.sgm[m.sgm_off[sgi] + (lower ? b : n1 + b)];
                            if (m.type_in_entry) mask |= (unsigned)m.iac[j] << 16;
                            if (ps < s.cap_gp) rp[ps] = make_uint2((unsigned)j | (flags << 28), mask);
                            ++ps;
                        }
                    }
                    npp += total & 0xffff;
                    npf += total >> 16;
                }
                }
                int* rw = s.row_gw + (size_t)g * s.cap_gw;
                for (int seg = 0; seg < NSEG; ++seg) {
                if (CELLS) R = stencil_runs<BOX>(s.cend_w, G, cs, seg);
                const int ncw = CELLS ? R.total : m.nwat;
                for (int j0 = 0; j0 < ncw; j0 += kWarp) {
                    const int t = j0 + lane;
                    const int bi = CELLS ? run_item(R, t) : 0;
                    bool ok = false;
                    int jw = t;
                    if (t < ncw) {
                        if (CELLS) {
                            float4 it = s.bin_w[bi];
                            jw = __float_as_int(it.w);
                            const int jo = m.nat_solute + m.sa * jw;
                            ok = BOX ? within_box(m, xs, it, bpw, x, is, jo) : within(r2_f(xs, it), bpw, x, is, jo);
                        } else if (BOX) {
                            const int jo = m.nat_solute + m.sa * jw;
                            ok = within_box(m, xs, xq[jo], bpw, x, is, jo);
                        } else {
                            int jo = m.nat_solute + m.sa * jw;
                            if (!m.excl[jo]) ok = gw_inside(m, x, xq, g, jo, bpw);
                        }
                    }
                    npw = row_append(rw, s.cap_gw, npw, ok, jw);
                }
                }
            }
            if (lane == 0) {
                s.cnt_gp[g] = min(npp, s.cap_gp);
                s.cnt_gf[g] = min(npf, s.cap_gf);
                s.cnt_gw[g] = min(npw, s.cap_gw);
                atomicMax(s.cnt + C_RGP, npp);
                atomicMax(s.cnt + C_RGF, npf);
                atomicMax(s.cnt + C_RGW, npw);
            }
        } else {
            int w = r - m.ncgp_solute, io = m.nat_solute + m.sa * w;
            int nww = 0, nwg = 0;
            if (!m.excl[io]) {
                const float4 xi = xq[io];
                Runs R{0, 0, 0};
                const int3 ci = CELLS ? cell_at<BOX>(m, G, xi) : make_int3(0, 0, 0);
                int* rw = s.row_ww + (size_t)w * s.cap_rww;
                for (int seg = 0; seg < NSEG; ++seg) {
                if (CELLS) R = stencil_runs<BOX>(s.cend_w, G, ci, seg);
                const int ncw = CELLS ? R.total : m.nwat;
                for (int j0 = 0; j0 < ncw; j0 += kWarp) {
                    const int t = j0 + lane;
                    const int bi = CELLS ? run_item(R, t) : 0;
                    bool ok = false;
                    int jw = t;
                    if (t < ncw) {
                        if (CELLS) {
                            float4 it = s.bin_w[bi];
                            jw = __float_as_int(it.w);
                            const int jo = m.nat_solute + m.sa * jw;
                            ok = jw != w && (BOX ? within_box(m, xi, it, bww, x, io, jo)
                                                 : within(r2_f(xi, it), bww, x, io, jo));
                        } else if (jw != w) {
                            int jo = m.nat_solute + m.sa * jw;
                            if (BOX) ok = within_box(m, xi, xq[jo], bww, x, io, jo);
                            else if (!m.excl[jo]) ok = within(r2_f(xi, xq[jo]), bww, x, io, jo);
                        }
                    }
                    nww = row_append(rw, s.cap_rww, nww, ok, jw);
                }
                }
                int* rg = s.row_wg + (size_t)w * s.cap_wg;
                for (int seg = 0; seg < NSEG; ++seg) {
                if (CELLS) R = stencil_runs<BOX>(s.cend_s, G, ci, seg);
                const int ncg = CELLS ? R.total : m.ncgp_solute;
                for (int j0 = 0; j0 < ncg; j0 += kWarp) {
                    const int t = j0 + lane;
                    const int bi = CELLS ? run_item(R, t) : 0;
                    bool ok = false;
                    int g = t;
                    if (t < ncg) {
                        // the same test as from the group side
                        if (CELLS) {
                            float4 it = s.bin_s[bi];
                            g = __float_as_int(it.w);
                            ok = BOX ? within_box(m, it, xi, bpw, x, m.gsw[g], io)
                                     : within(r2_f(it, xi), bpw, x, m.gsw[g], io);
                        } else if (BOX) {
                            ok = within_box(m, xq[m.gsw[g]], xi, bpw, x, m.gsw[g], io);
                        } else if (!m.excl[m.gsw[g]]) {
                            ok = gw_inside(m, x, xq, g, io, bpw);
                        }
                    }
                    nwg = row_append(rg, s.cap_wg, nwg, ok, g);
                }
                }
            }
            if (lane == 0) {
                s.cnt_ww[w] = min(nww, s.cap_rww);
                s.cnt_wg[w] = min(nwg, s.cap_wg);
                atomicMax(s.cnt + C_RWW, nww);
                atomicMax(s.cnt + C_RWG, nwg);
            }
        }
    }
}

// nonbond_solvent_internal, src/nonbondene.f90:6082-6154 (in a box
// nonbond_solvent_internal_box, 6158-6228): the listed pairs
// (offsets in a molecule, nonbnd_solv_int) inside every solvent molecule, for
// solvents with torsions; q_dist2 and the reference's grouping of dv.  FP64
// in both forms (a few pairs per molecule); the mixed form accumulates in
// fixed point.
template <bool MIX>
__global__ void k_solvent_internal(DevModel m, const DevState* __restrict__ states, const int2* __restrict__ ij,
                                   const double* __restrict__ par, int n) {
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel, evdw;
    for (int iw = blockIdx.x * blockDim.x + threadIdx.x; iw < m.nwat; iw += gridDim.x * blockDim.x) {
        int is = m.nat_solute + m.sa * iw;
        for (int ip = 0; ip < n; ++ip) {
            int ia = is + ij[ip].x, ib = is + ij[ip].y;
            double tx = x[3 * ib] - x[3 * ia], ty = x[3 * ib + 1] - x[3 * ia + 1], tz = x[3 * ib + 2] - x[3 * ia + 2];
            if (m.box) {   // nonbond_solvent_internal_box, src/nonbondene.f90:6158-6228: minimum image
                double sx, sy, sz;
                box_shift(m, x, ia, ib, sx, sy, sz);
                tx += sx, ty += sy, tz += sz;
            }
            double r2 = 1.0 / (tx * tx + ty * ty + tz * tz);
            double r = sqrt(r2);
            double r6 = r2 * r2 * r2;
            double r12 = r6 * r6;
            double vel = par[3 * ip + 2] * r, va = par[3 * ip] * r12, vb = par[3 * ip + 1] * r6;
            double dv = r2 * (-vel) + r2 * (-12.0 * va + 6.0 * vb);
            eel.add(vel);
            evdw.add(va - vb);
            if constexpr (MIX) {
                acc.gradd(ia, -tx * dv, -ty * dv, -tz * dv);
                acc.gradd(ib, tx * dv, ty * dv, tz * dv);
            } else {
                acc.grad(ia, -tx * dv, -ty * dv, -tz * dv);
                acc.grad(ib, tx * dv, ty * dv, tz * dv);
            }
        }
    }
    eel.flush(acc, E_WW_EL);
    evdw.flush(acc, E_WW_VDW);
}

// FP32 pair (nbe / nbe_spc): adds the gradient on atom i to g, returns energies
__device__ __forceinline__ void pair_f(float4 a, float4 b, float A, float B, float el, bool lj, float& gx,
                                      float& gy, float& gz, float& vel, float& vdw) {
    PairF q = nbe_f(a, b, A, B, el, lj);
    gx -= q.tx * q.dv;
    gy -= q.ty * q.dv;
    gz -= q.tz * q.dv;
    vel = q.vel;
    vdw = q.vdw;
}

// type-pair LJ parameters (code ljcod: A,B; code 3: A,B) staged in shared
// memory when the type table is small; the kernels take it as dynamic shared
// memory of exactly natyps^2 entries, leaving the rest of the SM's 256 KB to
// the L1 cache that serves the partner gathers
struct TypeTab {
    const float4* t;
    int nt;
    __device__ __forceinline__ float4 operator()(int a, int b) const { return t[a * nt + b]; }
};
__device__ __forceinline__ TypeTab stage_types(const DevModel& m, float4* sh) {
    if (m.natyps <= kMaxTypesShared) {
        for (int k = threadIdx.x; k < m.natyps * m.natyps; k += blockDim.x) sh[k] = m.ljpair[k];
        __syncthreads();
        return TypeTab{sh, m.natyps};
    }
    return TypeTab{m.ljpair, m.natyps};
}

// Asynchronous global-to-shared copies of row entries (16 bytes per lane,
// L2 only): a warp fetches the next chunk of its row while it evaluates the
// current one, so the DRAM latency of the streamed rows is paid once per
// chunk instead of once per loop iteration.  Row capacities are multiples of
// 4 entries, so every row starts on a 16-byte boundary and a chunk rounded up
// to whole 16-byte units stays inside its row.
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
constexpr int kRowChunk = 128;   // entries per prefetched chunk

// solute group rows: pp (partner atoms with exclusion / 1-4 kinds) and pw
// (partner waters): gradient of the group's own atoms.  Every solute pair sits
// in the rows of both of its atoms (a pair inside one group twice in that
// group's row) and both evaluations give the same FP32 energy, so the row sums
// of all pp energies are halved instead of testing which side counts a pair.
// Groups of at most 8 atoms carry the partner's LJ type in entry bits 16..31.
//
// Resident 128-thread blocks per SM asked of the register allocator: the
// kernel waits mostly on its gathers, so occupancy pays more than the few
// spilled registers (6 blocks = 80 registers for groups of up to 6 atoms).
// Two row atoms against one partner in packed FP32x2 arithmetic (GB300's
// FFMA2 / FMUL2 / FADD2; one rsqrt per atom on the SFU): the plain code-1
// pair of the geometric rule, A = fa fj.x and B = fb fj.y.  The row kernels
// are bound by the latency of each pair's dependent chain, and a packed
// instruction advances two chains.  n* are the negated row positions, q the
// row charges; adds the row atoms' gradient into g* and their energies into
// pel / pvdw.
__device__ __forceinline__ void pair2_plain(float2 nx, float2 ny, float2 nz, float2 q, float2 fa, float2 fb,
                                            float2 bx, float2 by, float2 bz, float2 bq, float2 fjx, float2 fjy,
                                            float2& gx, float2& gy, float2& gz, float2& pel, float2& pvdw) {
    const float2 tx = __fadd2_rn(bx, nx), ty = __fadd2_rn(by, ny), tz = __fadd2_rn(bz, nz);
    float2 rr = __fmul2_rn(tx, tx);
    rr = __ffma2_rn(ty, ty, rr);
    rr = __ffma2_rn(tz, tz, rr);
    const float2 ri = make_float2(rsqrtf(rr.x), rsqrtf(rr.y));
    const float2 r2 = __fmul2_rn(ri, ri);
    const float2 vel = __fmul2_rn(__fmul2_rn(q, bq), ri);
    const float2 r6 = __fmul2_rn(__fmul2_rn(r2, r2), r2);
    const float2 va = __fmul2_rn(__fmul2_rn(__fmul2_rn(fa, fjx), r6), r6);
    const float2 vb = __fmul2_rn(__fmul2_rn(fb, fjy), r6);
    // -dv = r2 (vel + 12 va - 6 vb); the gradient of the row atom is -t dv
    float2 t = __ffma2_rn(make_float2(12.f, 12.f), va, vel);
    t = __ffma2_rn(make_float2(-6.f, -6.f), vb, t);
    const float2 ndv = __fmul2_rn(r2, t);
    gx = __ffma2_rn(tx, ndv, gx);
    gy = __ffma2_rn(ty, ndv, gy);
    gz = __ffma2_rn(tz, ndv, gz);
    pel = __fadd2_rn(pel, vel);
    pvdw = __fadd2_rn(pvdw, __ffma2_rn(make_float2(-1.f, -1.f), vb, va));
}

// periodic box: partner position p at the image of its unit's reference
// atom ref_p nearest the row's reference atom ref_row, p + boxlength *
// nint((ref_row - ref_p) / boxlength) in FP32 (the unit pair's shift of the
// *_box energy routines; for a listed pair the lattice index is never near a
// half, since the reference atoms are within a cut-off below half a box)
__device__ __forceinline__ float4 at_image(const DevModel& m, float4 p, float4 ref_row, float4 ref_p) {
    p.x += m.boxlf[0] * roundf((ref_row.x - ref_p.x) * m.inv_boxlf[0]);
    p.y += m.boxlf[1] * roundf((ref_row.y - ref_p.y) * m.inv_boxlf[1]);
    p.z += m.boxlf[2] * roundf((ref_row.z - ref_p.z) * m.inv_boxlf[2]);
    return p;
}

#ifndef QNB_ROWS_MIN_BLOCKS
#define QNB_ROWS_MIN_BLOCKS 0   // 0: the per-size default below
#endif
// resident 128-thread blocks per SM the row kernel is compiled for: the
// packed plain loop of the geometric rule holds twice the row-atom registers
// and measured best at 5 (96 registers: 212 us per 51-window R25 step, 226 at
// 6 blocks, where it spills inside the loop); the scalar loop at 6
template <int MAXG, bool GEOM>
constexpr int rows_min_blocks() {
    return QNB_ROWS_MIN_BLOCKS ? QNB_ROWS_MIN_BLOCKS
                               : (MAXG <= 6 ? (GEOM ? 5 : 6) : (MAXG <= 8 ? 4 : 1));
}
template <int MAXG, bool GEOM, bool BOX>
__global__ void __launch_bounds__(128, rows_min_blocks<MAXG, GEOM>()) k_rows_solute(DevModel m, const DevState* __restrict__ states) {
    extern __shared__ float4 sh_lj[];   // natyps^2 type-pair table (dynamic: only its real size)
    __shared__ __align__(16) uint2 sh_pp[4][2][kRowChunk];   // per warp: double-buffered special pp entries
    __shared__ __align__(16) int sh_pf[4][2][kRowChunk];     // per warp: double-buffered plain pp entries
    __shared__ __align__(16) int sh_pw[4][kRowChunk];        // per warp: first chunk of pw entries
    constexpr bool kTypeInEntry = MAXG <= 8;
    const DevState& s = states[blockIdx.y];
    const int wib = threadIdx.x >> 5;
    TypeTab lj = stage_types(m, sh_lj);
    const float4* __restrict__ xq = s.xq;
    // m.el14f, not (float)m.el14: under register pressure the compiler may
    // rematerialise a double-to-float conversion of the parameter inside the
    // pair loop, and that conversion runs on the narrow FP64 pipe
    const float el14 = m.el14f;
    int lane = threadIdx.x & 31;
    for (int g = warp_id_global(); g < m.ncgp_solute; g += warps_total()) {
        int npp = s.cnt_gp[g], npw = s.cnt_gw[g];   // an empty row still writes its zeros
        int a0 = m.gslot[g], n1 = m.gslot[g + 1] - a0;
        if (n1 > MAXG) {   // a Q-only group larger than the rows handle: empty row, zero gradient
            for (int a = lane; a < 3 * n1; a += kWarp) s.frow[3 * m.gatom[a0 + a / 3] + a % 3] = 0.f;
            continue;
        }
        // periodic box: the row group's reference atom (its lattice shifts)
        const float4 xsw = BOX ? xq[m.gsw[g]] : make_float4(0.f, 0.f, 0.f, 0.f);
        int ta[MAXG];
        float4 xa[MAXG];
        bool qa[MAXG];
        float f[MAXG][3];
#pragma unroll
        for (int a = 0; a < MAXG; ++a) {
            f[a][0] = f[a][1] = f[a][2] = 0.f;
            if (a < n1) {
                int i = m.gatom[a0 + a];
                ta[a] = m.iac[i];
                xa[a] = xq[i];
                qa[a] = m.iqatom[i] >= 0;
            } else {
                ta[a] = 0;
                xa[a] = make_float4(0, 0, 0, 0);
                qa[a] = true;
            }
        }
        // per-row FP32 energy sums of this lane, converted to fixed point once
        // per row (row contents do not depend on the grid, so neither do they)
        float rpel = 0.f, rpvdw = 0.f, rwel = 0.f, rwvdw = 0.f;
        // ---- solute partner atoms (nonbond_pp, src/nonbondene.f90:4694-4760):
        // the special entries (kinds, any LJ code) first, then the water
        // partners, then the plain solute partners (the hot loop, last, so the
        // type indices are no longer live in it)
        const uint2* rp = s.row_gp + (size_t)g * s.cap_gp;
        const int* rf = s.row_gf + (size_t)g * s.cap_gf;
        const int* rw = s.row_gw + (size_t)g * s.cap_gw;
        const int npf = s.cnt_gf[g];
        const int nchunk = (npp + kRowChunk - 1) / kRowChunk, nfchunk = (npf + kRowChunk - 1) / kRowChunk;
        auto fetch_pp = [&](int ch) {
            int e0 = ch * kRowChunk, units = (min(kRowChunk, npp - e0) + 1) >> 1;
            for (int u = lane; u < units; u += kWarp) cp_async16(&sh_pp[wib][ch & 1][2 * u], rp + e0 + 2 * u);
        };
        auto fetch_pf = [&](int ch) {
            int e0 = ch * kRowChunk, units = (min(kRowChunk, npf - e0) + 3) >> 2;
            for (int u = lane; u < units; u += kWarp) cp_async16(&sh_pf[wib][ch & 1][4 * u], rf + e0 + 4 * u);
        };
        if (nchunk > 0) fetch_pp(0);
        if (nfchunk > 0) fetch_pf(0);
        for (int u = lane; u < (min(kRowChunk, npw) + 3) >> 2; u += kWarp) cp_async16(&sh_pw[wib][4 * u], rw + 4 * u);
        cp_async_commit();
        for (int ch = 0; ch < nchunk; ++ch) {
          if (ch + 1 < nchunk) {
              fetch_pp(ch + 1);
              cp_async_commit();
              cp_async_wait<1>();
          } else {
              cp_async_wait<0>();
          }
          __syncwarp();
          const uint2* buf = sh_pp[wib][ch & 1];
          const int n = min(kRowChunk, npp - ch * kRowChunk);
          for (int k = lane; k < n; k += kWarp) {
            uint2 e = buf[k];
            int j = (int)(e.x & 0x0fffffffu);
            float4 xb = xq[j];
            if (BOX) xb = at_image(m, xb, xsw, xq[m.swat[j]]);
            int tj = kTypeInEntry ? (int)(e.y >> 16) : m.iac[j];
            const unsigned kinds = kTypeInEntry ? (e.y & 0xffffu) : e.y;
#pragma unroll
            for (int a = 0; a < MAXG; ++a) {
                if (qa[a]) continue;
                unsigned kind = (kinds >> (2 * a)) & 3u;
                if (kind == 1u) continue;
                float4 p = lj(ta[a], tj);
                bool is14 = kind == 3u;
                float A = is14 ? p.z : p.x, B = is14 ? p.w : p.y;
                float el = xa[a].w * xb.w;
                if (is14) el *= el14;
                float vel, vdw;
                pair_f(xa[a], xb, A, B, el, true, f[a][0], f[a][1], f[a][2], vel, vdw);
                rpel += vel;
                rpvdw += vdw;
            }
          }
          __syncwarp();   // this buffer is refilled two chunks later
        }
        if (nchunk == 0) {
            cp_async_wait<0>();
            __syncwarp();
        }
        // ---- water partners (nonbond_pw, src/nonbondene.f90:4856-4916); energy counted here
        if (m.sa == 3 && m.wlj_mask == 1u) {   // SPC: O with LJ, two LJ-free H; the molecule loaded at once
          const float qo = m.wcrgf[0], qh1 = m.wcrgf[1], qh2 = m.wcrgf[2];
          const int to = m.wtype[0];
          for (int k = lane; k < npw; k += kWarp) {
            int j0 = m.nat_solute + 3 * (k < kRowChunk ? sh_pw[wib][k] : rw[k]);
            float4 xo = xq[j0], xh1 = xq[j0 + 1], xh2 = xq[j0 + 2];
            if (BOX) {
                const float4 xr = xo;
                xo = at_image(m, xo, xsw, xr), xh1 = at_image(m, xh1, xsw, xr), xh2 = at_image(m, xh2, xsw, xr);
            }
#pragma unroll
            for (int a = 0; a < MAXG; ++a) {
                if (qa[a]) continue;
                float4 p = lj(ta[a], to);
                float v1, d1, v2, d2, v3, d3;
                pair_f(xa[a], xo, p.x, p.y, xa[a].w * qo, true, f[a][0], f[a][1], f[a][2], v1, d1);
                pair_f(xa[a], xh1, 0.f, 0.f, xa[a].w * qh1, false, f[a][0], f[a][1], f[a][2], v2, d2);
                pair_f(xa[a], xh2, 0.f, 0.f, xa[a].w * qh2, false, f[a][0], f[a][1], f[a][2], v3, d3);
                rwel += v1 + v2 + v3;
                rwvdw += d1;
            }
          }
        } else {
        for (int k = lane; k < npw; k += kWarp) {
            int j0 = m.nat_solute + m.sa * (k < kRowChunk ? sh_pw[wib][k] : rw[k]);
            const float4 xr = BOX ? xq[j0] : make_float4(0.f, 0.f, 0.f, 0.f);
            for (int b = 0; b < m.sa; ++b) {
                float4 xb = xq[j0 + b];
                if (BOX) xb = at_image(m, xb, xsw, xr);
                int tw = m.wtype[b];
                if ((m.wlj_mask >> b) & 1u) {
#pragma unroll
                    for (int a = 0; a < MAXG; ++a) {
                        if (qa[a]) continue;
                        float4 p = lj(ta[a], tw);
                        float vel, vdw;
                        pair_f(xa[a], xb, p.x, p.y, xa[a].w * m.wcrgf[b], true, f[a][0], f[a][1], f[a][2], vel, vdw);
                        rwel += vel;
                        rwvdw += vdw;
                    }
                } else {   // A = B = 0 with every solute type: the Coulomb term alone, bit for bit
#pragma unroll
                    for (int a = 0; a < MAXG; ++a) {
                        if (qa[a]) continue;
                        float vel, vdw;
                        pair_f(xa[a], xb, 0.f, 0.f, xa[a].w * m.wcrgf[b], false, f[a][0], f[a][1], f[a][2], vel, vdw);
                        rwel += vel;
                    }
                }
            }
        }
        }
        // plain partners: LJ code 1 with every row atom, no excluded or 1-4
        // pair; with the geometric rule A and B are the products of the atoms'
        // FP32 code-1 factors (the type table holds the same products)
        {
          // with the geometric rule a Q row atom gets zero charge and LJ
          // factors here, so its terms are exact zeros (its row gradient is
          // discarded) and the loop needs no per-atom test
          float fa[MAXG], fb[MAXG];
#pragma unroll
          for (int a = 0; a < MAXG; ++a) {
              float2 f1 = (GEOM && a < n1 && !qa[a]) ? m.ljf1[m.gatom[a0 + a]] : make_float2(0.f, 0.f);
              fa[a] = f1.x;
              fb[a] = f1.y;
              if (GEOM && qa[a]) xa[a].w = 0.f;
          }
          for (int ch = 0; ch < nfchunk; ++ch) {
            if (ch + 1 < nfchunk) {   // chunk 0 came with the first group
                fetch_pf(ch + 1);
                cp_async_commit();
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncwarp();
            const int* buf = sh_pf[wib][ch & 1];
            const int n = min(kRowChunk, npf - ch * kRowChunk);
            // the next entry's partner data is loaded one iteration ahead
            float4 xbn = make_float4(0.f, 0.f, 0.f, 0.f);
            float2 fjn = make_float2(0.f, 0.f);
            int tjn = 0;
            if (lane < n) {
                const int j = buf[lane];
                xbn = xq[j];
                if (BOX) xbn = at_image(m, xbn, xsw, xq[m.swat[j]]);
                if constexpr (GEOM) fjn = m.ljf1[j];
                else tjn = m.iac[j];
            }
            if constexpr (GEOM) {
              // row atoms in pairs (2p, 2p + 1); an odd group's last pair has a
              // dummy atom far away with zero charge and factors
              constexpr int NP = MAXG / 2;
              float2 nx[NP], ny[NP], nz[NP], q2[NP], fa2[NP], fb2[NP], gx[NP], gy[NP], gz[NP];
              float2 pel = make_float2(0.f, 0.f), pvdw = make_float2(0.f, 0.f);
#pragma unroll
              for (int p = 0; p < NP; ++p) {
                  const int a = 2 * p, b = 2 * p + 1;
                  const bool hb = b < n1;
                  nx[p] = make_float2(-xa[a].x, hb ? -xa[b].x : -1.0e4f);
                  ny[p] = make_float2(-xa[a].y, hb ? -xa[b].y : -1.0e4f);
                  nz[p] = make_float2(-xa[a].z, hb ? -xa[b].z : -1.0e4f);
                  q2[p] = make_float2(xa[a].w, hb ? xa[b].w : 0.f);
                  fa2[p] = make_float2(fa[a], hb ? fa[b] : 0.f);
                  fb2[p] = make_float2(fb[a], hb ? fb[b] : 0.f);
                  gx[p] = make_float2(f[a][0], f[b][0]);   // the accumulators move into the pairs
                  gy[p] = make_float2(f[a][1], f[b][1]);
                  gz[p] = make_float2(f[a][2], f[b][2]);
              }
              for (int k = lane; k < n; k += kWarp) {
                const float4 xb = xbn;
                const float2 fj = fjn;
                if (k + kWarp < n) {
                    const int jn = buf[k + kWarp];
                    xbn = xq[jn];
                    if (BOX) xbn = at_image(m, xbn, xsw, xq[m.swat[jn]]);
                    fjn = m.ljf1[jn];
                }
                const float2 bx = make_float2(xb.x, xb.x), by = make_float2(xb.y, xb.y),
                             bz = make_float2(xb.z, xb.z), bq = make_float2(xb.w, xb.w),
                             fjx = make_float2(fj.x, fj.x), fjy = make_float2(fj.y, fj.y);
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    if (2 * p >= n1) break;   // warp-uniform
                    pair2_plain(nx[p], ny[p], nz[p], q2[p], fa2[p], fb2[p], bx, by, bz, bq, fjx, fjy, gx[p], gy[p],
                                gz[p], pel, pvdw);
                }
              }
#pragma unroll
              for (int p = 0; p < NP; ++p) {
                  f[2 * p][0] = gx[p].x;
                  f[2 * p][1] = gy[p].x;
                  f[2 * p][2] = gz[p].x;
                  f[2 * p + 1][0] = gx[p].y;
                  f[2 * p + 1][1] = gy[p].y;
                  f[2 * p + 1][2] = gz[p].y;
              }
              rpel += pel.x + pel.y;
              rpvdw += pvdw.x + pvdw.y;
            } else {
              for (int k = lane; k < n; k += kWarp) {
                const float4 xb = xbn;
                const int tj = tjn;
                if (k + kWarp < n) {
                    const int jn = buf[k + kWarp];
                    tjn = m.iac[jn];
                    xbn = xq[jn];
                    if (BOX) xbn = at_image(m, xbn, xsw, xq[m.swat[jn]]);
                }
#pragma unroll
                for (int a = 0; a < MAXG; ++a) {
                    if (qa[a]) continue;   // warp-uniform
                    float4 p = lj(ta[a], tj);
                    float vel, vdw;
                    pair_f(xa[a], xb, p.x, p.y, xa[a].w * xb.w, true, f[a][0], f[a][1], f[a][2], vel, vdw);
                    rpel += vel;
                    rpvdw += vdw;
                }
              }
            }
            __syncwarp();   // this buffer is refilled two chunks later
          }
        }
        __syncwarp();   // sh_pw is refilled by the next row
        // The row owns its atoms' pp and pw gradient and its energies: FP32
        // warp sums in a fixed shuffle order, stored without atomics
        // (k_apply_fixed converts each atom's sum once to 64-bit fixed point
        // and adds it as an integer); the row's four energies are converted
        // to fixed point once and added to the window's energy slots as
        // integers (order-free, so the step needs no separate energy sum)
        if constexpr (MAXG <= 8) {
            // the row atoms' 3 x 8 gradient components and the 4 energies in
            // one transposed warp sum: lane v ends with value v
            float gv[32];
#pragma unroll
            for (int a = 0; a < 8; ++a) {
#pragma unroll
                for (int c = 0; c < 3; ++c) gv[3 * a + c] = a < MAXG ? f[a < MAXG ? a : 0][c] : 0.f;
            }
            gv[24] = 0.5f * rpel, gv[25] = 0.5f * rpvdw, gv[26] = rwel, gv[27] = rwvdw;
            gv[28] = gv[29] = gv[30] = gv[31] = 0.f;
            const float v = reduce_scatter<32>(gv, lane);
            if (lane < 3 * n1) {
                const int i = m.gatom[a0 + lane / 3];
                s.frow[3 * i + lane % 3] = m.iqatom[i] >= 0 ? 0.f : v;
            } else if (lane >= 24 && lane < 28 && v != 0.f) {   // E_PP_EL, E_PP_VDW, E_PW_EL, E_PW_VDW
                atomicAdd(s.efix + E_PP_EL + (lane - 24), to_fix(v));
            }
        } else {
            float e0 = warp_sum(0.5f * rpel), e1 = warp_sum(0.5f * rpvdw), e2 = warp_sum(rwel), e3 = warp_sum(rwvdw);
            if (lane == 0) {
                const float ev[4] = {e0, e1, e2, e3};
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (ev[k] != 0.f) atomicAdd(s.efix + E_PP_EL + k, to_fix(ev[k]));
            }
#pragma unroll
            for (int a = 0; a < MAXG; ++a) {
                if (a >= n1) break;   // warp-uniform
                float v0 = warp_sum(f[a][0]), v1 = warp_sum(f[a][1]), v2 = warp_sum(f[a][2]);
                if (lane == 0) {
                    int i = m.gatom[a0 + a];
                    float* fr = s.frow + 3 * i;
                    fr[0] = qa[a] ? 0.f : v0;
                    fr[1] = qa[a] ? 0.f : v1;
                    fr[2] = qa[a] ? 0.f : v2;
                }
            }
        }
    }
}

// water rows: ww (waters, SPC fast path as nonbond_ww_spc) and wp (solute
// groups) gradient of the water's atoms
template <bool SPC, bool BOX>
__global__ void __launch_bounds__(128, 8) k_rows_water(DevModel m, const DevState* __restrict__ states) {
    extern __shared__ float4 sh_lj[];   // natyps^2 type-pair table (dynamic: only its real size)
    __shared__ __align__(16) int sh_ww[4][2][kRowChunk];   // per warp: double-buffered ww entries
    __shared__ __align__(16) int sh_wg[4][kRowChunk];      // per warp: first chunk of wp entries
    const DevState& s = states[blockIdx.y];
    const int wib = threadIdx.x >> 5;
    TypeTab lj = stage_types(m, sh_lj);
    const float4* __restrict__ xq = s.xq;
    int lane = threadIdx.x & 31;
    const int sa = m.sa;
    // SPC rows: 3-atom molecules (the launcher's choice), so the row's atom
    // arrays hold 3 entries and a partner's atoms are loaded one iteration
    // ahead
    constexpr int NA = SPC ? 3 : kMaxSolv;
    for (int w = warp_id_global(); w < m.nwat; w += warps_total()) {
        int nww = s.cnt_ww[w], nwg = s.cnt_wg[w];   // an empty row still writes its zeros
        int i0 = m.nat_solute + sa * w;
        float4 xa[NA];
        float f[NA][3];
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            f[a][0] = f[a][1] = f[a][2] = 0.f;
            xa[a] = a < sa ? xq[i0 + a] : make_float4(0, 0, 0, 0);
        }
        float rel = 0.f, rvdw = 0.f;
        const int* rw = s.row_ww + (size_t)w * s.cap_rww;
        const int* rg = s.row_wg + (size_t)w * s.cap_wg;
        const int nchunk = (nww + kRowChunk - 1) / kRowChunk;
        auto fetch_ww = [&](int ch) {
            int e0 = ch * kRowChunk, units = (min(kRowChunk, nww - e0) + 3) >> 2;
            for (int u = lane; u < units; u += kWarp) cp_async16(&sh_ww[wib][ch & 1][4 * u], rw + e0 + 4 * u);
        };
        if (nchunk > 0) fetch_ww(0);
        for (int u = lane; u < (min(kRowChunk, nwg) + 3) >> 2; u += kWarp) cp_async16(&sh_wg[wib][4 * u], rg + 4 * u);
        cp_async_commit();
        for (int ch = 0; ch < nchunk; ++ch) {
          if (ch + 1 < nchunk) {
              fetch_ww(ch + 1);
              cp_async_commit();
              cp_async_wait<1>();
          } else {
              cp_async_wait<0>();
          }
          __syncwarp();
          const int* buf = sh_ww[wib][ch & 1];
          const int n = min(kRowChunk, nww - ch * kRowChunk);
          if constexpr (SPC) {
            float4 nx0 = make_float4(0.f, 0.f, 0.f, 0.f), nx1 = nx0, nx2 = nx0;
            int nw2 = 0;
            if (lane < n) {
                nw2 = buf[lane];
                const int j = m.nat_solute + 3 * nw2;
                nx0 = xq[j], nx1 = xq[j + 1], nx2 = xq[j + 2];
            }
            for (int k = lane; k < n; k += kWarp) {
              const int w2 = nw2;
              const float4 xp[3] = {nx0, nx1, nx2};
              if (k + kWarp < n) {   // the next partner, one iteration ahead
                  nw2 = buf[k + kWarp];
                  const int j = m.nat_solute + 3 * nw2;
                  nx0 = xq[j], nx1 = xq[j + 1], nx2 = xq[j + 2];
              }
              float pel = 0.f, pvdw = 0.f;
#pragma unroll
              for (int b = 0; b < 3; ++b) {
                  float4 xb = xp[b];
                  if (BOX) xb = at_image(m, xb, xa[0], xp[0]);
#pragma unroll
                  for (int a = 0; a < 3; ++a) {
                      const int kk = a * kMaxSolv + b;
                      const bool lj = a == 0 && b == 0;
                      float vel, vdw;
                      pair_f(xa[a], xb, m.wwAf[kk], m.wwBf[kk], m.wwEf[kk], lj, f[a][0], f[a][1], f[a][2], vel, vdw);
                      pel += vel;
                      if (lj) pvdw += vdw;
                  }
              }
              if (w < w2) {   // each molecule pair's energy once
                  rel += pel;
                  rvdw += pvdw;
              }
            }
          } else {
          for (int k = lane; k < n; k += kWarp) {
            int w2 = buf[k];
            int j0 = m.nat_solute + sa * w2;
            float pel = 0.f, pvdw = 0.f;
            const float4 xr = BOX ? xq[j0] : make_float4(0.f, 0.f, 0.f, 0.f);   // partner's first atom
#pragma unroll
            for (int b = 0; b < kMaxSolv; ++b) {
                if (b >= sa) break;
                float4 xb = xq[j0 + b];
                if (BOX) xb = at_image(m, xb, xa[0], xr);
#pragma unroll
                for (int a = 0; a < NA; ++a) {
                    if (a >= sa) break;
                    int kk = a * kMaxSolv + b;
                    float vel, vdw;
                    pair_f(xa[a], xb, m.wwAf[kk], m.wwBf[kk], m.wwEf[kk], true, f[a][0], f[a][1], f[a][2], vel, vdw);
                    pel += vel;
                    pvdw += vdw;
                }
            }
            if (w < w2) {   // each molecule pair's energy once
                rel += pel;
                rvdw += pvdw;
            }
          }
          }
          __syncwarp();   // this buffer is refilled two chunks later
        }
        if (nchunk == 0) {
            cp_async_wait<0>();
            __syncwarp();
        }
        for (int k = lane; k < nwg; k += kWarp) {
            int g = k < kRowChunk ? sh_wg[wib][k] : rg[k];
            const float4 xr = BOX ? xq[m.gsw[g]] : make_float4(0.f, 0.f, 0.f, 0.f);   // group's switch atom
            for (int bb = m.gslot[g]; bb < m.gslot[g + 1]; ++bb) {
                int j = m.gatom[bb];
                if (m.iqatom[j] >= 0) continue;
                float4 xb = xq[j];
                if (BOX) xb = at_image(m, xb, xa[0], xr);
                int tj = m.iac[j];
#pragma unroll
                for (int a = 0; a < NA; ++a) {
                    if (a >= sa) break;
                    bool ljw = (m.wlj_mask >> a) & 1u;
                    float4 p = ljw ? lj(tj, m.wtype[a]) : make_float4(0.f, 0.f, 0.f, 0.f);
                    float vel, vdw;
                    pair_f(xa[a], xb, p.x, p.y, xb.w * m.wcrgf[a], ljw, f[a][0], f[a][1], f[a][2], vel, vdw);
                }
            }
        }
        __syncwarp();   // sh_wg is refilled by the next row
        // row gradient and energies stored as in k_rows_solute
        float e0 = warp_sum(rel), e1 = warp_sum(rvdw);
        if (lane == 0) {
            if (e0 != 0.f) atomicAdd(s.efix + E_WW_EL, to_fix(e0));
            if (e1 != 0.f) atomicAdd(s.efix + E_WW_VDW, to_fix(e1));
        }
#pragma unroll
        for (int a = 0; a < NA; ++a) {
            if (a >= sa) break;
            float v0 = warp_sum(f[a][0]), v1 = warp_sum(f[a][1]), v2 = warp_sum(f[a][2]);
            if (lane == 0) {
                float* fr = s.frow + 3 * (i0 + a);
                fr[0] = v0;
                fr[1] = v1;
                fr[2] = v2;
            }
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

// grid for per-window work `work` (items) in blocks of bs: at most per_sm
// resident blocks per SM over all windows
dim3 grid_for(int64_t work, int bs, int per_sm, int nwin) {
    int64_t b = (work + bs - 1) / bs;
    int64_t lim = ((int64_t)sms() * per_sm + nwin - 1) / nwin;
    if (b > lim) b = lim;
    if (b < 1) b = 1;
    return dim3((unsigned)b, (unsigned)nwin);
}

}  // namespace

__global__ void k_reset_counts(const DevState* __restrict__ states, unsigned keep) {
    int k = threadIdx.x;
    if (k < C_NUM && !((keep >> k) & 1u)) states[blockIdx.x].cnt[k] = 0;
}

void launch_reset_counts(const Launch& L, unsigned keep_mask) {
    k_reset_counts<<<L.nwin, 32, 0, L.st>>>(L.ds, keep_mask);
}

void launch_pack(const Launch& L) {
    k_pack<<<dim3((L.m.natom + 255) / 256, L.nwin), 256, 0, L.st>>>(L.m, L.ds);
}
void launch_group_centres(const Launch& L) {
    k_group_centres<<<dim3((L.m.ncgp + 63) / 64, L.nwin), 64, 0, L.st>>>(L.m, L.ds);
}
void launch_build_ww(const Launch& L, const Cut& c) {
    if (L.m.nwat == 0) return;
    int half = (L.m.nwat + 1) / 2;
    k_build_ww<<<grid_for((int64_t)half * 32, 256, 8, L.nwin), 256, 0, L.st>>>(L.m, L.ds, c.rcww2);
}
void launch_build_pw(const Launch& L, const Cut& c) {
    if (L.m.nwat == 0 || L.m.ncgp_solute == 0) return;
    k_build_pw<<<grid_for((int64_t)L.m.ncgp_solute * 32, 256, 8, L.nwin), 256, 0, L.st>>>(L.m, L.ds, c.rcpw2);
}
void launch_build_pp(const Launch& L, const Cut& c) {
    if (L.m.ncgp_solute == 0) return;
    int half = (L.m.ncgp_solute + 1) / 2;
    k_build_pp_groups<<<grid_for((int64_t)half * 32, 256, 8, L.nwin), 256, 0, L.st>>>(L.m, L.ds, c.rcpp2);
    k_expand_pp<<<grid_for(L.s0.cap_ppg, 128, 8, L.nwin), 128, 0, L.st>>>(L.m, L.ds);
}
void launch_build_qw(const Launch& L, const Cut& c) {
    if (L.m.nwat == 0 || L.m.nqat == 0) return;
    k_build_qw<<<dim3(1, L.nwin), 1024, 0, L.st>>>(L.m, L.ds, c.rcq2);
}
void launch_build_qp(const Launch& L, const uint8_t* qnear, double rcq2) {
    if (L.m.ncgp_solute == 0 || L.m.nqat == 0) return;
    k_build_qp<<<dim3(1, L.nwin), 1024, 0, L.st>>>(L.m, L.ds, qnear, rcq2);
}
int launch_lrf_accumulate(const Launch& L, const Cut& c, int mixed, const int* lrf_src) {
    if (L.m.any_atom && L.m.box) {
        k_lrf_accumulate_any_box<<<grid_for((int64_t)L.m.ncgp * 32, 128, 16, L.nwin), 128, 0, L.st>>>(L.m, L.ds, c);
        return 1;
    }
    if (L.m.any_atom) {
        dim3 g = grid_for((int64_t)L.m.ncgp * 32, 128, 16, L.nwin);
        if (mixed) k_lrf_accumulate_any<true><<<g, 128, 0, L.st>>>(L.m, L.ds, c);
        else k_lrf_accumulate_any<false><<<g, 128, 0, L.st>>>(L.m, L.ds, c);
        return 1;
    }
// FP64 form: the unstaged kernel measured faster (its FP64 terms, not the
// loads, bound it, and the staged block holds more registers)
#ifndef QNB_LRF_FP64_STAGED
#define QNB_LRF_FP64_STAGED 0
#endif
#ifndef QNB_LRF_PAIR
#define QNB_LRF_PAIR 1   // mixed form: two target groups per warp (k_lrf_accumulate2)
#endif
#ifndef QNB_LRF_NBODY
#define QNB_LRF_NBODY 1  // mixed form: one thread per target group (k_lrf_nbody)
#endif
    dim3 g = grid_for((int64_t)L.m.ncgp * 32, kLrfBlock, L.tu.v[T_LRF], L.nwin);
    if (mixed && QNB_LRF_NBODY) {
        // source ranges of at least one staged tile each; the split depends on
        // the topology only, so a window's coefficients are the same in a
        // batch of any size (51 windows of a 1,400-source-group system:
        // 8 ranges, about 9 waves of resident target threads)
        const int nsplit = std::min(kLrfSplitMax, std::max(1, L.m.nlrf_groups / kLrfGT));
        dim3 g((L.m.ncgp + kLrfNB - 1) / kLrfNB, L.nwin, nsplit);
        if (L.m.box) k_lrf_nbody<true><<<g, kLrfNB, 0, L.st>>>(L.m, L.ds, c, nsplit);
        else k_lrf_nbody<false><<<g, kLrfNB, 0, L.st>>>(L.m, L.ds, c, nsplit);
        k_lrf_combine<<<dim3((L.m.ncgp + 127) / 128, L.nwin), 128, 0, L.st>>>(L.m, L.ds, nsplit);
        return 2;
    } else if (mixed && QNB_LRF_PAIR)
        k_lrf_accumulate2<<<grid_for((int64_t)L.m.ncgp * 32 / kLrfPair, kLrfBlock, L.tu.v[T_LRF], L.nwin), kLrfBlock, 0,
                            L.st>>>(L.m, L.ds, c, lrf_src);
    else if (mixed) k_lrf_accumulate<true><<<g, kLrfBlock, 0, L.st>>>(L.m, L.ds, c, lrf_src);
    else if (QNB_LRF_FP64_STAGED) k_lrf_accumulate<false><<<g, kLrfBlock, 0, L.st>>>(L.m, L.ds, c, lrf_src);
    else if (L.m.box)
        k_lrf_accumulate_direct<false, true><<<grid_for((int64_t)L.m.ncgp * 32, 128, 16, L.nwin), 128, 0, L.st>>>(
            L.m, L.ds, c, lrf_src);
    else k_lrf_accumulate_direct<false, false><<<grid_for((int64_t)L.m.ncgp * 32, 128, 16, L.nwin), 128, 0, L.st>>>(L.m, L.ds, c, lrf_src);
    return 1;
}

// cells of half the largest cut-off plus a margin far above the FP32 rounding
// of the packed positions (a few 1e-6 A)
static double cell_edge(const Cut& c) {
    double rc = std::sqrt(std::max(c.rcpp2, std::max(c.rcpw2, c.rcww2)));
    return 0.5 * (rc + std::max(0.01, 1e-4 * rc));
}
int box_cells(const DevModel& m, const Cut& c, int* n) {
    const double h = cell_edge(c);
    for (int k = 0; k < 3; ++k) n[k] = (int)std::min(1.0e6, m.boxl[k] / h);
    while ((int64_t)n[0] * n[1] * n[2] > kCellCap) {   // fewer, larger cells
        int k = n[0] >= n[1] && n[0] >= n[2] ? 0 : (n[1] >= n[2] ? 1 : 2);
        --n[k];
    }
    return n[0] >= 5 && n[1] >= 5 && n[2] >= 5;
}
int launch_build_rows(const Launch& L, const Cut& c) {
    int nrows = L.m.ncgp_solute + L.m.nwat;
    if (nrows == 0) return 0;
    dim3 g = grid_for((int64_t)nrows * 32, 128, L.tu.v[T_BUILD], L.nwin);
    if (L.m.box) {   // periodic box (switch atoms): minimum-image tests, wrapped stencil
        int n[3];
        if (!box_cells(L.m, c, n)) {   // fewer than 5 cells per edge: every unit is a candidate
            k_build_rows<false, true><<<g, 128, 0, L.st>>>(L.m, L.ds, c);
            return 1;
        }
        k_bin_cells<<<L.nwin, 1024, 0, L.st>>>(L.m, L.ds, 0.f, make_int3(n[0], n[1], n[2]));
        k_build_rows<true, true><<<g, 128, 0, L.st>>>(L.m, L.ds, c);
        return 2;
    }
    if (L.m.any_atom) {   // any-atom group tests: every group and water is a candidate
        k_build_rows<false, false><<<g, 128, 0, L.st>>>(L.m, L.ds, c);
        return 1;
    }
    k_bin_cells<<<L.nwin, 1024, 0, L.st>>>(L.m, L.ds, (float)(1.0 / cell_edge(c)), make_int3(0, 0, 0));
    k_build_rows<true, false><<<g, 128, 0, L.st>>>(L.m, L.ds, c);
    return 2;
}
int lj_smem(const DevModel& m) {
    return m.natyps <= kMaxTypesShared ? (int)(m.natyps * m.natyps * sizeof(float4)) : 0;
}
void launch_rows_solute(const Launch& L, int maxg) {
    if (L.m.ncgp_solute == 0) return;
    dim3 g = grid_for((int64_t)L.m.ncgp_solute * 32, 128, L.tu.v[T_ROWS_SOLUTE], L.nwin);
    int sm = lj_smem(L.m);
#define RS(MG, GE, BX) k_rows_solute<MG, GE, BX><<<g, 128, sm, L.st>>>(L.m, L.ds)
#define RSB(MG, GE) do { if (L.m.box) RS(MG, GE, true); else RS(MG, GE, false); } while (0)
    if (L.m.geom) {
        if (maxg <= 4) RSB(4, true); else if (maxg <= 6) RSB(6, true); else if (maxg <= 8) RSB(8, true); else RSB(16, true);
    } else {
        if (maxg <= 4) RSB(4, false); else if (maxg <= 6) RSB(6, false); else if (maxg <= 8) RSB(8, false);
        else RSB(16, false);
    }
#undef RSB
#undef RS
}
void launch_solvent_internal(const Launch& L, const int2* ij, const double* par, int n, int mixed) {
    if (L.m.nwat == 0 || n == 0) return;
    dim3 g = grid_for(L.m.nwat, 64, 8, L.nwin);   // FP64 work: small blocks over all SMs
    if (mixed) k_solvent_internal<true><<<g, 64, 0, L.st>>>(L.m, L.ds, ij, par, n);
    else k_solvent_internal<false><<<g, 64, 0, L.st>>>(L.m, L.ds, ij, par, n);
}
void launch_rows_water(const Launch& L) {
    if (L.m.nwat == 0) return;
    dim3 g = grid_for((int64_t)L.m.nwat * 32, 128, L.tu.v[T_ROWS_WATER], L.nwin);
    int sm = lj_smem(L.m);
    const bool spc = L.m.spc && L.m.sa == 3;   // the SPC rows assume 3-atom molecules
    if (L.m.box) {
        if (spc) k_rows_water<true, true><<<g, 128, sm, L.st>>>(L.m, L.ds);
        else k_rows_water<false, true><<<g, 128, sm, L.st>>>(L.m, L.ds);
    } else if (spc) k_rows_water<true, false><<<g, 128, sm, L.st>>>(L.m, L.ds);
    else k_rows_water<false, false><<<g, 128, sm, L.st>>>(L.m, L.ds);
}
void launch_ww(const Launch& L, int mixed) {
    if (L.m.nwat == 0) return;
    dim3 g = grid_for(L.s0.cap_ww, 256, 8, L.nwin);
    bool spc = L.m.spc != 0;
    if (mixed) { if (spc) k_ww<true, true><<<g, 256, 0, L.st>>>(L.m, L.ds); else k_ww<true, false><<<g, 256, 0, L.st>>>(L.m, L.ds); }
    else { if (spc) k_ww<false, true><<<g, 256, 0, L.st>>>(L.m, L.ds); else k_ww<false, false><<<g, 256, 0, L.st>>>(L.m, L.ds); }
}
#ifndef QNB_Q_LANES
#define QNB_Q_LANES 1   // mixed form: k_qenv_lanes (1) or k_qenv (0)
#endif
template <bool WATER>
void launch_qenv(const Launch& L, int mixed, dim3 g) {
    bool spc = L.m.spc != 0;
    bool s4 = L.m.S <= 4;
#define QL(MIX, SPC, SM) k_qenv<MIX, SPC, WATER, SM><<<g, kQBlock, 0, L.st>>>(L.m, L.ds, L.tu.v[T_QCHUNK])
#define QT(SPC, SM) k_qenv_lanes<SPC, WATER, SM><<<g, kQBlock, 0, L.st>>>(L.m, L.ds)
    if (mixed && QNB_Q_LANES) {
        if (spc) { if (s4) QT(true, 4); else QT(true, kMaxStates); }
        else { if (s4) QT(false, 4); else QT(false, kMaxStates); }
    } else if (mixed) {
        if (spc) { if (s4) QL(true, true, 4); else QL(true, true, kMaxStates); }
        else { if (s4) QL(true, false, 4); else QL(true, false, kMaxStates); }
    } else {
        if (spc) { if (s4) QL(false, true, 4); else QL(false, true, kMaxStates); }
        else { if (s4) QL(false, false, 4); else QL(false, false, kMaxStates); }
    }
#undef QL
#undef QT
}
void launch_qw(const Launch& L, int mixed) {
    if (L.m.nwat == 0 || L.m.nqat == 0) return;
    launch_qenv<true>(L, mixed, grid_for(L.s0.cap_qw * 32, kQBlock, L.tu.v[T_QW], L.nwin));
}
void launch_pw(const Launch& L, int mixed) {
    if (L.m.nwat == 0 || L.m.ncgp_solute == 0) return;
    dim3 g = grid_for(L.s0.cap_pw, 256, 8, L.nwin);
    if (mixed) k_pw<true><<<g, 256, 0, L.st>>>(L.m, L.ds); else k_pw<false><<<g, 256, 0, L.st>>>(L.m, L.ds);
}
void launch_pp(const Launch& L, int mixed) {
    if (L.m.ncgp_solute == 0) return;
    dim3 g = grid_for(L.s0.cap_pp, 256, 8, L.nwin);
    if (mixed) k_pp<true><<<g, 256, 0, L.st>>>(L.m, L.ds); else k_pp<false><<<g, 256, 0, L.st>>>(L.m, L.ds);
}
void launch_qp(const Launch& L, int mixed) {
    if (L.m.nqat == 0 || L.m.nat_solute == 0) return;
    launch_qenv<false>(L, mixed, grid_for(L.s0.cap_qp * 32, kQBlock, L.tu.v[T_QP], L.nwin));
}
void launch_nonbond_qq(const Launch& L, int mixed) {
    if (L.s0.nqq == 0) return;
    dim3 g((L.s0.nqq + 255) / 256, L.nwin);
    if (mixed) k_qq<true><<<g, 256, 0, L.st>>>(L.m, L.ds); else k_qq<false><<<g, 256, 0, L.st>>>(L.m, L.ds);
}
void launch_lrf_taylor(const Launch& L, const int* iwhich, int mixed) {
    dim3 g = grid_for(L.m.natom, 64, L.tu.v[T_TAYLOR], L.nwin);
    if (mixed) k_lrf_taylor<true><<<g, 64, 0, L.st>>>(L.m, L.ds, iwhich);
    else k_lrf_taylor<false><<<g, 64, 0, L.st>>>(L.m, L.ds, iwhich);
}
void launch_apply_fixed(const Launch& L, int rows, int qenv) {
    int n = 3 * L.m.natom;
    k_apply_fixed<<<grid_for(n, 256, 16, L.nwin), 256, 0, L.st>>>(n, L.ds, rows, qenv);
}
__global__ void k_clear_fq(int n, const DevState* __restrict__ states) {
    float* __restrict__ fq = states[blockIdx.y].fq;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) fq[k] = 0.f;
}
void launch_clear_fq(const Launch& L) {
    int n = 3 * L.m.natom;
    k_clear_fq<<<grid_for(n, 256, 4, L.nwin), 256, 0, L.st>>>(n, L.ds);
}
// =============================================================================
// Bonded terms: FP64 in the plain form; FP32 arithmetic in the mixed form
// (the reference's single-precision build, QREAL_EPS 1e-5), fixed-point sums
// =============================================================================
template <typename T>
struct V3 {
    T x, y, z;
};
template <typename T>
__device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return V3<T>{a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
__device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return V3<T>{a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T>
__device__ __forceinline__ V3<T> operator-(V3<T> a) { return V3<T>{-a.x, -a.y, -a.z}; }
template <typename T>
__device__ __forceinline__ V3<T> operator*(V3<T> a, T f) { return V3<T>{a.x * f, a.y * f, a.z * f}; }
template <typename T>
__device__ __forceinline__ V3<T> operator/(V3<T> a, T f) { return V3<T>{a.x / f, a.y / f, a.z / f}; }
template <typename T>
__device__ __forceinline__ T vdot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T>
__device__ __forceinline__ V3<T> vcross(V3<T> a, V3<T> b) {
    return V3<T>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// QREAL_EPS of the reference's double- and single-precision builds
template <typename T>
__device__ __forceinline__ constexpr T qreal_eps() { return std::is_same<T, float>::value ? T(1e-5) : T(1e-10); }
constexpr double kPi = 3.14159265358979323846;   // 4 atan(1)

// atom position: FP64 coordinates, or the mixed form's centred FP32 copy
template <bool MIX>
__device__ __forceinline__ V3<typename std::conditional<MIX, float, double>::type> atom_pos(const DevState& s, int i) {
    if constexpr (MIX) {
        float4 q = s.xq[i];
        return V3<float>{q.x, q.y, q.z};
    } else {
        return V3<double>{s.x[3 * i], s.x[3 * i + 1], s.x[3 * i + 2]};
    }
}

// angle_calc, src/bonded.f90:78-118
template <typename T>
struct AngleVal {
    T angl;
    V3<T> a, b, c;
};
template <typename T>
__device__ AngleVal<T> angle_calc(V3<T> a, V3<T> b, V3<T> c) {
    V3<T> ab = a - b, bc = c - b;
    T ab2 = T(1) / vdot(ab, ab), bc2 = T(1) / vdot(bc, bc);
    T abd = sqrt(ab2), bcd = sqrt(bc2);
    T scalar = vdot(ab, bc) * abd * bcd;
    scalar = fmin(T(1), fmax(T(-1), scalar));
    AngleVal<T> r;
    r.angl = acos(scalar);
    T inv = sin(r.angl);
    if (fabs(inv) < qreal_eps<T>()) inv = qreal_eps<T>();
    inv = T(-1) / inv;
    V3<T> af = ((bc * abd * bcd) - (ab * (ab2 * scalar))) * inv;
    V3<T> cf = ((ab * abd * bcd) - (bc * (bc2 * scalar))) * inv;
    r.a = af;
    r.b = af + cf;
    r.c = cf;
    return r;
}

// torsion_calc / improper_calc (identical), src/bonded.f90:151-320
template <typename T>
struct TorsVal {
    T angl;
    V3<T> a, b, c, d;
};
template <typename T>
__device__ TorsVal<T> torsion_calc(V3<T> a, V3<T> b, V3<T> c, V3<T> d) {
    V3<T> ab = a - b, bc = c - b, cd = d - c;
    V3<T> cabc = vcross(ab, bc), cbcd = vcross(-bc, cd);
    T a2abc = vdot(cabc, cabc), a2bcd = vdot(cbcd, cbcd);
    T aabc = sqrt(a2abc), abcd = sqrt(a2bcd);
    T scalar = vdot(cabc, cbcd) / (aabc * abcd);
    scalar = fmin(T(1), fmax(T(-1), scalar));
    TorsVal<T> r;
    r.angl = acos(scalar);
    if (vdot(bc, vcross(cabc, cbcd)) < T(0)) r.angl = -r.angl;
    T inv = sin(r.angl);
    if (fabs(inv) < qreal_eps<T>()) inv = qreal_eps<T>();
    inv = T(-1) / inv;
    V3<T> v1 = ((cbcd / (aabc * abcd)) - ((cabc / a2abc) * scalar)) * inv;
    V3<T> v2 = ((cabc / (aabc * abcd)) - ((cbcd / a2bcd) * scalar)) * inv;
    V3<T> ca = ab - bc, db = -bc - cd;
    r.a = vcross(bc, v1);
    r.b = vcross(ca, v1) + vcross(cd, v2);
    r.c = vcross(db, v2) - vcross(ab, v1);
    r.d = vcross(bc, v2);
    return r;
}

constexpr int kBondedSlots = 8 + 4 * kMaxStates;   // E_B0 .. qb_slot(kMaxStates - 1, 3)
constexpr int kBondedBlock = 128;

template <bool MIX>
struct BondedSink {
    typedef typename std::conditional<MIX, float, double>::type T;
    typedef typename std::conditional<MIX, unsigned long long, double>::type ET;
    Acc<MIX> acc;
    ET* red;   // shared per-block energy sums, slot - E_B0
    __device__ __forceinline__ void grad(int i, V3<T> g) const {
        if constexpr (MIX) acc.grad_alu(i, g.x, g.y, g.z);
        else acc.grad(i, g.x, g.y, g.z);
    }
    __device__ __forceinline__ void energy(int slot, T e) const {
        if constexpr (MIX) atomicAdd(red + (slot - E_B0), to_fix_alu(e));
        else atomicAdd(red + (slot - E_B0), e);
    }
};

// A Q term's Morse coupling in state st (qbond's EMorseD and dMorse,
// src/bondene.f90:530-548): gamma and the bond's gradient direction
// dMorse_i (dMorse_j = -dMorse_i); gamma 1 and no gradient when uncoupled,
// when the bond is absent in the state or shorter than r0.
template <typename T>
struct Coupling {
    int i = -1, j = -1;
    T gamma = T(1);
    V3<T> dmi{T(0), T(0), T(0)};
};
template <typename T, typename PF>
__device__ __forceinline__ Coupling<T> morse_coupling(const BondedDev& b, int cpl, int st, int S, T lam, PF P) {
    Coupling<T> c;
    if (cpl < 0) return c;
    const int ib = cpl & 0x3fffffff, brk = cpl >> 30;
    const int code = b.qbond_code[ib * S + st];
    T emd = T(1);
    if (code >= 0) {
        int2 e = b.qbonds[ib];
        double4_16a lib = b.qbondlib[code];
        const T amz = (T)lib.y, r0 = (T)lib.z;
        V3<T> av = P(e.y) - P(e.x);
        T dist = sqrt(vdot(av, av));
        T db = dist - r0;
        if (db > T(0)) {
            T fexp = exp(-amz * db);
            emd = -(fexp * fexp - T(2) * fexp);
            c.dmi = av * (T(2) * amz * (fexp - fexp * fexp) * lam / dist);
            c.i = e.x;
            c.j = e.y;
        }
    }
    c.gamma = brk ? T(1) - emd : emd;
    return c;
}

// One thread per term: classical bonds, angles (+ Urey-Bradley), torsions,
// impropers; then Q bonds, angles, torsions, impropers per state.  Energies
// are summed per block in shared memory and added once per block and slot.
template <bool MIX>
__global__ void __launch_bounds__(kBondedBlock) k_bonded(DevModel m, const DevState* __restrict__ states, BondedDev b) {
    typedef typename std::conditional<MIX, float, double>::type T;
    typedef typename BondedSink<MIX>::ET ET;
    __shared__ ET red[kBondedSlots];
    const DevState& s = states[blockIdx.y];
    for (int k = threadIdx.x; k < kBondedSlots; k += blockDim.x) red[k] = ET(0);
    __syncthreads();
    const BondedSink<MIX> out{make_acc<MIX>(s), red};
    const int S = m.S;
    const T two_pi = T(2.0 * kPi);
    auto lam = [&](int st) -> T {
        if constexpr (MIX) return s.lambdaf[st];
        else return s.lambda[st];
    };
    auto P = [&](int i) { return atom_pos<MIX>(s, i); };
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < b.nterms; t += gridDim.x * blockDim.x) {
        int u = t;
        if (u < b.nb) {   // bond, src/bondene.f90:182-245
            int4 e = b.bonds[u];
            if (e.z < 0) continue;
            double2 lib = b.bondlib[e.z];
            const T fk = (T)lib.x, b0 = (T)lib.y;
            V3<T> av = P(e.y) - P(e.x);
            T dist = sqrt(vdot(av, av));
            T db = dist - b0;
            out.energy(E_B0 + (u < b.nb_sol ? 0 : 4), T(0.5) * fk * db * db);
            T dv = fk * db / dist;
            out.grad(e.x, -(av * dv));
            out.grad(e.y, av * dv);
            continue;
        }
        u -= b.nb;
        if (u < b.na) {   // angle, src/bondene.f90:41-113 (+ urey_bradley 115-180)
            int4 e = b.angles[u];
            if (e.w < 0) continue;
            double4_16a lib = b.anglib[e.w];
            const T fk = (T)lib.x, th0 = (T)lib.y, ufk = (T)lib.z, ur0 = (T)lib.w;
            const int slot = E_B0 + (u < b.na_sol ? 1 : 5);
            AngleVal<T> c = angle_calc(P(e.x), P(e.y), P(e.z));
            T da = c.angl - th0;
            T ea = T(0.5) * fk * da * da;
            T dv = fk * da;
            out.grad(e.x, c.a * dv);
            out.grad(e.y, -(c.b * dv));
            out.grad(e.z, c.c * dv);
            if (b.urey && ufk > T(0)) {
                // the reference's solute/solvent Urey-Bradley adds the gradient
                // with these signs (d(k) -= a du, d(i) += a du)
                V3<T> av = P(e.z) - P(e.x);
                T dist = sqrt(vdot(av, av));
                T ru = dist - ur0;
                ea += ufk * ru * ru;
                T du = T(2) * ufk * ru / dist;
                out.grad(e.z, -(av * du));
                out.grad(e.x, av * du);
            }
            out.energy(slot, ea);
            continue;
        }
        u -= b.na;
        if (u < b.nt) {   // torsion, src/bondene.f90:689-762
            const int* e = b.tors + 5 * u;
            if (e[4] < 0) continue;
            double4_16a lib = b.torlib[e[4]];
            const T fk = (T)lib.x, rm = (T)lib.y, dl = (T)lib.z, ip = (T)lib.w;
            TorsVal<T> c = torsion_calc(P(e[0]), P(e[1]), P(e[2]), P(e[3]));
            T arg = rm * c.angl - dl;
            out.energy(E_B0 + (u < b.nt_sol ? 2 : 6), fk * (T(1) + cos(arg)) * ip);
            T dv = -rm * fk * sin(arg) * ip;
            out.grad(e[0], c.a * dv);
            out.grad(e[1], c.b * dv);
            out.grad(e[2], c.c * dv);
            out.grad(e[3], c.d * dv);
            continue;
        }
        u -= b.nt;
        if (u < b.ni) {   // improper (harmonic) / improper2 (periodic), src/bondene.f90:247-385
            const int* e = b.imps + 5 * u;
            if (e[4] < 0) continue;
            double2 lib = b.implib[e[4]];
            const T fk = (T)lib.x, p0 = (T)lib.y;
            TorsVal<T> c = torsion_calc(P(e[0]), P(e[1]), P(e[2]), P(e[3]));
            T ei, dv;
            if (b.imp_type == 2) {
                T arg = T(2) * c.angl - p0;
                ei = fk * (T(1) + cos(arg));
                dv = T(-2) * fk * sin(arg);
            } else {
                T arg = c.angl - p0;
                arg = arg - two_pi * round(arg / two_pi);
                dv = fk * arg;
                ei = T(0.5) * dv * arg;
            }
            out.energy(E_B0 + (u < b.ni_sol ? 3 : 7), ei);
            out.grad(e[0], c.a * dv);
            out.grad(e[1], c.b * dv);
            out.grad(e[2], c.c * dv);
            out.grad(e[3], c.d * dv);
            continue;
        }
        u -= b.ni;
        // Q terms: index = term * S + state
        if (u < b.nqb * S) {   // qbond, src/bondene.f90:506-553
            const int q = u / S, st = u % S, code = b.qbond_code[u];
            if (code < 0) continue;
            int2 e = b.qbonds[q];
            double4_16a lib = b.qbondlib[code];   // Dmz amz r0 fk
            const T Dmz = (T)lib.x, amz = (T)lib.y, r0 = (T)lib.z, fk = (T)lib.w;
            V3<T> av = P(e.y) - P(e.x);
            T dist = sqrt(vdot(av, av));
            T db = dist - r0;
            T fexp = exp(-amz * db);
            out.energy(qb_slot(st, 0), Dmz * (fexp * fexp - T(2) * fexp) + T(0.5) * fk * db * db);
            T dv = (T(2) * Dmz * amz * (fexp - fexp * fexp) + fk * db) * lam(st) / dist;
            out.grad(e.x, -(av * dv));
            out.grad(e.y, av * dv);
            continue;
        }
        u -= b.nqb * S;
        if (u < b.nqa * S) {   // qangle (+ qurey_bradley), src/bondene.f90:387-504
            const int q = u / S, st = u % S, code = b.qangle_code[u];
            if (code < 0) continue;
            int4 e = b.qangles[q];
            double4_16a lib = b.qanglib[code];
            const T fk = (T)lib.x, th0 = (T)lib.y, ufk = (T)lib.z, ur0 = (T)lib.w;
            const T l = lam(st);
            const auto cp = morse_coupling<T>(b, b.qang_cpl[q], st, S, l, P);
            AngleVal<T> c = angle_calc(P(e.x), P(e.y), P(e.z));
            T da = c.angl - th0;
            T ea = T(0.5) * fk * da * da;   // the unscaled energy drives the coupled bond
            T dv = cp.gamma * fk * da * l;
            out.grad(e.x, c.a * dv);
            out.grad(e.y, -(c.b * dv));
            out.grad(e.z, c.c * dv);
            if (b.urey && ufk != T(0)) {
                V3<T> av = P(e.z) - P(e.x);
                T dist = sqrt(vdot(av, av));
                T ru = dist - ur0;
                ea += ufk * ru * ru;
                T du = cp.gamma * T(2) * (ufk * ru / dist) * l;
                out.grad(e.x, -(av * du));
                out.grad(e.z, av * du);
            }
            out.energy(qb_slot(st, 1), ea * cp.gamma);
            if (cp.i >= 0) {
                out.grad(cp.i, cp.dmi * ea);
                out.grad(cp.j, -(cp.dmi * ea));
            }
            continue;
        }
        u -= b.nqa * S;
        if (u < b.nqt * S) {   // qtorsion, src/bondene.f90:624-688
            const int q = u / S, st = u % S, code = b.qtor_code[u];
            if (code < 0) continue;
            int4 e = b.qtors[q];
            double4_16a lib = b.qtorlib[code];
            const T fk = (T)lib.x, rm = (T)lib.y, dl = (T)lib.z;
            const auto cp = morse_coupling<T>(b, b.qtor_cpl[q], st, S, lam(st), P);
            TorsVal<T> c = torsion_calc(P(e.x), P(e.y), P(e.z), P(e.w));
            T arg = rm * c.angl - dl;
            T pe = fk * (T(1) + cos(arg));
            out.energy(qb_slot(st, 2), pe * cp.gamma);
            T dv = -rm * fk * sin(arg) * cp.gamma * lam(st);
            out.grad(e.x, c.a * dv);
            out.grad(e.y, c.b * dv);
            out.grad(e.z, c.c * dv);
            out.grad(e.w, c.d * dv);
            if (cp.i >= 0) {
                out.grad(cp.i, cp.dmi * pe);
                out.grad(cp.j, -(cp.dmi * pe));
            }
            continue;
        }
        u -= b.nqt * S;
        if (u < b.nqi * S) {   // qimproper (harmonic), src/bondene.f90:555-622
            const int q = u / S, st = u % S, code = b.qimp_code[u];
            if (code < 0) continue;
            int4 e = b.qimps[q];
            double2 lib = b.qimplib[code];
            const T fk = (T)lib.x, p0 = (T)lib.y;
            const auto cp = morse_coupling<T>(b, b.qimp_cpl[q], st, S, lam(st), P);
            TorsVal<T> c = torsion_calc(P(e.x), P(e.y), P(e.z), P(e.w));
            T arg = c.angl - p0;
            arg = arg - two_pi * round(arg / two_pi);
            T dv = fk * arg;
            T pe = T(0.5) * dv * arg;
            out.energy(qb_slot(st, 3), pe * cp.gamma);
            dv = dv * cp.gamma * lam(st);
            out.grad(e.x, c.a * dv);
            out.grad(e.y, c.b * dv);
            out.grad(e.z, c.c * dv);
            out.grad(e.w, c.d * dv);
            if (cp.i >= 0) {
                out.grad(cp.i, cp.dmi * pe);
                out.grad(cp.j, -(cp.dmi * pe));
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kBondedSlots; k += blockDim.x) {
        ET v = red[k];
        if (v != ET(0)) {
            if constexpr (MIX) out.acc.energy_fix(E_B0 + k, v);
            else out.acc.energy(E_B0 + k, v);
        }
    }
}

void launch_bonded(const Launch& L, const BondedDev& b, int mixed) {
    if (b.nterms == 0) return;
    int blocks = std::min(512, (b.nterms + kBondedBlock - 1) / kBondedBlock);
    dim3 g(blocks, L.nwin);
    if (mixed) k_bonded<true><<<g, kBondedBlock, 0, L.st>>>(L.m, L.ds, b);
    else k_bonded<false><<<g, kBondedBlock, 0, L.st>>>(L.m, L.ds, b);
}

// fix_shell, src/potene.f90:386-423: excluded atoms (fk_fix) and shell atoms
// (fk_pshell) restrained to their topology positions, FP64 in both forms
// With freeze (excluded_freeze) an excluded atom is put back to xtop, its
// velocity (v, the window's MD velocities, or null) zeroed, and its force
// constant is zero (src/potene.f90:401-405).
template <bool MIX>
__global__ void k_fix_shell(DevModel m, const DevState* __restrict__ states, const uint8_t* __restrict__ flags,
                            const double* __restrict__ xtop, double fk_fix, double fk_pshell, int freeze,
                            double* __restrict__ v) {
    const DevState& s = states[blockIdx.y];
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> efix, eshell;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < m.natom; i += gridDim.x * blockDim.x) {
        const unsigned f = flags[i];
        if (!f) continue;
        if (freeze && (f & 1u)) {
            for (int c = 0; c < 3; ++c) {
                s.x[3 * i + c] = xtop[3 * i + c];
                if (v) v[((size_t)blockIdx.y * m.natom + i) * 3 + c] = 0.0;
            }
            continue;
        }
        const double fk = (f & 1u) ? fk_fix : fk_pshell;
        double vx = s.x[3 * i] - xtop[3 * i], vy = s.x[3 * i + 1] - xtop[3 * i + 1], vz = s.x[3 * i + 2] - xtop[3 * i + 2];
        double erst = 0.5 * fk * (vx * vx + vy * vy + vz * vz);
        if (f & 1u) efix.add(erst);
        if (f & 2u) eshell.add(erst);
        if constexpr (MIX) acc.gradd(i, vx * fk, vy * fk, vz * fk);
        else acc.grad(i, vx * fk, vy * fk, vz * fk);
    }
    efix.flush(acc, E_RST_FIX);
    eshell.flush(acc, E_RST_SHELL);
}
void launch_fix_shell(const Launch& L, const uint8_t* flags, const double* xtop, double fk_fix, double fk_pshell,
                      int mixed, int freeze, double* v) {
    dim3 g = grid_for(L.m.natom, 64, 8, L.nwin);
    if (mixed) k_fix_shell<true><<<g, 64, 0, L.st>>>(L.m, L.ds, flags, xtop, fk_fix, fk_pshell, freeze, v);
    else k_fix_shell<false><<<g, 64, 0, L.st>>>(L.m, L.ds, flags, xtop, fk_fix, fk_pshell, freeze, v);
}
// offdiag, src/nonbondene.f90:6238-6260: the EVB couplings
// Hij = A exp(-mu r_kl) of Q-atom pairs, FP64 in both forms
__global__ void k_offdiag(const DevState* __restrict__ states, OffdDev o) {
    const int w = blockIdx.y;
    const double* __restrict__ x = states[w].x;
    for (int io = blockIdx.x * blockDim.x + threadIdx.x; io < o.n; io += gridDim.x * blockDim.x) {
        int2 kl = o.kl[io];
        double dx = x[3 * kl.y] - x[3 * kl.x], dy = x[3 * kl.y + 1] - x[3 * kl.x + 1],
               dz = x[3 * kl.y + 2] - x[3 * kl.x + 2];
        double r = sqrt(dx * dx + dy * dy + dz * dz);
        double2 am = o.Amu[io];
        o.out[((size_t)w * o.n + io) * 2] = am.x * exp(-am.y * r);
        o.out[((size_t)w * o.n + io) * 2 + 1] = r;
    }
}
void launch_offdiag(const Launch& L, const OffdDev& o) {
    if (o.n == 0) return;
    k_offdiag<<<dim3((o.n + 63) / 64, L.nwin), 64, 0, L.st>>>(L.ds, o);
}
// Listed pair energies with nbe_qq's arithmetic (src/nonbonded.f90:111-150;
// nbe_qx, 200-222, is the same without the soft-pair branch): the energies of
// monitor group pairs (nonbond_monitor, src/nonbondene.f90:4636-4680) and the
// excluded interactions of group contributions (calculate_exc, 6825-6920).
// FP64 in both forms; one block per (slot, window) sums its entries in a
// fixed order, so the sums do not depend on the launch.
constexpr int kPairSetBlock = 128;
__global__ void __launch_bounds__(kPairSetBlock) k_pair_sets(const DevState* __restrict__ states, PairSetDev p) {
    __shared__ double red[2][kPairSetBlock];
    const int k = blockIdx.x, w = blockIdx.y;
    const double* __restrict__ x = states[w].x;
    double vel = 0.0, vlj = 0.0;
    for (int q = p.slot_first[k] + threadIdx.x; q < p.slot_first[k + 1]; q += kPairSetBlock) {
        PairSetEntry e = p.e[q];
        double tx = x[3 * e.j] - x[3 * e.i], ty = x[3 * e.j + 1] - x[3 * e.i + 1], tz = x[3 * e.j + 2] - x[3 * e.i + 2];
        double r2 = 1.0 / (tx * tx + ty * ty + tz * tz);
        double r = sqrt(r2);
        vel += e.el * r;
        if (e.soft) {
            vlj += e.A * exp(-e.B / r);
        } else {
            double r6 = 1.0 / (1.0 / (r2 * r2 * r2) + e.sc);
            vlj += e.A * r6 * r6 - e.B * r6;
        }
    }
    red[0][threadIdx.x] = vel;
    red[1][threadIdx.x] = vlj;
    __syncthreads();
    for (int h = kPairSetBlock / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            red[0][threadIdx.x] += red[0][threadIdx.x + h];
            red[1][threadIdx.x] += red[1][threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        p.out[((size_t)w * p.nslots + k) * 2] = red[0][0];
        p.out[((size_t)w * p.nslots + k) * 2 + 1] = red[1][0];
    }
}
void launch_pair_sets(const Launch& L, const PairSetDev& p) {
    if (p.nslots == 0) return;
    k_pair_sets<<<dim3(p.nslots, L.nwin), kPairSetBlock, 0, L.st>>>(L.ds, p);
}

// -----------------------------------------------------------------------------
// Periodic box (use_PBC).  Every interaction is between two units (solute
// charge group, water molecule, the Q region around qswitch) and uses one
// lattice shift per unit pair, boxlength * nint((x_a - x_b) / boxlength) of
// the units' reference atoms (q_nint, src/math.f90:566-574); the partner atom
// is taken at x_j + shift.  The list decisions are FP64 in both forms; the
// FP64 form computes the pairs in FP64, the mixed form in FP32 from the
// packed coordinates with an FP32 shift (fixed-point sums), as its sphere
// kernels do.
// -----------------------------------------------------------------------------
// (the mixed form's lattice shift box_shift_f is defined with the Q kernels)
struct BoxPairF {
    float tx, ty, tz, r2, r;
};
__device__ __forceinline__ BoxPairF box_pair_f(float4 a, float4 b, float3 sh) {
    BoxPairF p;
    p.tx = sh.x - (a.x - b.x);
    p.ty = sh.y - (a.y - b.y);
    p.tz = sh.z - (a.z - b.z);
    p.r = rsqrtf(p.tx * p.tx + p.ty * p.ty + p.tz * p.tz);
    p.r2 = p.r * p.r;
    return p;
}
template <bool MIX>
__device__ __forceinline__ void box_grad(const Acc<MIX>& acc, int i, double gx, double gy, double gz) {
    if constexpr (MIX) acc.gradd(i, gx, gy, gz);
    else acc.grad(i, gx, gy, gz);
}
// one shifted pair: vec = shift - (x_i - x_j) (q_dist2(x(i)-x(j), shift))
struct BoxPair {
    double tx, ty, tz, r2, r;
};
__device__ __forceinline__ BoxPair box_pair(const double* __restrict__ x, int i, int j, double sx, double sy,
                                            double sz) {
    BoxPair p;
    p.tx = sx - (x[3 * i] - x[3 * j]);
    p.ty = sy - (x[3 * i + 1] - x[3 * j + 1]);
    p.tz = sz - (x[3 * i + 2] - x[3 * j + 2]);
    p.r2 = 1.0 / (p.tx * p.tx + p.ty * p.ty + p.tz * p.tz);
    p.r = sqrt(p.r2);
    return p;
}

// nbpplist_box, src/nonbondene.f90:1643-1775: solute group pairs whose switch
// atoms are within Rcpp in the minimum image (each pair once, a group with
// itself always); nbpwlist_box, 2730-2841: switch atom to the water's first
// atom; nbwwlist_box, 4174-4273: first atoms of two waters.  The pair sets
// are the reference's; the order inside a list is not.
__global__ void k_build_box_groups(DevModel m, const DevState* __restrict__ states, double rcpp2, double rcpw2,
                                   double rcww2) {
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    const int G = m.ncgp_solute, W = m.nwat;
    const int64_t npp = (int64_t)G * (G + 1) / 2, npw = (int64_t)G * W, nww = (int64_t)W * (W - 1) / 2;
    const int64_t total = npp + npw + nww;
    for (int64_t t0 = (int64_t)blockIdx.x * blockDim.x; t0 < total; t0 += (int64_t)gridDim.x * blockDim.x) {
        int64_t t = t0 + threadIdx.x;
        int kind = -1, a = 0, b = 0;
        if (t < npp) {   // (g1, g2), g1 <= g2, row-major over the upper triangle
            // t = g1*(g1+1)/2 + g2 with g2 <= g1
            int g1 = (int)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
            while ((int64_t)(g1 + 1) * (g1 + 2) / 2 <= t) ++g1;
            while ((int64_t)g1 * (g1 + 1) / 2 > t) --g1;
            int g2 = (int)(t - (int64_t)g1 * (g1 + 1) / 2);
            a = g2;
            b = g1;
            bool ok = (a == b);
            if (!ok && m.any_atom) {   // nbpplis2_box, src/nonbondene.f90:1091-1218: any atom pair
                for (int p = m.gslot[a]; p < m.gslot[a + 1] && !ok; ++p)
                    for (int q = m.gslot[b]; q < m.gslot[b + 1] && !ok; ++q)
                        ok = box_d2(m, x, m.gatom[p], m.gatom[q]) <= rcpp2;
            } else if (!ok) {
                ok = box_d2(m, x, m.gsw[a], m.gsw[b]) <= rcpp2;
            }
            kind = ok ? 0 : -1;
        } else if (t < npp + npw) {
            int64_t u = t - npp;
            a = (int)(u / W);
            b = (int)(u % W);
            const int o = m.nat_solute + m.sa * b;
            bool ok = false;
            if (m.any_atom) {   // nbpwlis2_box, src/nonbondene.f90:2247-2357: any atom of the group
                for (int p = m.gslot[a]; p < m.gslot[a + 1] && !ok; ++p) ok = box_d2(m, x, m.gatom[p], o) <= rcpw2;
            } else {
                ok = box_d2(m, x, m.gsw[a], o) <= rcpw2;
            }
            kind = ok ? 1 : -1;
        } else if (t < total) {
            int64_t u = t - npp - npw;   // (i, j), i < j over the strict upper triangle
            int j = (int)((sqrt(8.0 * (double)u + 1.0) + 1.0) * 0.5);
            while ((int64_t)j * (j - 1) / 2 > u) --j;
            while ((int64_t)(j + 1) * j / 2 <= u) ++j;
            int i = (int)(u - (int64_t)j * (j - 1) / 2);
            a = i;
            b = j;
            bool ok = box_d2(m, x, m.nat_solute + m.sa * a, m.nat_solute + m.sa * b) <= rcww2;
            kind = ok ? 2 : -1;
        }
        // one append per kind and warp
        for (int k = 0; k < 3; ++k) {
            bool mine = kind == k;
            int npairs = 0;
            if (mine && k == 1) {
                for (int q = m.gslot[a]; q < m.gslot[a + 1]; ++q) npairs += (m.iqatom[m.gatom[q]] < 0);
                if (npairs == 0) mine = false;
            }
            if (!__any_sync(0xffffffffu, mine)) continue;
            if (k == 0) {
                int pos = warp_append(s.cnt + C_PPG, mine ? 1 : 0);
                if (mine && pos < s.cap_ppg) s.ppg[pos] = make_int2(a, b);
            } else if (k == 1) {
                int pos = warp_append(s.cnt + C_PW, mine ? npairs : 0);
                if (mine)
                    for (int q = m.gslot[a]; q < m.gslot[a + 1]; ++q) {
                        int i = m.gatom[q];
                        if (m.iqatom[i] >= 0) continue;
                        if (pos < s.cap_pw) s.pw[pos] = make_int2(i, b);
                        ++pos;
                    }
            } else {
                int pos = warp_append(s.cnt + C_WW, mine ? 1 : 0);
                if (mine && pos < s.cap_ww) s.ww[pos] = make_int2(a, b);
            }
        }
    }
}

// nbqplist_box / nbqplis2_box, src/nonbondene.f90:3747-3860, 3525-3644: solute
// groups with any atom within Rcq of qswitch in the minimum image; their
// atoms not bonded/angled to a Q atom.  nbqwlist_box, 3949-4026: waters whose
// first atom is within Rcq of qswitch.  One block per window, appends in order.
__global__ void __launch_bounds__(1024) k_build_box_q(DevModel m, const DevState* __restrict__ states,
                                                      const uint8_t* __restrict__ qnear, double rcq2) {
    const DevState& s = states[blockIdx.y];
    const double* __restrict__ x = s.x;
    int base = 0;
    for (int g0 = 0; g0 < m.ncgp_solute; g0 += blockDim.x) {
        int ig = g0 + threadIdx.x, na = 0;
        if (ig < m.ncgp_solute) {
            bool inside = false;
            for (int a = m.gslot[ig]; a < m.gslot[ig + 1] && !inside; ++a)
                inside = box_d2(m, x, m.gatom[a], m.qswitch) <= rcq2;
            if (inside)
                for (int a = m.gslot[ig]; a < m.gslot[ig + 1]; ++a) na += !qnear[m.gatom[a]];
        }
        int tot;
        int pos = base + block_excl_scan(na, &tot);
        if (na)
            for (int a = m.gslot[ig]; a < m.gslot[ig + 1]; ++a) {
                int i = m.gatom[a];
                if (qnear[i]) continue;
                if (pos < s.cap_qp) s.qp[pos] = i;
                ++pos;
            }
        base += tot;
    }
    if (threadIdx.x == 0) s.cnt[C_QP] = base;
    __syncthreads();
    base = 0;
    for (int w0 = 0; w0 < m.nwat; w0 += blockDim.x) {
        int iw = w0 + threadIdx.x;
        bool ok = iw < m.nwat && box_d2(m, x, m.nat_solute + m.sa * iw, m.qswitch) <= rcq2;
        int tot;
        int pos = base + block_excl_scan(ok ? 1 : 0, &tot);
        if (ok && pos < s.cap_qw) s.qw[pos] = iw;
        base += tot;
    }
    if (threadIdx.x == 0) s.cnt[C_QW] = base;
}

void launch_build_box_pairs(const Launch& L, const Cut& c) {
    const int64_t G = L.m.ncgp_solute, W = L.m.nwat;
    const int64_t total = G * (G + 1) / 2 + G * W + W * (W - 1) / 2;
    if (total > 0) {
        k_build_box_groups<<<grid_for(total, 256, 8, L.nwin), 256, 0, L.st>>>(L.m, L.ds, c.rcpp2, c.rcpw2, c.rcww2);
        if (G > 0) k_expand_pp<<<grid_for(L.s0.cap_ppg, 128, 8, L.nwin), 128, 0, L.st>>>(L.m, L.ds);
    }
}
void launch_build_box(const Launch& L, const Cut& c, const uint8_t* qnear, int pairs) {
    if (pairs) launch_build_box_pairs(L, c);
    if (L.m.nqat > 0) k_build_box_q<<<dim3(1, L.nwin), 1024, 0, L.st>>>(L.m, L.ds, qnear, c.rcq2);
}

// nonbond_pp_box, src/nonbondene.f90:4763-4853 (nbe_b, src/nonbonded.f90:78-108)
template <bool MIX>
__global__ void __launch_bounds__(256) k_box_pp(DevModel m, const DevState* __restrict__ states,
                                                const int* __restrict__ iwhich) {
    const DevState& s = states[blockIdx.y];
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel, evdw;
    const double* __restrict__ x = s.x;
    int n = min((int64_t)s.cnt[C_PP], s.cap_pp);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int2 e = s.pp[p];
        int i = e.x, j = e.y & 0x0fffffff, code = e.y >> 28;
        if constexpr (MIX) {   // FP32 pair arithmetic as k_pp's mixed form
            const float4 xi = s.xq[i], xj = s.xq[j];
            BoxPairF q = box_pair_f(xi, xj, box_shift_f(m, s.xq[m.gsw[iwhich[i]]], s.xq[m.gsw[iwhich[j]]]));
            float2 ab = m.ljf[((size_t)(code - 1) * m.natyps + m.iac[i]) * m.natyps + m.iac[j]];
            float el = xi.w * xj.w;
            if (code == 3) el *= m.el14f;
            float vel = el * q.r, r6 = q.r2 * q.r2 * q.r2;
            float va = ab.x * r6 * r6, vb = ab.y * r6;
            float dv = q.r2 * (-vel - 12.0f * va + 6.0f * vb);
            acc.grad(i, -q.tx * dv, -q.ty * dv, -q.tz * dv);
            acc.grad(j, q.tx * dv, q.ty * dv, q.tz * dv);
            eel.add(vel);
            evdw.add(va - vb);
            continue;
        }
        double sx, sy, sz;
        box_shift(m, x, m.gsw[iwhich[i]], m.gsw[iwhich[j]], sx, sy, sz);
        BoxPair q = box_pair(x, i, j, sx, sy, sz);
        double2 ab = m.lj[((size_t)(code - 1) * m.natyps + m.iac[i]) * m.natyps + m.iac[j]];
        double el = m.crg[i] * m.crg[j];
        if (code == 3) el = el * m.el14;
        double vel = el * q.r, r6 = q.r2 * q.r2 * q.r2;
        double va = ab.x * r6 * r6, vb = ab.y * r6;
        double dv = q.r2 * (-vel - 12.0 * va + 6.0 * vb);
        box_grad<MIX>(acc, i, -q.tx * dv, -q.ty * dv, -q.tz * dv);
        box_grad<MIX>(acc, j, q.tx * dv, q.ty * dv, q.tz * dv);
        eel.add(vel);
        evdw.add(va - vb);
    }
    eel.flush(acc, E_PP_EL);
    evdw.flush(acc, E_PP_VDW);
}

// nonbond_pw_box, src/nonbondene.f90:4920-5009
template <bool MIX>
__global__ void __launch_bounds__(256) k_box_pw(DevModel m, const DevState* __restrict__ states,
                                                const int* __restrict__ iwhich) {
    const DevState& s = states[blockIdx.y];
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel, evdw;
    const double* __restrict__ x = s.x;
    int n = min((int64_t)s.cnt[C_PW], s.cap_pw);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int2 e = s.pw[p];
        int i = e.x, j0 = m.nat_solute + m.sa * e.y, ti = m.iac[i];
        if constexpr (MIX) {
            const float4 xi = s.xq[i];
            const float3 sh = box_shift_f(m, s.xq[m.gsw[iwhich[i]]], s.xq[j0]);
            float g[3] = {0.f, 0.f, 0.f};
            for (int a = 0; a < m.sa; ++a) {
                int tw = m.wtype[a];
                int code = m.ljcod[ti * m.natyps + tw];
                float2 ab = m.ljf[((size_t)(code - 1) * m.natyps + ti) * m.natyps + tw];
                BoxPairF q = box_pair_f(xi, s.xq[j0 + a], sh);
                float vel = xi.w * m.wcrgf[a] * q.r, r6 = q.r2 * q.r2 * q.r2;
                float va = ab.x * r6 * r6, vb = ab.y * r6;
                float dv = q.r2 * (-vel - 12.0f * va + 6.0f * vb);
                g[0] -= q.tx * dv;
                g[1] -= q.ty * dv;
                g[2] -= q.tz * dv;
                acc.grad(j0 + a, q.tx * dv, q.ty * dv, q.tz * dv);
                eel.add(vel);
                evdw.add(va - vb);
            }
            acc.grad(i, g[0], g[1], g[2]);
            continue;
        }
        double sx, sy, sz;
        box_shift(m, x, m.gsw[iwhich[i]], j0, sx, sy, sz);
        double g[3] = {0, 0, 0};
        for (int a = 0; a < m.sa; ++a) {
            int tw = m.wtype[a];
            int code = m.ljcod[ti * m.natyps + tw];
            double2 ab = m.lj[((size_t)(code - 1) * m.natyps + ti) * m.natyps + tw];
            BoxPair q = box_pair(x, i, j0 + a, sx, sy, sz);
            double vel = m.crg[i] * m.wcrg[a] * q.r, r6 = q.r2 * q.r2 * q.r2;
            double va = ab.x * r6 * r6, vb = ab.y * r6;
            double dv = q.r2 * (-vel - 12.0 * va + 6.0 * vb);
            g[0] -= q.tx * dv;
            g[1] -= q.ty * dv;
            g[2] -= q.tz * dv;
            box_grad<MIX>(acc, j0 + a, q.tx * dv, q.ty * dv, q.tz * dv);
            eel.add(vel);
            evdw.add(va - vb);
        }
        box_grad<MIX>(acc, i, g[0], g[1], g[2]);
    }
    eel.flush(acc, E_PW_EL);
    evdw.flush(acc, E_PW_VDW);
}

// nonbond_ww_spc_box / nonbond_ww_box, src/nonbondene.f90:5979-6077, 5576-5654
// (nbe_spcb, src/nonbonded.f90:271-291): one shift per molecule pair from
// the first atoms; SPC: LJ between the first atoms only
template <bool MIX, bool SPC>
__global__ void __launch_bounds__(256) k_box_ww(DevModel m, const DevState* __restrict__ states) {
    const DevState& s = states[blockIdx.y];
    Acc<MIX> acc = make_acc<MIX>(s);
    ESum<MIX> eel, evdw;
    const double* __restrict__ x = s.x;
    int n = min((int64_t)s.cnt[C_WW], s.cap_ww);
    const int sa = m.sa;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int2 e = s.ww[p];
        int i0 = m.nat_solute + sa * e.x, j0 = m.nat_solute + sa * e.y;
        if constexpr (MIX) {
            float4 xi[kMaxSolv], xj[kMaxSolv];
            for (int a = 0; a < sa; ++a) {
                xi[a] = s.xq[i0 + a];
                xj[a] = s.xq[j0 + a];
            }
            const float3 sh = box_shift_f(m, xi[0], xj[0]);
            float gi[kMaxSolv][3] = {}, gj[kMaxSolv][3] = {};
            for (int la = 0; la < sa; ++la)
                for (int ka = 0; ka < sa; ++ka) {
                    bool lj = !SPC || (la == 0 && ka == 0);
                    int k = la * kMaxSolv + ka;
                    BoxPairF q = box_pair_f(xi[la], xj[ka], sh);
                    float vel = m.wwEf[k] * q.r, dv, vdw = 0.0f;
                    if (lj) {
                        float r6 = q.r2 * q.r2 * q.r2;
                        float va = m.wwAf[k] * r6 * r6, vb = m.wwBf[k] * r6;
                        dv = q.r2 * (-vel - 12.0f * va + 6.0f * vb);
                        vdw = va - vb;
                    } else {
                        dv = q.r2 * (-vel);
                    }
                    gi[la][0] -= q.tx * dv; gi[la][1] -= q.ty * dv; gi[la][2] -= q.tz * dv;
                    gj[ka][0] += q.tx * dv; gj[ka][1] += q.ty * dv; gj[ka][2] += q.tz * dv;
                    eel.add(vel);
                    evdw.add(vdw);
                }
            for (int a = 0; a < sa; ++a) {
                acc.grad(i0 + a, gi[a][0], gi[a][1], gi[a][2]);
                acc.grad(j0 + a, gj[a][0], gj[a][1], gj[a][2]);
            }
            continue;
        }
        double sx, sy, sz;
        box_shift(m, x, i0, j0, sx, sy, sz);
        double gi[kMaxSolv][3] = {}, gj[kMaxSolv][3] = {};
        for (int la = 0; la < sa; ++la)
            for (int ka = 0; ka < sa; ++ka) {
                bool lj = !SPC || (la == 0 && ka == 0);
                int k = la * kMaxSolv + ka;
                BoxPair q = box_pair(x, i0 + la, j0 + ka, sx, sy, sz);
                double vel = m.wwE[k] * q.r, dv, vdw = 0.0;
                if (lj) {
                    double r6 = q.r2 * q.r2 * q.r2;
                    double va = m.wwA[k] * r6 * r6, vb = m.wwB[k] * r6;
                    dv = q.r2 * (-vel - 12.0 * va + 6.0 * vb);
                    vdw = va - vb;
                } else {
                    dv = q.r2 * (-vel);
                }
                gi[la][0] -= q.tx * dv; gi[la][1] -= q.ty * dv; gi[la][2] -= q.tz * dv;
                gj[ka][0] += q.tx * dv; gj[ka][1] += q.ty * dv; gj[ka][2] += q.tz * dv;
                eel.add(vel);
                evdw.add(vdw);
            }
        for (int a = 0; a < sa; ++a) {
            box_grad<MIX>(acc, i0 + a, gi[a][0], gi[a][1], gi[a][2]);
            box_grad<MIX>(acc, j0 + a, gj[a][0], gj[a][1], gj[a][2]);
        }
    }
    eel.flush(acc, E_WW_EL);
    evdw.flush(acc, E_WW_VDW);
}

// nonbond_qp_box, src/nonbondene.f90:5234-5335, and nonbond_qw_box /
// nonbond_qw_spc_box, 5422-5505, 5771-5881 (nbe_qx, nbe_qspc), FP64 form
// (the mixed form runs k_qenv_lanes<..., BOX>): one thread per (listed unit,
// Q atom); the unit's shift brings it next to qswitch, taken from the first
// group atom inside Rcq (qp, nbqp_cgp) or the water's first atom (qw).
// Per-state energies are summed in registers.
template <bool MIX, bool WATER, bool SPC>
__global__ void __launch_bounds__(256) k_box_q(DevModel m, const DevState* __restrict__ states,
                                               const int* __restrict__ iwhich, double rcq2) {
    const DevState& s = states[blockIdx.y];
    Acc<MIX> acc = make_acc<MIX>(s);
    const double* __restrict__ x = s.x;
    const int S = m.S, nq = m.nqat;
    ESum<MIX> eel[kMaxStates], evdw[kMaxStates];
    int n = WATER ? min((int64_t)s.cnt[C_QW], s.cap_qw) : min((int64_t)s.cnt[C_QP], s.cap_qp);
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)n * nq;
         t += (int64_t)gridDim.x * blockDim.x) {
        int u = (int)(t / nq), iq = (int)(t % nq);
        int i = m.iqseq[iq];
        double sx, sy, sz;
        int j0, na;
        if (WATER) {
            j0 = m.nat_solute + m.sa * s.qw[u];
            na = m.sa;
            box_shift(m, x, m.qswitch, j0, sx, sy, sz);
        } else {
            j0 = s.qp[u];
            na = 1;
            int g = iwhich[j0], ref = m.gatom[m.gslot[g]];
            for (int a = m.gslot[g]; a < m.gslot[g + 1]; ++a)
                if (box_d2(m, x, m.gatom[a], m.qswitch) <= rcq2) {
                    ref = m.gatom[a];
                    break;
                }
            box_shift(m, x, m.qswitch, ref, sx, sy, sz);
        }
        double gi[3] = {0, 0, 0};
        for (int a = 0; a < na; ++a) {
            int j = j0 + a;
            BoxPair q = box_pair(x, i, j, sx, sy, sz);
            bool lj = !(WATER && SPC) || a == 0;
            double dvs = 0.0;
            double r6hc = 1.0 / (q.r2 * q.r2 * q.r2);
            for (int st = 0; st < S; ++st) {
                const QPar P = WATER ? m.qw_tab[((size_t)iq * m.sa + a) * S + st] : m.qp_tab[((size_t)j * nq + iq) * S + st];
                double lam = s.lambda[st];
                if (lj) {
                    double vel, vdw, dv;
                    nbe_qx_d(q.r2, q.r, r6hc, P.A, P.B, P.el, P.sc, lam, vel, vdw, dv);
                    dvs += dv;
                    eel[st].add(vel);
                    evdw[st].add(vdw);
                } else {   // nbe_qspc
                    double vel = P.el * q.r;
                    dvs += -q.r2 * vel * lam;
                    eel[st].add(vel);
                }
            }
            gi[0] -= q.tx * dvs;
            gi[1] -= q.ty * dvs;
            gi[2] -= q.tz * dvs;
            box_grad<MIX>(acc, j, q.tx * dvs, q.ty * dvs, q.tz * dvs);
        }
        box_grad<MIX>(acc, i, gi[0], gi[1], gi[2]);
    }
    for (int st = 0; st < S; ++st) {
        eel[st].flush(acc, eq_slot(st, WATER ? 4 : 2));
        evdw[st].flush(acc, eq_slot(st, WATER ? 5 : 3));
    }
}

// the mixed form's box Q terms (k_qenv_lanes<..., BOX>)
template <bool WATER>
void launch_box_qenv(const Launch& L, const int* iwhich, double rcq2, dim3 g) {
    const bool spc = L.m.spc != 0, s4 = L.m.S <= 4;
    const float rq2 = (float)rcq2;
#define QB(SPC, SM) k_qenv_lanes<SPC, WATER, SM, true><<<g, kQBlock, 0, L.st>>>(L.m, L.ds, iwhich, rq2)
    if (spc) { if (s4) QB(true, 4); else QB(true, kMaxStates); }
    else { if (s4) QB(false, 4); else QB(false, kMaxStates); }
#undef QB
}
int launch_box_nonbond(const Launch& L, int md, int mixed, const int* iwhich, double rcq2, int pairs) {
    const DevModel& m = L.m;
    int nl = 0;
    auto grid = [&](int64_t n) { return grid_for(n > 1 ? n : 1, 256, 8, L.nwin); };
    if (!pairs) md = 0;   // the gather rows evaluate pp, pw and ww (the mixed form's box rows)
    if (md && m.ncgp_solute > 0) {
        if (mixed) k_box_pp<true><<<grid(L.s0.cap_pp), 256, 0, L.st>>>(m, L.ds, iwhich);
        else k_box_pp<false><<<grid(L.s0.cap_pp), 256, 0, L.st>>>(m, L.ds, iwhich);
        ++nl;
    }
    if (m.nwat > 0) {
        if (md) {
            if (mixed) k_box_pw<true><<<grid(L.s0.cap_pw), 256, 0, L.st>>>(m, L.ds, iwhich);
            else k_box_pw<false><<<grid(L.s0.cap_pw), 256, 0, L.st>>>(m, L.ds, iwhich);
            dim3 g = grid(L.s0.cap_ww);
            if (mixed) { if (m.spc) k_box_ww<true, true><<<g, 256, 0, L.st>>>(m, L.ds); else k_box_ww<true, false><<<g, 256, 0, L.st>>>(m, L.ds); }
            else { if (m.spc) k_box_ww<false, true><<<g, 256, 0, L.st>>>(m, L.ds); else k_box_ww<false, false><<<g, 256, 0, L.st>>>(m, L.ds); }
            nl += 2;
        }
        if (m.nqat > 0) {
            if (mixed) {   // lane = water, Q atoms looped (k_qenv_lanes' box form); environment gradient into fq
                launch_box_qenv<true>(L, iwhich, rcq2, grid_for(L.s0.cap_qw * 32, kQBlock, L.tu.v[T_QW], L.nwin));
            } else {
                dim3 g = grid(L.s0.cap_qw * m.nqat);
                if (m.spc) k_box_q<false, true, true><<<g, 256, 0, L.st>>>(m, L.ds, iwhich, rcq2); else k_box_q<false, true, false><<<g, 256, 0, L.st>>>(m, L.ds, iwhich, rcq2);
            }
            ++nl;
        }
    }
    if (m.nqat > 0 && m.nat_solute > 0) {
        if (mixed) {
            launch_box_qenv<false>(L, iwhich, rcq2, grid_for(L.s0.cap_qp * 32, kQBlock, L.tu.v[T_QP], L.nwin));
        } else {
            dim3 g = grid(L.s0.cap_qp * m.nqat);
            k_box_q<false, false, false><<<g, 256, 0, L.st>>>(m, L.ds, iwhich, rcq2);
        }
        ++nl;
    }
    return nl;
}
// p_restrain, src/bondene.f90:764-1020 (FP64 in both forms).  Blocks
// [0, nseq) take one sequence restraint each (the centre modes sum their
// atoms in a fixed-order tree), blocks [nseq, nseq + nwall) one wall
// restraint each, the rest the position / distance / angle restraints.
template <bool MIX>
__device__ __forceinline__ void restr_energy(const Acc<MIX>& acc, int slot, double e) {
    if constexpr (MIX) acc.energy_fix(slot, to_fixd(e));
    else acc.energy(slot, e);
}
template <bool MIX>
__device__ __forceinline__ void restr_grad(const Acc<MIX>& acc, int i, double gx, double gy, double gz) {
    if constexpr (MIX) acc.gradd(i, gx, gy, gz);
    else acc.grad(i, gx, gy, gz);
}
// a state-dependent restraint's energy: every state's EQ(s)%restraint for
// state -1 (E%restraint%protein without states), else that state's
template <bool MIX>
__device__ __forceinline__ void restr_state_energy(const Acc<MIX>& acc, int S, int st, double e) {
    if (st >= 0) restr_energy<MIX>(acc, qr_slot(st), e);
    else if (S == 0) restr_energy<MIX>(acc, E_RST_PROT, e);
    else
        for (int k = 0; k < S; ++k) restr_energy<MIX>(acc, qr_slot(k), e);
}
constexpr int kRestrBlock = 128;
template <bool MIX>
__global__ void __launch_bounds__(kRestrBlock) k_restraints(DevModel m, const DevState* __restrict__ states, RestrDev r) {
    const DevState& s = states[blockIdx.y];
    const Acc<MIX> acc = make_acc<MIX>(s);
    const double* __restrict__ x = s.x;
    const int b = blockIdx.x;
    if (b < r.nseq + r.nwall) {
        const bool wall = b >= r.nseq;
        const int4 q = wall ? r.wall[b - r.nseq] : r.seq[b];
        const int first = q.x, last = q.y, ih = q.z, mode = wall ? 0 : q.w;
        // heavy(i) .or. ih == 1 .and. .not.(excl(i) .and. freeze): bit 0 heavy,
        // bit 1 an excluded atom frozen (qnb_set_freeze)
        auto pick = [&](int i) { return (r.heavy[i] & 1) || (ih == 1 && !(r.heavy[i] & 2)); };
        if (wall) {   // half-harmonic wall about xwcent, Morse inside
            const double* p = r.wall_p + 4 * (b - r.nseq);
            const double d0 = p[0], fk = p[1], aM = p[2], dM = p[3];
            ESum<MIX> e;
            for (int i = first + threadIdx.x; i <= last; i += kRestrBlock) {
                if (!pick(i)) continue;
                double vx = x[3 * i] - m.xwcent[0], vy = x[3 * i + 1] - m.xwcent[1], vz = x[3 * i + 2] - m.xwcent[2];
                double dist = sqrt(vx * vx + vy * vy + vz * vz);
                double db = dist - d0, erst, dv;
                if (db > 0.0) {
                    erst = 0.5 * fk * db * db - dM;
                    dv = fk * db / dist;
                } else {
                    double fexp = exp(aM * db);
                    erst = dM * (fexp * fexp - 2.0 * fexp);
                    dv = -2.0 * dM * aM * (fexp - fexp * fexp) / dist;
                }
                e.add(erst);
                restr_grad<MIX>(acc, i, vx * dv, vy * dv, vz * dv);
            }
            e.flush(acc, E_RST_PROT);
            return;
        }
        const double fk = r.seq_fk[b];
        if (mode == 0) {   // each atom to its topology position
            ESum<MIX> e;
            for (int i = first + threadIdx.x; i <= last; i += kRestrBlock) {
                if (!pick(i)) continue;
                double dx = x[3 * i] - r.xtop[3 * i], dy = x[3 * i + 1] - r.xtop[3 * i + 1],
                       dz = x[3 * i + 2] - r.xtop[3 * i + 2];
                e.add(0.5 * fk * (dx * dx + dy * dy + dz * dz));
                restr_grad<MIX>(acc, i, dx * fk, dy * fk, dz * fk);
            }
            e.flush(acc, E_RST_PROT);
            return;
        }
        // geometric (1) or mass (2) centre of the picked atoms
        __shared__ double red[4][kRestrBlock];
        double a[4] = {0.0, 0.0, 0.0, 0.0};
        for (int i = first + threadIdx.x; i <= last; i += kRestrBlock) {
            if (!pick(i)) continue;
            const double w = mode == 2 ? r.mass[i] : 1.0;
#pragma unroll
            for (int c = 0; c < 3; ++c) a[c] += (x[3 * i + c] - r.xtop[3 * i + c]) * w;
            a[3] += w;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = a[k];
        __syncthreads();
        for (int h = kRestrBlock / 2; h > 0; h >>= 1) {
            if (threadIdx.x < h)
#pragma unroll
                for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
            __syncthreads();
        }
        const double tot = red[3][0];
        if (tot <= 0.0) return;
        const double drx = red[0][0] / tot, dry = red[1][0] / tot, drz = red[2][0] / tot;
        if (threadIdx.x == 0) restr_energy<MIX>(acc, E_RST_PROT, 0.5 * fk * (drx * drx + dry * dry + drz * drz));
        for (int i = first + threadIdx.x; i <= last; i += kRestrBlock) {
            if (!pick(i)) continue;
            const double f = mode == 2 ? fk : fk * r.mass[i] / 12.010;   // the reference's geometric-centre force
            restr_grad<MIX>(acc, i, drx * f, dry * f, drz * f);
        }
        return;
    }
    const int nterm = r.npos + r.ndist + r.nang;
    const int S = m.S;
    for (int t = (b - r.nseq - r.nwall) * kRestrBlock + threadIdx.x; t < nterm;
         t += (gridDim.x - r.nseq - r.nwall) * kRestrBlock) {
        if (t < r.npos) {   // position restraint
            int2 q = r.pos[t];
            const double* p = r.pos_xfk + 6 * t;
            const int i = q.x, st = q.y;
            double dx = x[3 * i] - p[0], dy = x[3 * i + 1] - p[1], dz = x[3 * i + 2] - p[2];
            const double wgt = st >= 0 ? s.lambda[st] : 1.0;
            restr_state_energy<MIX>(acc, S, st, 0.5 * (p[3] * (dx * dx) + p[4] * (dy * dy) + p[5] * (dz * dz)));
            restr_grad<MIX>(acc, i, p[3] * dx * wgt, p[4] * dy * wgt, p[5] * dz * wgt);
            continue;
        }
        int u = t - r.npos;
        if (u < r.ndist) {   // flat-bottom distance restraint
            int4 q = r.dist[u];
            const double* p = r.dist_p + 3 * u;
            double vx = x[3 * q.y] - x[3 * q.x], vy = x[3 * q.y + 1] - x[3 * q.x + 1], vz = x[3 * q.y + 2] - x[3 * q.x + 2];
            double dist = sqrt(vx * vx + vy * vy + vz * vz);
            double db;
            if (dist < p[0]) db = dist - p[0];
            else if (dist > p[1]) db = dist - p[1];
            else continue;
            const double wgt = q.z >= 0 ? s.lambda[q.z] : 1.0;
            restr_state_energy<MIX>(acc, S, q.z, 0.5 * p[2] * db * db);
            double dv = wgt * p[2] * db / dist;
            restr_grad<MIX>(acc, q.x, -vx * dv, -vy * dv, -vz * dv);
            restr_grad<MIX>(acc, q.y, vx * dv, vy * dv, vz * dv);
            continue;
        }
        u -= r.ndist;
        {   // angle restraint
            int4 q = r.ang[u];
            const double* p = r.ang_p + 2 * u;
            AngleVal<double> c = angle_calc(atom_pos<false>(s, q.x), atom_pos<false>(s, q.y), atom_pos<false>(s, q.z));
            double db = c.angl - p[0];
            const double wgt = q.w >= 0 ? s.lambda[q.w] : 1.0;
            restr_state_energy<MIX>(acc, S, q.w, 0.5 * p[1] * db * db);
            double dv = wgt * p[1] * db;
            restr_grad<MIX>(acc, q.x, c.a.x * dv, c.a.y * dv, c.a.z * dv);
            restr_grad<MIX>(acc, q.y, -c.b.x * dv, -c.b.y * dv, -c.b.z * dv);
            restr_grad<MIX>(acc, q.z, c.c.x * dv, c.c.y * dv, c.c.z * dv);
        }
    }
}
void launch_restraints(const Launch& L, const RestrDev& r, int mixed) {
    const int nterm = r.npos + r.ndist + r.nang;
    const int nb = r.nseq + r.nwall + std::min(64, (nterm + kRestrBlock - 1) / kRestrBlock);
    if (nb == 0) return;
    dim3 g(nb, L.nwin);
    if (mixed) k_restraints<true><<<g, kRestrBlock, 0, L.st>>>(L.m, L.ds, r);
    else k_restraints<false><<<g, kRestrBlock, 0, L.st>>>(L.m, L.ds, r);
}
void launch_restrain_solvent(const Launch& L, const SolventDev& p, double Tfree, int mixed, const int* wsw,
                             const uint8_t* heavy_solv) {
    if (L.m.nwat == 0) return;
    const int tdev = Tfree < 0.0;
    double shift = (!tdev && p.fk_wsphere != 0.0) ? sqrt(p.boltz * Tfree / p.fk_wsphere) : 0.0;
    dim3 g = grid_for(L.m.nwat, 32, 16, L.nwin);
    if (mixed) k_restrain_solvent<true><<<g, 32, 0, L.st>>>(L.m, L.ds, p, shift, wsw, heavy_solv, tdev);
    else k_restrain_solvent<false><<<g, 32, 0, L.st>>>(L.m, L.ds, p, shift, wsw, heavy_solv, tdev);
}
// returns the number of launches
int launch_watpol(const Launch& L, const SolventDev& p, int istep, int md, int mixed) {
    if (L.m.nwat == 0 || !p.wpol || p.nshell <= 0) return 0;
    int nl = 0;
    dim3 gw((L.m.nwat + 31) / 32, L.nwin);   // FP64 math per water: 32-thread blocks
    if (md) {
        k_watpol_reset<<<L.nwin, kMaxShell, 0, L.st>>>(L.ds);
        if (mixed) k_watpol_theta<true><<<gw, 32, 0, L.st>>>(L.m, L.ds, p);
        else k_watpol_theta<false><<<gw, 32, 0, L.st>>>(L.m, L.ds, p);
        k_watpol_rank<<<dim3(p.nshell * kRankParts, L.nwin), kRankBlock, 0, L.st>>>(L.m, L.ds);
        nl += 3;
    }
    if (istep > 0 && md && (istep % (int)llround(p.itdis)) == 0) {
        k_watpol_update<<<dim3(1, L.nwin), kMaxShell, 0, L.st>>>(p, L.ds);
        ++nl;
    }
    if (md) {
        if (mixed) k_watpol_force<true, true><<<gw, 32, 0, L.st>>>(L.m, L.ds, p);
        else k_watpol_force<false, true><<<gw, 32, 0, L.st>>>(L.m, L.ds, p);
    } else {
        if (mixed) k_watpol_force<true, false><<<gw, 32, 0, L.st>>>(L.m, L.ds, p);
        else k_watpol_force<false, false><<<gw, 32, 0, L.st>>>(L.m, L.ds, p);
    }
    ++nl;
    if (md) {
        k_watpol_average<<<dim3(1, L.nwin), 512, 0, L.st>>>(L.m, p, L.ds);
        ++nl;
    }
    return nl;
}

void launch_q_adjoint(const Launch& L) {
    if (L.m.nqat == 0) return;
    bool spc = L.m.spc != 0, s4 = L.m.S <= 4;
#define QA(SPC, W, SM) k_qadj_env<SPC, W, SM><<<g, kQBlock, 0, L.st>>>(L.m, L.ds)
    if (L.m.nwat > 0) {
        dim3 g = grid_for(L.s0.cap_qw * 32, kQBlock, 8, L.nwin);
        if (spc) { if (s4) QA(true, true, 4); else QA(true, true, kMaxStates); }
        else { if (s4) QA(false, true, 4); else QA(false, true, kMaxStates); }
    }
    if (L.m.nat_solute > 0) {
        dim3 g = grid_for(L.s0.cap_qp * 32, kQBlock, 8, L.nwin);
        if (s4) QA(true, false, 4); else QA(true, false, kMaxStates);
    }
#undef QA
    if (L.s0.nqq > 0) k_qadj_qq<<<dim3((L.s0.nqq + 63) / 64, L.nwin), 64, 0, L.st>>>(L.m, L.ds);
}

void launch_export_pairs(const Launch& L, int win, int kind, int32_t* di, int32_t* dj, int64_t cap, int* dcount) {
    k_export<<<blocks_for(1 << 20, 256, 8), 256, 0, L.st>>>(L.m, L.ds, win, kind, di, dj, cap, dcount);
}

}  // namespace qnb
