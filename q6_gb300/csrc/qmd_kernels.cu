// Device-resident MD step of qdyn (leap-frog, Berendsen, SHAKE), FP64.
//
// newvel_ber        src/md.f90:1451-1466
// shake             src/bondene.f90:1069-1150 (initial_constraint 1025-1048)
// v = (x - xx)/dt   src/md.f90:1787-1789
// temperature       src/md.f90:1379-1447
//
// Every kernel covers all windows of a context (grid.y = window).  The
// arithmetic is written with explicitly rounded FP64 operations (no fused
// multiply-add) in the reference's evaluation order, so a step reproduces
// a strict-IEEE CPU restatement of the same formulas bit for bit given the
// same gradient; only the kinetic-energy sums are regrouped (a fixed tree).
#include "qnb_internal.h"

namespace qnb {

namespace {

__device__ __forceinline__ int tgroup_of(const MdDev& md, int i) {
    for (int g = 0; g < md.ntg; ++g)
        if (i >= md.tg_first[g] && i <= md.tg_last[g]) return g;
    return -1;
}

// newvel_ber / newvel_nos, src/md.f90:1451-1466, 1505-1521:
// v = (v - d*winv*step) * sfact;  xx = x;  x = x + v*dt; with velocity Verlet
// step = dt/2 and the force half-step is applied again after the move.
// Nose-Hoover scales in nh_prop instead (sfact 1 here).
// Langevin random forces: a uniform draw per (window, step, atom component)
// from SplitMix64 (Steele, Lea and Flood 2014) chained over seed, window,
// step and component; the reference draws from its own sequential randm
// stream, which a parallel step cannot reproduce (same distribution).
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double lan_uniform(unsigned long long seed, int w, int istep, int k) {
    unsigned long long z = splitmix64(splitmix64(splitmix64(seed + (unsigned long long)w) +
                                                 (unsigned long long)(unsigned)istep) + (unsigned long long)k);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

__global__ void k_md_newvel(MdDev md, const DevState* __restrict__ states) {
    const int w = blockIdx.y;
    const DevState& s = states[w];
    const size_t off = (size_t)w * 3 * md.natom;
    double* __restrict__ v = md.v + off;
    double* __restrict__ xx = md.xx + off;
    double* __restrict__ x = s.x;
    const double* __restrict__ d = s.d;
    const MdWin& mw = md.win[w];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < md.natom; i += gridDim.x * blockDim.x) {
        if (md.thermostat == 2) {   // newvel_lan, src/md.f90:1468-1503 (uniform random forces)
            const double wi = md.winv[i];
            const double step = md.vv ? 0.5 * md.dt : md.dt;
            const double lf = 1.0 - md.lan_friction * step;
            const double rs = sqrt(__ddiv_rn(md.lan_gkT, wi));
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const int k = 3 * i + c;
                const double re = __dmul_rn(rs, __dsub_rn(lan_uniform(md.lan_seed, w, md.istep, k), 0.5));
                const double fd = __dmul_rn(__dmul_rn(__dsub_rn(d[k], re), wi), step);
                double vk = __dsub_rn(__dmul_rn(v[k], lf), fd);
                xx[k] = x[k];
                x[k] = __dadd_rn(x[k], __dmul_rn(vk, md.dt));
                if (md.vv) vk = __dsub_rn(__dmul_rn(vk, lf), fd);
                v[k] = vk;
            }
            continue;
        }
        const int g = md.thermostat == 1 ? 0 : tgroup_of(md, i);
        if (g < 0) continue;
        const double sf = md.thermostat == 1 ? 1.0 : mw.sfact[g], wi = md.winv[i];
        const double step = md.vv ? 0.5 * md.dt : md.dt;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const int k = 3 * i + c;
            double vk = __dmul_rn(__dsub_rn(v[k], __dmul_rn(__dmul_rn(d[k], wi), step)), sf);
            xx[k] = x[k];
            x[k] = __dadd_rn(x[k], __dmul_rn(vk, md.dt));
            if (md.vv) vk = __dmul_rn(__dsub_rn(vk, __dmul_rn(__dmul_rn(d[k], wi), step)), sf);
            v[k] = vk;
        }
    }
}

// SHAKE, one thread per (molecule, window), the reference's sweep order.
// mode 0: x is corrected against the reference positions xx; mode 1: xx
// against x.  Bounded by kShakeMaxIter sweeps per molecule.
__global__ void k_md_shake(MdDev md, const DevState* __restrict__ states, int mode) {
    const int w = blockIdx.y;
    const size_t off = (size_t)w * 3 * md.natom;
    double* __restrict__ xw = states[w].x;
    double* __restrict__ xxw = md.xx + off;
    double* __restrict__ X = mode == 0 ? xw : xxw;          // corrected
    const double* __restrict__ R = mode == 0 ? xxw : xw;    // reference
    uint8_t* __restrict__ ready = md.ready + (size_t)w * md.ncons;
    MdWin& mw = md.win[w];
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < md.nmol; m += gridDim.x * blockDim.x) {
        const int c0 = md.mol_first[m], c1 = md.mol_first[m + 1];
        for (int c = c0; c < c1; ++c) ready[c] = 0;
        int nits = 0;
        bool ok = false;
        while (true) {
            for (int c = c0; c < c1; ++c) {
                if (ready[c]) continue;
                const int i = md.con[c].x, j = md.con[c].y;
                // q_dist5(x(j), x(i)): vec = x(i) - x(j)
                double ex = __dsub_rn(X[3 * i], X[3 * j]), ey = __dsub_rn(X[3 * i + 1], X[3 * j + 1]),
                       ez = __dsub_rn(X[3 * i + 2], X[3 * j + 2]);
                double r2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
                double diff = __dsub_rn(md.dist2[c], r2);
                if (fabs(diff) < __dmul_rn(0.0001, md.dist2[c])) ready[c] = 1;   // CONST_TOL
                double fx = __dsub_rn(R[3 * i], R[3 * j]), fy = __dsub_rn(R[3 * i + 1], R[3 * j + 1]),
                       fz = __dsub_rn(R[3 * i + 2], R[3 * j + 2]);
                double scp = __dadd_rn(__dadd_rn(__dmul_rn(ex, fx), __dmul_rn(ey, fy)), __dmul_rn(ez, fz));
                const double wi = md.winv[i], wj = md.winv[j];
                double corr = __ddiv_rn(diff, __dmul_rn(__dmul_rn(2.0, scp), __dadd_rn(wi, wj)));
                // x(i) += xxij*corr*winv(i); x(j) += -xxij*corr*winv(j), left to right
                X[3 * i] = __dadd_rn(X[3 * i], __dmul_rn(__dmul_rn(fx, corr), wi));
                X[3 * i + 1] = __dadd_rn(X[3 * i + 1], __dmul_rn(__dmul_rn(fy, corr), wi));
                X[3 * i + 2] = __dadd_rn(X[3 * i + 2], __dmul_rn(__dmul_rn(fz, corr), wi));
                X[3 * j] = __dadd_rn(X[3 * j], __dmul_rn(__dmul_rn(-fx, corr), wj));
                X[3 * j + 1] = __dadd_rn(X[3 * j + 1], __dmul_rn(__dmul_rn(-fy, corr), wj));
                X[3 * j + 2] = __dadd_rn(X[3 * j + 2], __dmul_rn(__dmul_rn(-fz, corr), wj));
            }
            ++nits;
            bool all = true;
            for (int c = c0; c < c1; ++c) all = all && ready[c];
            if (all) { ok = true; break; }
            if (nits >= kShakeMaxIter) break;
        }
        atomicAdd(&mw.shake_iters, (unsigned long long)nits);
        if (!ok) atomicCAS(md.fail + w, 0, m + 1);
    }
}

// nh_prop, src/simprep.f90:2509-2550, one thread per window: the chain's
// half-step update around the velocity scale s = exp(-vnh(1) dt/2), driven
// by the last temperature() (Temp, Ndegf); k_md_scale_v then applies s.
__global__ void k_md_nh_prop(MdDev md, int nwin) {
    const int w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= nwin) return;
    MdWin& mw = md.win[w];
    const int M = md.nhchains;
    double* q = mw.qnh;
    double* vn = mw.vnh;
    double* xn = mw.xnh;
    const double dt2 = 0.5 * md.dt, dt4 = 0.5 * dt2, dt8 = 0.5 * dt4;
    const double kbT = md.boltz * md.temp0;
    double G[kMaxNh];
    G[0] = md.ndegf * md.boltz * (mw.temp - md.temp0) / q[0];
    for (int i = 1; i < M; ++i) G[i] = (q[i - 1] * vn[i - 1] * vn[i - 1] - kbT) / q[i];
    vn[M - 1] = vn[M - 1] + G[M - 1] * dt4;
    xn[M - 1] = xn[M - 1] + vn[M - 1] * dt2;
    double ex = 1.0;
    for (int i = M - 2; i >= 0; --i) {
        ex = exp(-dt8 * vn[i + 1]);
        vn[i] = (vn[i] * ex + G[i] * dt4) * ex;
        xn[i] = xn[i] + vn[i] * dt2;
    }
    const double sc = exp(-vn[0] * dt2);
    mw.nh_s = sc;
    G[0] = md.ndegf * md.boltz * (sc * sc * mw.temp - md.temp0) / q[0];
    vn[0] = (vn[0] * ex + G[0] * dt4) * ex;
    for (int i = 1; i < M - 1; ++i) {
        ex = exp(-dt8 * vn[i + 1]);
        G[i] = (q[i - 1] * vn[i - 1] * vn[i - 1] - kbT) / q[i];
        vn[i] = (vn[i] * ex + G[i] * dt4) * ex;
    }
    G[M - 1] = (q[M - 2] * vn[M - 2] * vn[M - 2] - kbT) / q[M - 1];
    vn[M - 1] = vn[M - 1] + G[M - 1] * dt4;
}
__global__ void k_md_scale_v(MdDev md) {
    const int w = blockIdx.y;
    double* __restrict__ v = md.v + (size_t)w * 3 * md.natom;
    const double sc = md.win[w].nh_s;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 3 * md.natom; k += gridDim.x * blockDim.x)
        v[k] = __dmul_rn(v[k], sc);
}

// v = (x - xx) / dt for every atom
__global__ void k_md_velocity(MdDev md, const DevState* __restrict__ states) {
    const int w = blockIdx.y;
    const size_t off = (size_t)w * 3 * md.natom;
    const double* __restrict__ x = states[w].x;
    const double* __restrict__ xx = md.xx + off;
    double* __restrict__ v = md.v + off;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 3 * md.natom; k += gridDim.x * blockDim.x)
        v[k] = __ddiv_rn(__dsub_rn(x[k], xx[k]), md.dt);
}

// initial_constraint's copies: xx = x (mode 1), xx = x - v dt (mode 2)
__global__ void k_md_copy_x(MdDev md, const DevState* __restrict__ states, int mode) {
    const int w = blockIdx.y;
    const size_t off = (size_t)w * 3 * md.natom;
    const double* __restrict__ x = states[w].x;
    const double* __restrict__ v = md.v + off;
    double* __restrict__ xx = md.xx + off;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 3 * md.natom; k += gridDim.x * blockDim.x)
        xx[k] = mode == 1 ? x[k] : __dsub_rn(x[k], __dmul_rn(v[k], md.dt));
    if (blockIdx.x == 0 && threadIdx.x == 0) md.win[w].shake_iters = 0ull;
}

// temperature(): one block per window; kinetic energies summed per group
// (all, non-excluded, excluded) by a fixed-order tree
constexpr int kTempBlock = 256;

// put_back_in_box, src/simprep.f90:4177-4352: the box centre (boxcentre
// fixed, or the plain mean of the solute atoms, else of all atoms), then every
// selected molecule whose mass centre lies outside the box around it moves by
// one box length per axis.  One block per window.
__global__ void __launch_bounds__(kTempBlock) k_md_put_back(DevModel m, MdDev md, const DevState* __restrict__ states) {
    __shared__ double red[3][kTempBlock];
    const int w = blockIdx.x;
    double* __restrict__ x = states[w].x;
    double c[3] = {md.pb_centre[0], md.pb_centre[1], md.pb_centre[2]};
    if (!md.pb_rigid) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int i = threadIdx.x; i < md.pb_nslu; i += kTempBlock) {
            sx += x[3 * i];
            sy += x[3 * i + 1];
            sz += x[3 * i + 2];
        }
        red[0][threadIdx.x] = sx;
        red[1][threadIdx.x] = sy;
        red[2][threadIdx.x] = sz;
        __syncthreads();
        for (int h = kTempBlock / 2; h > 0; h >>= 1) {
            if (threadIdx.x < h)
                for (int k = 0; k < 3; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
            __syncthreads();
        }
        for (int k = 0; k < 3; ++k) c[k] = red[k][0] / (double)md.pb_nslu;
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) md.pb_boxc[3 * w + k] = c[k];
    for (int mol = md.pb_first_mol + threadIdx.x; mol < md.pb_last_mol; mol += kTempBlock) {
        double cm[3] = {0.0, 0.0, 0.0}, mt = 0.0;
        for (int q = md.pb_mol_first[mol]; q < md.pb_mol_first[mol + 1]; ++q) {
            const int a = md.pb_atoms[q];
            const double ma = md.mass[a];
            mt += ma;
            for (int k = 0; k < 3; ++k) cm[k] += x[3 * a + k] * ma;
        }
        for (int k = 0; k < 3; ++k) {
            const double cmk = cm[k] * (1.0 / mt);
            const double hi = c[k] + m.boxl[k] / 2.0, lo = c[k] - m.boxl[k] / 2.0;
            const double sh = cmk > hi ? -m.boxl[k] : (cmk < lo ? m.boxl[k] : 0.0);
            if (sh != 0.0)
                for (int q = md.pb_mol_first[mol]; q < md.pb_mol_first[mol + 1]; ++q) x[3 * md.pb_atoms[q] + k] += sh;
        }
    }
}

__global__ void __launch_bounds__(kTempBlock) k_md_temperature(MdDev md, const uint8_t* __restrict__ excl) {
    const int w = blockIdx.x;
    const size_t off = (size_t)w * 3 * md.natom;
    const double* __restrict__ v = md.v + off;
    __shared__ double red[3 * kMaxTg][kTempBlock];
    double a[3 * kMaxTg];
#pragma unroll
    for (int k = 0; k < 3 * kMaxTg; ++k) a[k] = 0.0;
    for (int i = threadIdx.x; i < md.natom; i += kTempBlock) {
        int g = tgroup_of(md, i);
        if (g < 0) continue;
        const double vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
        double sq = __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
        double ek = __dmul_rn(__dmul_rn(0.5, md.mass[i]), sq);
#pragma unroll
        for (int q = 0; q < kMaxTg; ++q) {
            if (q != g) continue;
            a[3 * q] = __dadd_rn(a[3 * q], ek);
            if (!excl[i]) a[3 * q + 1] = __dadd_rn(a[3 * q + 1], ek);
            else a[3 * q + 2] = __dadd_rn(a[3 * q + 2], ek);
        }
    }
#pragma unroll
    for (int k = 0; k < 3 * kMaxTg; ++k) red[k][threadIdx.x] = a[k];
    __syncthreads();
    for (int h = kTempBlock / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h)
#pragma unroll
            for (int k = 0; k < 3 * kMaxTg; ++k)
                red[k][threadIdx.x] = __dadd_rn(red[k][threadIdx.x], red[k][threadIdx.x + h]);
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    MdWin& mw = md.win[w];
    const double boltz = md.boltz;
    double temp = 0.0, tfree = 0.0;
    for (int g = 0; g < md.ntg; ++g) {
        tfree = __dadd_rn(tfree, red[3 * g + 1][0]);
        temp = __dadd_rn(temp, red[3 * g][0]);
    }
    mw.ekin = temp;
    mw.temp = __ddiv_rn(__ddiv_rn(__dmul_rn(2.0, temp), boltz), md.ndegf);
    mw.tfree = __ddiv_rn(__ddiv_rn(__dmul_rn(2.0, tfree), boltz), md.ndegfree);
    for (int g = 0; g < md.ntg; ++g) {
        mw.tg_temp[g] = __ddiv_rn(__ddiv_rn(__dmul_rn(2.0, red[3 * g][0]), boltz), md.tg_ndegf[g]);
        mw.tg_tfree[g] = __ddiv_rn(__ddiv_rn(__dmul_rn(2.0, red[3 * g + 1][0]), boltz), md.tg_ndegfree[g]);
        mw.tg_texcl[g] = md.tg_ndegf[g] != md.tg_ndegfree[g]
                             ? __ddiv_rn(__ddiv_rn(__dmul_rn(2.0, red[3 * g + 2][0]), boltz),
                                         __dsub_rn(md.tg_ndegf[g], md.tg_ndegfree[g]))
                             : red[3 * g + 2][0];
        // Berendsen: a group with Tfree 0 keeps its previous factor inside the root
        if (mw.tg_tfree[g] != 0.0) mw.sfact[g] = __dsub_rn(__ddiv_rn(md.temp0, mw.tg_tfree[g]), 1.0);
        mw.sfact[g] = sqrt(__dadd_rn(1.0, __dmul_rn(__ddiv_rn(md.dt, md.tau), mw.sfact[g])));
    }
}

// stop_cm_translation (src/simprep.f90:4496-4518): v -= sum(m v) / sum(m),
// one block per window, the sums by a fixed-order tree
__global__ void __launch_bounds__(kTempBlock) k_md_stop_cm(MdDev md) {
    const int w = blockIdx.x;
    double* __restrict__ v = md.v + (size_t)w * 3 * md.natom;
    __shared__ double red[4][kTempBlock];
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i = threadIdx.x; i < md.natom; i += kTempBlock) {
        const double rm = md.mass[i];
        a[0] = __dadd_rn(a[0], rm);
#pragma unroll
        for (int c = 0; c < 3; ++c) a[1 + c] = __dadd_rn(a[1 + c], __dmul_rn(v[3 * i + c], rm));
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = a[k];
    __syncthreads();
    for (int h = kTempBlock / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h)
#pragma unroll
            for (int k = 0; k < 4; ++k) red[k][threadIdx.x] = __dadd_rn(red[k][threadIdx.x], red[k][threadIdx.x + h]);
        __syncthreads();
    }
    const double vcm[3] = {__ddiv_rn(red[1][0], red[0][0]), __ddiv_rn(red[2][0], red[0][0]),
                           __ddiv_rn(red[3][0], red[0][0])};
    for (int i = threadIdx.x; i < md.natom; i += kTempBlock)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[3 * i + c] = __dsub_rn(v[3 * i + c], vcm[c]);
}

// Qmin's steepest descent step (src/minim.f90:891-935, 1056-1070), one
// block per window: the largest atomic force; a rise above the previous
// largest resets the scale to the initial step, otherwise it grows by 1.2;
// below force_cutoff the window has converged and stays put.  xx keeps the
// positions before the move (the SHAKE reference).
__global__ void __launch_bounds__(kTempBlock) k_md_min_step(MdDev md, const DevState* __restrict__ states,
                                                           double step0, double fcut, double max_move) {
    const int w = blockIdx.x;
    const size_t off = (size_t)w * 3 * md.natom;
    double* __restrict__ x = states[w].x;
    const double* __restrict__ d = states[w].d;
    double* __restrict__ xx = md.xx + off;
    MdWin& mw = md.win[w];
    __shared__ double red[kTempBlock];
    __shared__ double scale;
    double mx = 0.0;
    for (int i = threadIdx.x; i < md.natom; i += kTempBlock) {
        const double fx = d[3 * i], fy = d[3 * i + 1], fz = d[3 * i + 2];
        mx = fmax(mx, sqrt(fx * fx + fy * fy + fz * fz));
    }
    red[threadIdx.x] = mx;
    __syncthreads();
    for (int h = kTempBlock / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + h]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double maxf = red[0];
        int rv = maxf > mw.min_oldmax ? 1 : 0;
        mw.min_oldmax = maxf;
        if (maxf < fcut) rv = 2;
        if (rv == 1) mw.min_scale = step0;
        else if (rv == 0) mw.min_scale = mw.min_scale * 1.20;
        mw.min_state = rv;
        mw.min_maxf = maxf;
        double sc = rv == 2 ? 0.0 : mw.min_scale;
        if (max_move > 0.0 && sc * maxf > max_move) sc = max_move / maxf;   // optional cap (not in Qmin)
        scale = sc;
    }
    __syncthreads();
    const double sc = scale;
    for (int k = threadIdx.x; k < 3 * md.natom; k += kTempBlock) {
        xx[k] = x[k];
        if (sc != 0.0) x[k] = x[k] - d[k] * sc;
    }
}

__global__ void k_md_record(MdDev md, int nwin, const double* __restrict__ e_all,
                            const unsigned long long* __restrict__ efix_all, double* __restrict__ rec) {
    const int w = blockIdx.x;
    double* r = rec + (size_t)w * kMdRec;
    for (int k = threadIdx.x; k < kNumE; k += blockDim.x) {
        r[k] = e_all[(size_t)w * kNumE + k];
        reinterpret_cast<unsigned long long*>(r)[kNumE + k] = efix_all[(size_t)w * kNumE + k];
    }
    if (threadIdx.x == 0) {
        const MdWin& mw = md.win[w];
        r[2 * kNumE] = mw.ekin;
        r[2 * kNumE + 1] = mw.temp;
        r[2 * kNumE + 2] = mw.tfree;
        r[2 * kNumE + 3] = (double)mw.shake_iters;
    }
}

// pot_energy's d = 0 and the step's SHAKE iteration count
__global__ void k_md_clear(const DevState* __restrict__ states, size_t n3, MdWin* win) {
    double* d = states[blockIdx.y].d;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n3; k += (size_t)gridDim.x * blockDim.x)
        d[k] = 0.0;
    if (blockIdx.x == 0 && threadIdx.x == 0) win[blockIdx.y].shake_iters = 0ull;
}

dim3 atoms_grid(const Launch& L, int64_t n, int block) {
    int64_t b = (n + block - 1) / block;
    if (b > 1024) b = 1024;
    if (b < 1) b = 1;
    return dim3((unsigned)b, (unsigned)L.nwin);
}

}  // namespace

void launch_md_put_back(const Launch& L, const MdDev& md) {
    k_md_put_back<<<L.nwin, kTempBlock, 0, L.st>>>(L.m, md, L.ds);
}
void launch_md_nh(const Launch& L, const MdDev& md) {
    k_md_nh_prop<<<(L.nwin + 31) / 32, 32, 0, L.st>>>(md, L.nwin);
    k_md_scale_v<<<dim3((3 * md.natom + 255) / 256, L.nwin), 256, 0, L.st>>>(md);
}
void launch_md_newvel(const Launch& L, const MdDev& md) {
    k_md_newvel<<<atoms_grid(L, md.natom, 128), 128, 0, L.st>>>(md, L.ds);
}
void launch_md_shake(const Launch& L, const MdDev& md, int mode) {
    if (md.nmol == 0) return;
    k_md_shake<<<atoms_grid(L, md.nmol, 64), 64, 0, L.st>>>(md, L.ds, mode);
}
void launch_md_velocity(const Launch& L, const MdDev& md) {
    k_md_velocity<<<atoms_grid(L, 3 * (int64_t)md.natom, 256), 256, 0, L.st>>>(md, L.ds);
}
void launch_md_copy_x(const Launch& L, const MdDev& md, int mode) {
    k_md_copy_x<<<atoms_grid(L, 3 * (int64_t)md.natom, 256), 256, 0, L.st>>>(md, L.ds, mode);
}
void launch_md_temperature(const Launch& L, const MdDev& md, const uint8_t* excl) {
    k_md_temperature<<<L.nwin, kTempBlock, 0, L.st>>>(md, excl);
}
void launch_md_stop_cm(const Launch& L, const MdDev& md) {
    k_md_stop_cm<<<L.nwin, kTempBlock, 0, L.st>>>(md);
}
void launch_md_min_step(const Launch& L, const MdDev& md, double step0, double fcut, double max_move) {
    k_md_min_step<<<L.nwin, kTempBlock, 0, L.st>>>(md, L.ds, step0, fcut, max_move);
}
void launch_md_record(const Launch& L, const MdDev& md, const double* e_all, const unsigned long long* efix_all,
                      double* rec) {
    k_md_record<<<L.nwin, 64, 0, L.st>>>(md, L.nwin, e_all, efix_all, rec);
}
void launch_md_clear_d(const Launch& L, const MdDev& md) {
    size_t n3 = 3 * (size_t)md.natom;
    k_md_clear<<<atoms_grid(L, (int64_t)n3, 256), 256, 0, L.st>>>(L.ds, n3, md.win);
}

}  // namespace qnb
