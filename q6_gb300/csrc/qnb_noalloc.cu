// Allocation-free variant of the FP64 solvent-solvent path.
//
// Some callers cannot allocate device memory while they run: a host program
// that a job scheduler or an embedding application gives a fixed device-memory
// budget, a process whose own pool allocator already holds the device's free
// memory (a cudaMalloc there fails or fragments that pool), and a timed step
// loop in which cudaMalloc/cudaFree would synchronise the whole device.
// qnb_ww_spc_noalloc serves them. It selects SPC water pairs within the
// cut-off and evaluates their energies and gradient (nbwwlist +
// nonbond_ww_spc, Q6 src/nonbondene.f90:4274-4395, 5886-5975) without
// allocating. Its scratch, the water-pair list and its counter, is the
// file-scope array below. The array is part of the module image, so every GPU
// that loads the library holds it until the process exits.
//
// Sums: the gradient and the two energies are added with FP64 atomics, so
// their last bits depend on the order in which blocks finish (as in the FP64
// form of the engine); repeated calls agree to rounding, not bit for bit.
#include <cuda_runtime.h>

#include <mutex>

#include "qnb_internal.h"

namespace {

constexpr int kNoAllocMaxPairs = 1 << 20;   // water pairs held by the scratch (8 MiB)
constexpr int kNoAllocMaxWaters = 1 << 16;  // waters per call
constexpr int kMaxDevices = 64;

// The scratch of every call on a device: element 0's x is the pair counter,
// elements 0..31 (256 bytes) are reserved, the water pairs (iw, jw), iw < jw,
// start at element 32.  Calls share the array and it keeps the last call's
// contents; the counter is cleared at the start of each call.
constexpr int kScratchHead = 32;
static __device__ __align__(256) int2 g_noalloc_scratch[kScratchHead + kNoAllocMaxPairs];

// device address of g_noalloc_scratch, looked up once per device and kept for
// the life of the process (a cudaDeviceReset invalidates it: this entry point
// is not for use after a device reset)
int2* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

__device__ __forceinline__ double d2_exact(const double* x, int a, int b) {
    double dx = __dsub_rn(x[3 * b], x[3 * a]), dy = __dsub_rn(x[3 * b + 1], x[3 * a + 1]),
           dz = __dsub_rn(x[3 * b + 2], x[3 * a + 2]);
    return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// water pairs with O-O r2 <= rc2 (neither O excluded), each unordered pair once
__global__ void k_noalloc_select(int2* sc, const double* __restrict__ x, const uint8_t* __restrict__ excl,
                                 int first, int nwat, double rc2) {
    int* count = &sc[0].x;
    int2* pairs = sc + kScratchHead;
    int lane = threadIdx.x & 31;
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int iw = warp; iw < nwat; iw += nwarps) {
        int io = first + 3 * iw;
        if (excl && excl[io]) continue;
        for (int j0 = iw + 1; j0 < nwat; j0 += 32) {
            int jw = j0 + lane;
            bool ok = false;
            if (jw < nwat) {
                int jo = first + 3 * jw;
                ok = !(excl && excl[jo]) && d2_exact(x, io, jo) <= rc2;
            }
            unsigned b = __ballot_sync(0xffffffffu, ok);
            int base = 0;
            if (lane == 0 && b) base = atomicAdd(count, __popc(b));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (ok) {
                int pos = base + __popc(b & ((1u << lane) - 1u));
                if (pos < kNoAllocMaxPairs) pairs[pos] = make_int2(iw, jw);
            }
        }
    }
}

// nonbond_ww_spc: LJ + Coulomb for O-O, Coulomb for the other eight pairs;
// the gradient is added into d and the energies into e[0] (el), e[1] (vdW)
__global__ void k_noalloc_ww(const int2* sc, const double* __restrict__ x, double* __restrict__ d,
                             double* __restrict__ e, int first, double qO, double qH, double A, double B) {
    int n = min(sc[0].x, kNoAllocMaxPairs);
    const int2* pairs = sc + kScratchHead;
    double el = 0.0, vdw = 0.0;
    const double q[3] = {qO, qH, qH};
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        int2 w = pairs[p];
        int i0 = first + 3 * w.x, j0 = first + 3 * w.y;
        double gi[3][3] = {}, gj[3][3] = {};
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                int i = i0 + a, j = j0 + b;
                double tx = x[3 * j] - x[3 * i], ty = x[3 * j + 1] - x[3 * i + 1], tz = x[3 * j + 2] - x[3 * i + 2];
                double r2 = 1.0 / (tx * tx + ty * ty + tz * tz);
                double r = sqrt(r2);
                double vel = q[a] * q[b] * r, dv;
                if (a == 0 && b == 0) {
                    double r6 = r2 * r2 * r2, r12 = r6 * r6;
                    double va = A * r12, vb = B * r6;
                    dv = r2 * (-vel - 12.0 * va + 6.0 * vb);
                    vdw += va - vb;
                } else {
                    dv = r2 * (-vel);
                }
                el += vel;
                gi[a][0] -= tx * dv; gi[a][1] -= ty * dv; gi[a][2] -= tz * dv;
                gj[b][0] += tx * dv; gj[b][1] += ty * dv; gj[b][2] += tz * dv;
            }
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) {
                atomicAdd(d + 3 * (i0 + a) + c, gi[a][c]);
                atomicAdd(d + 3 * (j0 + a) + c, gj[a][c]);
            }
    }
    for (int o = 16; o > 0; o >>= 1) {
        el += __shfl_down_sync(0xffffffffu, el, o);
        vdw += __shfl_down_sync(0xffffffffu, vdw, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(e, el);
        atomicAdd(e + 1, vdw);
    }
}

int fail(int code, const char* msg) { return qnb::set_error(code, msg); }   // read by qnb_last_error

}  // namespace

extern "C" {

int qnb_ww_spc_noalloc(const double* x_dev, const uint8_t* excl_dev, int32_t first_water_atom, int32_t nwat,
                       double q_oxygen, double q_hydrogen, double A_oo, double B_oo, double rc2, double* d_dev,
                       double* e_dev, void* stream) {
    if (!x_dev || !d_dev || !e_dev) return fail(QNB_ERR_ARG, "null device pointer");
    if (nwat < 0 || first_water_atom < 0) return fail(QNB_ERR_ARG, "negative size");
    if (nwat > kNoAllocMaxWaters) return fail(QNB_ERR_CAPACITY, "more than 65536 waters for the no-alloc scratch");
    if (nwat < 2) return QNB_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(QNB_ERR_CUDA, "no current CUDA device");
    int2* sc = nullptr;
    {
        // one-time set-up on this device (the device is current): the host
        // name g_noalloc_scratch is only a stand-in, kernels need this address
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) return fail(QNB_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed");
            g_scratch_ptr[dev] = (int2*)p;
        }
        sc = g_scratch_ptr[dev];
    }
    if (cudaMemsetAsync(&sc[0].x, 0, sizeof(int), st) != cudaSuccess) return fail(QNB_ERR_CUDA, "counter reset failed");
    int blocks = (nwat * 32 + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_noalloc_select<<<blocks, 256, 0, st>>>(sc, x_dev, excl_dev, first_water_atom, nwat, rc2);
    int count = 0;
    if (cudaMemcpyAsync(&count, &sc[0].x, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return fail(QNB_ERR_CUDA, "pair selection failed");
    if (count > kNoAllocMaxPairs)
        return fail(QNB_ERR_CAPACITY, "more than 1048576 water pairs within the cut-off for the no-alloc scratch");
    int fb = (count + 255) / 256;
    if (fb < 1) fb = 1;
    if (fb > 4096) fb = 4096;
    k_noalloc_ww<<<fb, 256, 0, st>>>(sc, x_dev, d_dev, e_dev, first_water_atom, q_oxygen, q_hydrogen, A_oo, B_oo);
    if (cudaGetLastError() != cudaSuccess) return fail(QNB_ERR_CUDA, "kernel launch failed");
    return QNB_OK;
}

}  // extern "C"
