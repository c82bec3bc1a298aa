// lbm_noalloc.cu - volume-averaged Nusselt and Reynolds numbers without any device
// allocation, for callers that cannot let a library call cudaMalloc.
//
// Who needs it: a caller whose device memory is already owned by an allocator of its own
// (the Fortran driver's OpenACC data region or memory pool, a framework's caching
// allocator, or a solve server that admits lattices against a fixed HBM budget).  In
// those programs a library-side cudaMalloc can fail although the owner still has free
// memory in its pool, it breaks the owner's accounting, and the matching cudaFree
// synchronises the whole device.  This entry point therefore works entirely in memory
// the caller passes (the fields and the two outputs) plus one fixed scratch array that is
// compiled into the library.
//
// Scratch: `g_nu_re_scratch`, a file-scope __device__ array of 3 partial sums per block
// for at most LBM_NOALLOC_MAX_BLOCKS blocks plus 3 totals (about 29 KB).  Every GPU that
// loads the library holds it until the process exits.  Every call shares it and it keeps
// the last call's contents; each call writes every slot it later reads, so nothing has to
// start at zero.  Calls that overlap on the GPU (on different streams, or from different
// host threads) race on it and must be serialised by the caller.
//
// Host code cannot use the array's name as a device address (it names a host-side
// shadow).  The first call on each device looks the address up with
// cudaGetSymbolAddress while that device is current and caches it, with the device's
// multiprocessor count; make that first call outside any stream capture.  The cached
// address belongs to the device's primary context (the one the runtime API uses): the entry
// point is for callers on that context, and not valid after cudaDeviceReset.
//
// Grid: min(LBM_NOALLOC_MAX_BLOCKS, 4 x multiprocessors) blocks stride over the lattice, so
// every SM of the device takes part whatever the lattice size; the partials are added in
// block order, so a call is reproducible on a given device.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/lbm_gpu.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = LBM_NOALLOC_MAX_BLOCKS;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_nu_re_scratch[3 * kMaxBlocks + 3];

double* g_scratch_addr[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};
std::mutex g_setup_mutex;

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}

// Block b sums the calNuRe terms (2DRB.F90:1631-1663, 3DRB.F90:1731-1768) over the cells
// b*kThreads + t + k*gridDim.x*kThreads and writes 3 partials to the scratch.
__global__ void __launch_bounds__(kThreads) k_nu_re_partials(const double* __restrict__ u, const double* __restrict__ v,
                                                             const double* __restrict__ w, const double* __restrict__ T,
                                                             long long ncell, int side, double* scratch) {
    const long long stride = (long long)gridDim.x * kThreads;
    double s_flux = 0.0, s_u2 = 0.0, s_bad = 0.0;
    for (long long c = (long long)blockIdx.x * kThreads + threadIdx.x; c < ncell; c += stride) {
        const double uc = u[c], vc = v[c], Tc = T[c];
        double r = uc * uc + vc * vc;
        double wc = 0.0;
        if (w) {
            wc = w[c];
            r = r + wc * wc;
        }
        s_flux += (side ? uc : vc) * Tc;
        s_u2 += r;
        s_bad += (isfinite(uc) && isfinite(vc) && isfinite(wc) && isfinite(Tc)) ? 0.0 : 1.0;
    }
    __shared__ double sh[kThreads / 32][3];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    s_flux = warp_sum(s_flux);
    s_u2 = warp_sum(s_u2);
    s_bad = warp_sum(s_bad);
    if (lane == 0) {
        sh[wid][0] = s_flux;
        sh[wid][1] = s_u2;
        sh[wid][2] = s_bad;
    }
    __syncthreads();
    if (wid == 0) {
        for (int s = 0; s < 3; ++s) {
            double x = lane < kThreads / 32 ? sh[lane][s] : 0.0;
            x = warp_sum(x);
            if (lane == 0) scratch[3 * blockIdx.x + s] = x;
        }
    }
}

// One thread per sum adds the block partials in block order (reproducible) into the
// three total slots at the end of the scratch.
__global__ void k_nu_re_total(double* scratch, int nblocks) {
    const int s = threadIdx.x;
    if (s >= 3) return;
    double t = 0.0;
    for (int b = 0; b < nblocks; ++b) t += scratch[3 * b + s];
    scratch[3 * kMaxBlocks + s] = t;
}

}  // namespace

extern "C" int lbm_calNuRe_noalloc(const double* u, const double* v, const double* w, const double* T, int64_t ncell,
                                   int side_heated, double lengthUnit, double diffusivity, double viscosity,
                                   void* stream, double* Nu, double* Re) {
    if (!u || !v || !T || !Nu || !Re || ncell <= 0) return LBM_ERR_PARAM;
    if (!(lengthUnit > 0.0) || !(diffusivity > 0.0) || !(viscosity > 0.0)) return LBM_ERR_PARAM;
    if (ncell > (int64_t)LBM_NOALLOC_MAX_CELLS) return LBM_ERR_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return LBM_ERR_CUDA;
    if (dev < 0 || dev >= kMaxDevices) return LBM_ERR_PARAM;
    double* scratch = nullptr;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_nu_re_scratch) != cudaSuccess || !p) return LBM_ERR_CUDA;
            int count = 0;
            if (cudaDeviceGetAttribute(&count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || count <= 0)
                return LBM_ERR_CUDA;
            g_sms[dev] = count;
            g_scratch_addr[dev] = (double*)p;
        }
        scratch = g_scratch_addr[dev];
        sms = g_sms[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    long long want = (ncell + kThreads - 1) / kThreads;
    if (want > 4LL * sms) want = 4LL * sms;
    if (want > kMaxBlocks) want = kMaxBlocks;
    const int nblocks = (int)want;
    k_nu_re_partials<<<nblocks, kThreads, 0, s>>>(u, v, w, T, (long long)ncell, side_heated ? 1 : 0, scratch);
    k_nu_re_total<<<1, 32, 0, s>>>(scratch, nblocks);
    if (cudaGetLastError() != cudaSuccess) return LBM_ERR_CUDA;
    double tot[3] = {0.0, 0.0, 0.0};
    if (cudaMemcpyAsync(tot, scratch + 3 * kMaxBlocks, sizeof(tot), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return LBM_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return LBM_ERR_CUDA;
    const double N = (double)ncell;
    *Nu = tot[0] / N * lengthUnit / diffusivity + 1.0;
    *Re = std::sqrt(tot[1] / N) * lengthUnit / viscosity;
    if (tot[2] != 0.0 || !std::isfinite(*Nu) || !std::isfinite(*Re)) return LBM_ERR_DIVERGED;
    return LBM_OK;
}
