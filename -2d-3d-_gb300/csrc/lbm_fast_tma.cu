// lbm_fast_tma.cu - the two-kernel FP32/FP16 step with its population rows staged in
// shared memory by the Tensor Memory Accelerator (cp.async.bulk) on an mbarrier pipeline.
//
// The one-cell kernels (lbm_fast.cu) issue each cell's 26 pulls from the cell's own
// thread, and the collision arithmetic that follows keeps too few of those loads in
// flight: the kernels wait on memory with DRAM a third busy.  Here a persistent block
// walks tiles of R whole x-rows (fixed k, rows j0..j0+R-1).  For every direction a the
// source rows of a tile, (j - ey_a, k - ez_a), are one contiguous run of R*nx values of
// plane a, so a tile arrives as one bulk copy per direction (plus the lag / B_prev rows),
// issued by one warp (a lane per copy) STAGES-1 tiles ahead of the tile being computed.  Tiles cover the
// interior rows, and the threads update their interior cells pulling from shared memory
// with the x shift applied there, with no boundary tests.  The cells on the lattice's
// faces (a few per cent) are updated by the same blocks after their last tile, with the
// one-cell path's scalar pull and the reference's boundary rule; a face test inside the
// tiles would put a global-memory round trip on every tile's critical path.  The per-cell
// arithmetic is the one-cell path's inline functions, so the values are the same bit for
// bit.
//
// The in-place (AA) pattern uses the same kernel with other row sources and stores: an
// array in the swapped layout is staged from plane opp(a) at the pull's source rows, one in
// the streamed layout from plane a at the tile's own rows (no shift), and the interior
// cells store either back into their own opposite slots (even sweep) or at c + e_a (odd
// sweep: every target of an interior cell lies inside the lattice).  Face cells take the
// in-place one-cell path (lbm_fast_aa.cuh).
//
// Requirements (else the one-cell kernels run): nx a multiple of 8 (16-byte aligned rows
// for FP16 and FP32), and one row of a tile fitting the stage budget.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <mutex>

#include "lbm_fast.h"
#include "lbm_fast_aa.cuh"
#include "lbm_fast_cells.cuh"

namespace lbm {

namespace {

constexpr unsigned kHeader = 128;          // mbarriers at the start of shared memory
constexpr unsigned kWaitLimit = 1u << 22;  // bounded mbarrier polling

// Where a staged population row comes from, and where a cell's new values go.
constexpr int kRowPull = 0;   // two buffers: plane a, source rows (j - ey, k - ez), shift ex
constexpr int kRowSwap = 1;   // in-place swapped layout: plane opp(a), source rows, shift ex
constexpr int kRowLocal = 2;  // in-place streamed layout: plane a, the tile's own rows, no shift
constexpr int kStoreOut = 0;  // two buffers: plane a of the output array at the cell
constexpr int kStorePush = 1; // in-place odd sweep: plane a at c + e_a
constexpr int kStoreOpp = 2;  // in-place even sweep: plane opp(a) at the cell

}  // namespace

// In-place pattern: what the face cells of a staged sweep need (lbm_fast_aa.cuh).
template <class S>
struct AAExtra {
    AAFace<S> face;  // snapshots of the periodic faces of the swept array
    int opar;        // layout of the other array
    int graw;        // the thermal array's streamed slots hold pushed values
};

// Pipeline shape: threads per block, stages, blocks per SM, stage budget and limit.
// PipeA: two blocks of 8 warps per SM, 3 x 36 KB each.  A deeper shape (one 16-warp block
// per SM, 6 stages) measured slower on GB300 at 128^3 and 256^3 for both storage types.
template <int THREADS, int STAGES, int BLOCKS, unsigned BUDGET, unsigned MAXSTAGE>
struct Pipe {
    static constexpr int threads = THREADS, stages = STAGES, blocks = BLOCKS, warps = THREADS / 32;
    static constexpr unsigned budget = BUDGET, max_stage = MAXSTAGE;
    static_assert(2 * STAGES * 8 <= (int)kHeader, "mbarriers fit the header");
    static_assert(kHeader + STAGES * MAXSTAGE <= 232448u, "shared memory per block");
};
using PipeA = Pipe<256, 3, 2, 36u * 1024u, 72u * 1024u>;

namespace {

__device__ __forceinline__ unsigned saddr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Global -> shared bulk copy completing on `bar` (bytes and both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(saddr(dst)),
        "l"(src), "r"(bytes), "r"(saddr(bar))
        : "memory");
}
// Orders this thread's earlier generic-proxy accesses to shared memory before later
// async-proxy (bulk copy) writes to it.
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Bounded wait for phase `parity` of `bar`; false (and the error flag set) on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int* err, unsigned limit = kWaitLimit) {
    for (unsigned it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    atomicExch(err, 1);
    return false;
}

// After a timed-out wait for a stage's copies: wait once more, again bounded, so that copies
// still in flight land before the block exits and its shared memory is released.
__device__ __forceinline__ void mbar_drain(uint64_t* bar, unsigned parity) {
    for (unsigned it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) return;
}

__device__ __forceinline__ float s2f(float x) { return x; }
__device__ __forceinline__ float s2f(__half x) { return __half2float(x); }

}  // namespace

// Shared-memory layout of one stage (R rows of nx cells, rc = R*nx):
//   f rows [Q][rc] S | g rows [QT][rc] S | float rows [NF][rc]
// flow:    NF = 1  (lag_in)
// thermal: NF = D  (B_prev) + 1 in 2D (lag_in = F_y,n)
struct TmaPlan {
    int R = 0;              // rows per tile
    unsigned stage = 0;     // bytes per stage
    unsigned smem = 0;      // dynamic shared memory per block
    int ntj = 0;            // tiles along j
    long long ntiles = 0;
    int grid = 0;
    bool ok = false;
};

template <int D, class S, class PP>
static TmaPlan tma_plan(const Geo& g, int nfloat) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    TmaPlan p;
    if (g.nx % 8 != 0) return p;
    const size_t row = (size_t)(Q + QT) * g.nx * sizeof(S) + (size_t)nfloat * g.nx * sizeof(float);
    if (row > PP::max_stage) return p;
    // tiles cover the interior rows j = 1..ny-2 (and k = 1..nz-2 in 3D); face cells are
    // updated after the tiles with the scalar boundary pull
    const int rows_in = g.ny - 2, planes_in = D == 3 ? g.nz - 2 : 1;
    if (rows_in < 1 || planes_in < 1 || g.nx < 3) return p;
    int R = (int)(PP::budget / row);
    if (R < 1) R = 1;
    if (R > rows_in) R = rows_in;
    p.R = R;
    p.stage = (unsigned)(((size_t)R * row + 127) / 128 * 128);
    p.smem = kHeader + PP::stages * p.stage;
    p.ntj = (rows_in + R - 1) / R;
    p.ntiles = (long long)p.ntj * planes_in;
    static int sms = 0;
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    });
    const long long want = (long long)PP::blocks * sms;
    p.grid = (int)(p.ntiles < want ? p.ntiles : want);
    p.ok = true;
    return p;
}

// Tile t: plane k, rows j0 .. j0+rows-1 (interior rows only).
template <int D>
__device__ __forceinline__ void tile_rows(const Geo& g, long long t, int R, int ntj, int& k, int& j0, int& rows) {
    k = (int)(t / ntj) + (D == 3 ? 1 : 0);
    j0 = 1 + (int)(t % ntj) * R;
    const int left = (g.ny - 1) - j0;  // interior rows from j0 to ny-2
    rows = left < R ? left : R;
}

// Number of face cells (on the lattice's outer faces) and the cell of face index f:
// x faces (i = 0, nx-1; all j, k), then y faces (j = 0, ny-1; i = 1..nx-2; all k), then
// in 3D the z faces (k = 0, nz-1; i = 1..nx-2, j = 1..ny-2).
template <int D>
__device__ __forceinline__ long long face_count(const Geo& g) {
    const long long nx = g.nx, ny = g.ny, nz = g.nz;
    long long c = 2 * ny * nz + 2 * (nx - 2) * nz;
    if (D == 3) c += 2 * (nx - 2) * (ny - 2);
    return c;
}
template <int D>
__device__ __forceinline__ void face_cell(const Geo& g, long long f, int& i, int& j, int& k) {
    const long long nx = g.nx, ny = g.ny, nz = g.nz;
    const long long nxf = 2 * ny * nz, nyf = 2 * (nx - 2) * nz;
    if (f < nxf) {
        i = (f & 1) ? g.nx - 1 : 0;
        const long long r = f >> 1;
        j = (int)(r % ny);
        k = (int)(r / ny);
        return;
    }
    f -= nxf;
    if (f < nyf) {
        j = (f & 1) ? g.ny - 1 : 0;
        const long long r = f >> 1;
        i = 1 + (int)(r % (nx - 2));
        k = (int)(r / (nx - 2));
        return;
    }
    f -= nyf;
    k = (f & 1) ? g.nz - 1 : 0;
    const long long r = f >> 1;
    i = 1 + (int)(r % (nx - 2));
    j = 1 + (int)(r / (nx - 2));
}

// Issue the bulk copies of tile t into stage buffer `st`: called by all 32 lanes of one
// warp, lane l issuing copy l (the Q + QT population rows, then the float rows).  Lane 0
// announces the byte count of the whole tile on the mbarrier before any copy is issued;
// the phase completes when every byte has landed.
template <int D, class S, int LF, int LG>
__device__ __forceinline__ void issue_tile(const Geo& g, long long t, int R, int ntj, unsigned char* st, uint64_t* bar,
                                           const S* __restrict__ fsrc, const S* __restrict__ gsrc, const float* fl0,
                                           const float* fl1, const float* fl2, int nfloat) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    static_assert(Q + QT + 3 <= 32, "one lane per copy");
    const int lane = (int)(threadIdx.x & 31);
    const int nx = g.nx, ny = g.ny;
    const long long n = g.ncell;
    int k, j0, rows;
    tile_rows<D>(g, t, R, ntj, k, j0, rows);
    const size_t rc = (size_t)R * nx;
    S* sf = reinterpret_cast<S*>(st);
    S* sg = sf + Q * rc;
    float* sfl = reinterpret_cast<float*>(sg + QT * rc);
    // interior rows: every source row (j - ey, k - ez) lies inside the lattice
    const void* src = nullptr;
    void* dst = nullptr;
    unsigned bytes = 0;
    if (lane < Q + QT) {
        const bool th = lane >= Q;
        const int b = th ? lane - Q : lane;
        const int mode = th ? LG : LF;
        const int ey = mode == kRowLocal ? 0 : (th ? Lat<QT>::ey(b) : Lat<Q>::ey(b));
        const int ez = mode == kRowLocal ? 0 : (th ? Lat<QT>::ez(b) : Lat<Q>::ez(b));
        const int plane = mode == kRowSwap ? (th ? Lat<QT>::opp(b) : Lat<Q>::opp(b)) : b;
        const long long row0 = (long long)nx * ((long long)(j0 - ey) + (long long)ny * (long long)(k - ez));
        src = (th ? gsrc : fsrc) + (long long)plane * n + row0;
        dst = (th ? sg : sf) + (size_t)b * rc;
        bytes = (unsigned)((size_t)rows * nx * sizeof(S));
    } else if (lane < Q + QT + nfloat) {
        const int q = lane - (Q + QT);
        const float* base = q == 0 ? fl0 : (q == 1 ? fl1 : fl2);
        src = base + (long long)nx * ((long long)j0 + (long long)ny * k);
        dst = sfl + (size_t)q * rc;
        bytes = (unsigned)((size_t)rows * nx * sizeof(float));
    }
    unsigned total = bytes;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xFFFFFFFFu, total, o);
    if (lane == 0) mbar_arrive_expect(bar, total);
    __syncwarp();
    if (bytes) bulk_load(dst, src, bytes, bar);
}

// Slot of direction a's new value for interior cell c.
template <int Q, int ST>
__device__ __forceinline__ long long store_index(const Geo& g, int a, long long c, long long n) {
    if (ST == kStoreOpp) return (long long)Lat<Q>::opp(a) * n + c;
    if (ST == kStorePush)
        return (long long)a * n + c + (long long)Lat<Q>::ex(a) +
               (long long)g.nx * ((long long)Lat<Q>::ey(a) + (long long)g.ny * (long long)Lat<Q>::ez(a));
    return (long long)a * n + c;
}

// KIND 0: flow collision (flow_cell_2k, not FIRST); KIND 1: thermal (thermal_cell_2k).
// LF / LG: row modes of f and g; ST: store mode (kRow* / kStore* above).  In the in-place
// pattern `out` is the swept array itself (fin for the flow, gin for the thermal kernel):
// no value a cell loads is stored in the same sweep by another cell (lbm_fast_aa.cuh).
template <int D, class S, int KIND, class PP, int LF = kRowPull, int LG = kRowPull, int ST = kStoreOut>
__global__ void __launch_bounds__(PP::threads, PP::blocks)
    k_fast_tma(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fin, const S* __restrict__ gin,
               S* __restrict__ out, int R, int ntj, long long ntiles, unsigned stage_bytes, int* err, AAExtra<S> X) {
    constexpr int kThreads = PP::threads, kStages = PP::stages, kWarps = PP::warps;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    constexpr int NF = KIND == 0 ? 1 : 3;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem);  // full: the stage's copies have landed
    uint64_t* empty = bars + kStages;                    // empty: every warp has read the stage
    unsigned char* buf = smem + kHeader;
    const int nx = g.nx, ny = g.ny;
    const long long n = g.ncell;
    const size_t rc = (size_t)R * nx;
    // float rows staged with the populations
    const float* fl0 = KIND == 0 ? A.lag_in : A.Bin0;
    const float* fl1 = KIND == 0 ? nullptr : A.Bin1;
    const float* fl2 = KIND == 0 ? nullptr : (D == 3 ? A.Bin2 : A.lag_in);
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&bars[s], 1);
            mbar_init(&empty[s], kWarps);
        }
        mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        for (int s = 0; s < kStages - 1; ++s) {
            const long long t = blockIdx.x + (long long)s * gridDim.x;
            if (t < ntiles)
                issue_tile<D, S, LF, LG>(g, t, R, ntj, buf + (size_t)s * stage_bytes, &bars[s], fin, gin, fl0, fl1, fl2, NF);
        }
    }
    long long it = 0;
    for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
        const int s = (int)(it % kStages);
        if (threadIdx.x < 32) {
            // refill the stage of tile it-1 with tile it+kStages-1 once every warp released it
            const long long tn = t + (long long)(kStages - 1) * gridDim.x;
            const int sn = (int)((it + kStages - 1) % kStages);
            if (tn < ntiles) {
                if (it >= 1 && !mbar_wait(&empty[sn], (unsigned)(((it - 1) / kStages) & 1), err)) return;
                fence_async_shared();
                issue_tile<D, S, LF, LG>(g, tn, R, ntj, buf + (size_t)sn * stage_bytes, &bars[sn], fin, gin, fl0, fl1, fl2,
                                         NF);
            }
        }
        if (!mbar_wait(&bars[s], (unsigned)((it / kStages) & 1), err)) {
            mbar_drain(&bars[s], (unsigned)((it / kStages) & 1));
            return;
        }
        const unsigned char* st = buf + (size_t)s * stage_bytes;
        const S* sf = reinterpret_cast<const S*>(st);
        const S* sg = sf + Q * rc;
        const float* sfl = reinterpret_cast<const float*>(sg + QT * rc);
        int k, j0, rows;
        tile_rows<D>(g, t, R, ntj, k, j0, rows);
        const int nin = nx - 2;  // interior cells i = 1..nx-2 of a row
        for (int ci = threadIdx.x; ci < rows * nin; ci += kThreads) {
            const int r = ci / nin, i = 1 + (ci - r * nin), j = j0 + r;
            const long long c = (long long)i + (long long)nx * ((long long)j + (long long)ny * k);
            float d[Q];
#pragma unroll
            for (int a = 0; a < Q; ++a) d[a] = s2f(sf[a * rc + (size_t)r * nx + (i - (LF == kRowLocal ? 0 : Lat<Q>::ex(a)))]);
            if (KIND == 0) {
                float ts = 0.0f;
#pragma unroll
                for (int a = 0; a < QT; ++a) ts += s2f(sg[a * rc + (size_t)r * nx + (i - (LG == kRowLocal ? 0 : Lat<QT>::ex(a)))]);
                const float T = ts + P.Tref;
                float dr, rho, u, v, w = 0.0f, Fm;
                fmacro<D>(d, sfl[(size_t)r * nx + i], P, dr, rho, u, v, w, Fm);
                const float Fy = rho * P.gBeta * (T - P.Tref);
                float dp[Q];
                if (D == 2) {
                    A.lag_out[c] = Fy;
                    fcollide_2d(d, dr, rho, u, v, Fy, P, dp);
                } else {
                    fcollide_3d(d, dr, rho, u, v, w, Fy, P, dp);
                }
                S hs[Q];
                round_cell<Q>(dp, hs, P.sr != 0, sr_seed(*A.tick, c, 0));
#pragma unroll
                for (int a = 0; a < Q; ++a) out[store_index<Q, ST>(g, a, c, n)] = hs[a];
            } else {
                float G[QT], GP[QT], ts = 0.0f;
#pragma unroll
                for (int a = 0; a < QT; ++a) {
                    G[a] = s2f(sg[a * rc + (size_t)r * nx + (i - (LG == kRowLocal ? 0 : Lat<QT>::ex(a)))]) + wT<QT>(P, a) * P.Tref;
                    ts += G[a];
                }
                const size_t e = (size_t)r * nx + i;
                float dr, rho, u, v, w, Fy;
                fmacro<D>(d, D == 2 ? sfl[2 * rc + e] : ts, P, dr, rho, u, v, w, Fy);
                if (D == 2) {
                    float Bx = sfl[e], By = sfl[rc + e];
                    fcollideT_2d(G, u, v, ts, Bx, By, P, GP);
                    A.Bout0[c] = Bx;
                    A.Bout1[c] = By;
                } else {
                    float Bx = sfl[e], By = sfl[rc + e], Bz = sfl[2 * rc + e];
                    fcollideT_3d(G, u, v, w, ts, Bx, By, Bz, P, GP);
                    A.Bout0[c] = Bx;
                    A.Bout1[c] = By;
                    A.Bout2[c] = Bz;
                    A.lag_out[c] = ts;
                }
                float ev[QT];
                S hs[QT];
#pragma unroll
                for (int a = 0; a < QT; ++a) ev[a] = GP[a] - wT<QT>(P, a) * P.Tref;
                round_cell<QT>(ev, hs, P.sr != 0, sr_seed(*A.tick, c, 1));
#pragma unroll
                for (int a = 0; a < QT; ++a) out[store_index<QT, ST>(g, a, c, n)] = hs[a];
            }
        }
        __syncwarp();
        if ((threadIdx.x & 31) == 0) mbar_arrive(&empty[s]);  // this warp is done with stage s
    }
    // face cells: the one-cell path with the reference's boundary rule (global loads)
    const long long nf = face_count<D>(g);
    for (long long f = (long long)blockIdx.x * kThreads + threadIdx.x; f < nf; f += (long long)gridDim.x * kThreads) {
        int i, j, k;
        face_cell<D>(g, f, i, j, k);
        const long long c = (long long)i + (long long)nx * ((long long)j + (long long)ny * k);
        if (ST == kStoreOut) {
            if (KIND == 0) flow_cell_2k<D, false, S, false>(g, P, A, fin, gin, out, c, i, j, k);
            else thermal_cell_2k<D, false, S, false>(g, P, A, fin, gin, out, c, i, j, k);
        } else if (KIND == 0) {
            aa_flow_cell<D, S, ST == kStorePush, false>(g, P, A, out, gin, X.face, X.opar, X.graw, c, i, j, k);
        } else {
            aa_thermal_cell<D, S, ST == kStorePush, false>(g, P, A, fin, out, X.face, X.opar, X.graw, c, i, j, k);
        }
    }
}

template <int D, class S, int KIND, class PP, int LF = kRowPull, int LG = kRowPull, int ST = kStoreOut>
static bool launch_tma(const Geo& g, const PhysF& pf, const FastArgs<S>& A, const S* fin, const S* gin, S* out,
                       int* err, cudaStream_t s, AAExtra<S> X = AAExtra<S>{}) {
    const TmaPlan p = tma_plan<D, S, PP>(g, KIND == 0 ? 1 : 3);
    if (!p.ok) return false;
    static bool configured = false;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!configured) {
            if (cudaFuncSetAttribute(k_fast_tma<D, S, KIND, PP, LF, LG, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(kHeader + PP::stages * PP::max_stage)) != cudaSuccess)
                return false;
            configured = true;
        }
    }
    k_fast_tma<D, S, KIND, PP, LF, LG, ST><<<p.grid, PP::threads, p.smem, s>>>(g, pf, A, fin, gin, out, p.R, p.ntj,
                                                                                p.ntiles, p.stage, err, X);
    return true;
}

bool fast_tma_supported(const Geo& g, int dim, int precision) {
    if (dim == 2)
        return precision == LBM_FP16 ? tma_plan<2, __half, PipeA>(g, 3).ok : tma_plan<2, float, PipeA>(g, 3).ok;
    return precision == LBM_FP16 ? tma_plan<3, __half, PipeA>(g, 3).ok : tma_plan<3, float, PipeA>(g, 3).ok;
}

// One non-first two-kernel step (part: 0 flow, 1 thermal, 2 both) with staged rows.
// Returns false (nothing launched) when the geometry does not qualify.
template <class S, class PP>
static bool step_tma_s(FastState& F, const Geo& g, const PhysF& pf, int dim, const FastArgs<S>& Af,
                       const FastArgs<S>& At, const S* fin, const S* gin, S* fout, S* gout, cudaStream_t s, int part) {
    const bool fl = part != 1, th = part != 0;
    if (dim == 2) {
        if (fl && !launch_tma<2, S, 0, PP>(g, pf, Af, fin, gin, fout, F.err, s)) return false;
        if (th && !launch_tma<2, S, 1, PP>(g, pf, At, fout, gin, gout, F.err, s)) return false;
    } else {
        if (fl && !launch_tma<3, S, 0, PP>(g, pf, Af, fin, gin, fout, F.err, s)) return false;
        if (th && !launch_tma<3, S, 1, PP>(g, pf, At, fout, gin, gout, F.err, s)) return false;
    }
    return true;
}

bool fast_step_tma(FastState& F, const Geo& g, const PhysF& pf, int dim, const void* Af, const void* At,
                   const void* fin, const void* gin, void* fout, void* gout, cudaStream_t s, int part) {
    if (F.precision == LBM_FP16)
        return step_tma_s<__half, PipeA>(F, g, pf, dim, *(const FastArgs<__half>*)Af, *(const FastArgs<__half>*)At,
                                         (const __half*)fin, (const __half*)gin, (__half*)fout, (__half*)gout, s, part);
    return step_tma_s<float, PipeA>(F, g, pf, dim, *(const FastArgs<float>*)Af, *(const FastArgs<float>*)At,
                                    (const float*)fin, (const float*)gin, (float*)fout, (float*)gout, s, part);
}

// In-place pattern, one sweep of the flow (part 0) or thermal (part 1) array with staged
// rows, when both arrays have the layouts of an ordinary step (flow sweep: g in the same
// layout as f; thermal sweep: f one layout ahead of g).  Returns false (nothing launched)
// otherwise or when the geometry does not qualify.
template <int D, class S>
static bool aa_tma_s(FastState& F, const Geo& g, const PhysF& pf, const FastArgs<S>& A, int part, cudaStream_t s) {
    const AAState& st = F.AA;
    S* f = (S*)F.fbuf[0];
    S* gg = (S*)F.gbuf[0];
    if (part == 0) {
        if (st.gpar != st.fpar) return false;
        const AAExtra<S> X{AAFace<S>{(const S*)st.face_f[0], (const S*)st.face_f[1], (const S*)st.face_f[2]}, st.gpar,
                           st.graw ? 1 : 0};
        if (st.fpar) return launch_tma<D, S, 0, PipeA, kRowSwap, kRowSwap, kStorePush>(g, pf, A, f, gg, f, F.err, s, X);
        return launch_tma<D, S, 0, PipeA, kRowLocal, kRowLocal, kStoreOpp>(g, pf, A, f, gg, f, F.err, s, X);
    }
    if (st.fpar == st.gpar) return false;
    const AAExtra<S> X{AAFace<S>{(const S*)st.face_g[0], (const S*)st.face_g[1], (const S*)st.face_g[2]}, st.fpar,
                       st.graw ? 1 : 0};
    if (st.gpar) return launch_tma<D, S, 1, PipeA, kRowLocal, kRowSwap, kStorePush>(g, pf, A, f, gg, gg, F.err, s, X);
    return launch_tma<D, S, 1, PipeA, kRowSwap, kRowLocal, kStoreOpp>(g, pf, A, f, gg, gg, F.err, s, X);
}

bool fast_aa_tma_sweep(FastState& F, const Geo& g, const PhysF& pf, int dim, const void* A, int part, cudaStream_t s) {
    if (dim != 3) return false;
    if (F.precision == LBM_FP16) return aa_tma_s<3, __half>(F, g, pf, *(const FastArgs<__half>*)A, part, s);
    return aa_tma_s<3, float>(F, g, pf, *(const FastArgs<float>*)A, part, s);
}

// Self-test of the bounded wait and its error report: one warp arms an mbarrier for 128
// bytes that no copy will deliver (no copy is issued, so nothing is in flight when the block
// exits), waits with the given iteration limit, and sets the error flag of the handle's
// staged kernels, which the next lbm_sync reports as LBM_ERR_TIMEOUT.
__global__ void k_wait_selftest(int* err, unsigned limit) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_arrive_expect(&bar, 128u);
    __syncthreads();
    mbar_wait(&bar, 0u, err, limit);
}

void fast_wait_selftest(FastState& F, unsigned limit, cudaStream_t s) { k_wait_selftest<<<1, 32, 0, s>>>(F.err, limit); }

}  // namespace lbm
