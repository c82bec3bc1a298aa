// lbm_fast.cu - the reduced-storage forms: FP32 or FP16 populations (deviations from the
// rest state), FP32 arithmetic, FMA contraction allowed.
//
// This unit holds the two-kernel step (used for the first step after `initial` or a
// state load, and to enter the single-kernel mode of lbm_fused.cu), the materialisation
// of the module arrays, and the conversions to and from the reference's FP64 layout.
// The moment space is the reference's: the forward transform is its integer matrix
// applied to the deviations, the relaxation acts on non-equilibrium moments
// m_k - meq_k = M_k d - (meq_k(rho,u) - meq_k(1,0)), and the inverse transform is its
// M^-1 with the divisions by constants turned into multiplications.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lbm_fast.h"
#include "lbm_fast_cells.cuh"
#include "lbm_fast_pairs.cuh"

namespace lbm {

template <class S>
static FastArgs<S> args_for(const FastState& F, int bin, int bout, int lin, int lout) {
    FastArgs<S> a;
    a.fref = (S*)F.fref;
    a.gref = (S*)F.gref;
    a.rho = F.rho; a.u = F.u; a.v = F.v; a.w = F.w; a.T = F.T;
    a.Bin0 = F.B[bin][0]; a.Bin1 = F.B[bin][1]; a.Bin2 = F.B[bin][2];
    a.Bout0 = F.B[bout][0]; a.Bout1 = F.B[bout][1]; a.Bout2 = F.B[bout][2];
    a.lag_in = F.L[lin];
    a.lag_out = F.L[lout];
    a.tick = F.tick;
    return a;
}

// ------------------------------------------------------------------------------------
// kernels
// ------------------------------------------------------------------------------------
template <int D, class S>
__global__ void k_fast_initial(Geo g, PhysF P, InitC I, FastArgs<S> A) {
    long long c;
    int i, j, k;
    if (!fcell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const double xpi = ((double)(i + 1) - 0.5) / I.L, yp_j = ((double)(j + 1) - 0.5) / I.L;
    const double xpe = (double)g.nx / I.L, ype = (double)g.ny / I.L;
    double T = 0.0;
    if (g.bct[0] == LBM_BCT_CONST) T = I.Thot + xpi / xpe * (I.Tcold - I.Thot);
    if (g.bct[1] == LBM_BCT_CONST) {
        T = I.Thot + yp_j / ype * (I.Tcold - I.Thot);
        if (I.perturb) T = T + I.pert_amp * I.sx[i] * I.sy[j];
    }
    if (I.noise_amp != 0.0) T = T + I.noise_amp * (2.0 * noise_xi(I.seed, (uint64_t)c) - 1.0);
    const long long n = g.ncell;
#pragma unroll
    for (int a = 0; a < Q; ++a) A.fref[a * n + c] = toS<S>(0.0f);  // f = w at rest
#pragma unroll
    for (int a = 0; a < QT; ++a)
        A.gref[a * n + c] = toS<S>((float)((a == 0 ? (double)P.omegaT0 : (double)P.omegaT1) * (T - (double)P.Tref)));
    A.rho[c] = 1.0f;
    A.u[c] = 0.0f;
    A.v[c] = 0.0f;
    if (D == 3) A.w[c] = 0.0f;
    A.T[c] = (float)T;
    A.Bout0[c] = 0.0f;
    A.Bout1[c] = 0.0f;
    if (D == 3) A.Bout2[c] = 0.0f;
    A.lag_out[c] = 0.0f;
}

// Flow collision and thermal kernels of the two-kernel step (bodies in lbm_fast_cells.cuh).
// I: int when every array index fits in 32 bits (the divisions of the cell index and the
// address arithmetic in 32 bits), else long long.
template <int D, bool FIRST, class S, class I>
__global__ void __launch_bounds__(128, (OneCellBlocks<S, false>::value)) k_fast_flow(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fin,
                                                   const S* __restrict__ gin, S* __restrict__ fout) {
    I c;
    int i, j, k;
    if (!fcell_i<I>(g, c, i, j, k)) return;
    flow_cell_2k<D, FIRST, S, true, I>(g, P, A, fin, gin, fout, c, i, j, k);
}

template <int D, bool FIRST, class S, class I>
__global__ void __launch_bounds__(128, (OneCellBlocks<S, true>::value)) k_fast_thermal(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fin,
                                                      const S* __restrict__ gin, S* __restrict__ gout) {
    I c;
    int i, j, k;
    if (!fcell_i<I>(g, c, i, j, k)) return;
    thermal_cell_2k<D, FIRST, S, true, I>(g, P, A, fin, gin, gout, c, i, j, k);
}

// Paired form of the two kernels (lbm_fast_pairs.cuh): thread (x, y) of a block holds the
// cells 2t and 2t+1 of row (j, k); blockDim.x * blockDim.y = 128.  nx even.
__device__ __forceinline__ bool pair_cell(const Geo& g, long long& c0, int& i0, int& j, int& k) {
    i0 = 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    k = (int)blockIdx.z;
    if (i0 >= g.nx || j >= g.ny) return false;
    c0 = (long long)i0 + (long long)g.nx * ((long long)j + (long long)g.ny * (long long)k);
    return true;
}

template <int D, class S>
__global__ void __launch_bounds__(128) k_fast_flow_pair(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fin,
                                                        const S* __restrict__ gin, S* __restrict__ fout) {
    long long c0;
    int i0, j, k;
    if (!pair_cell(g, c0, i0, j, k)) return;
    flow_pair_2k<D, S>(g, P, A, fin, gin, fout, c0, i0, j, k);
}

template <int D, class S>
__global__ void __launch_bounds__(128) k_fast_thermal_pair(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fin,
                                                           const S* __restrict__ gin, S* __restrict__ gout) {
    long long c0;
    int i0, j, k;
    if (!pair_cell(g, c0, i0, j, k)) return;
    thermal_pair_2k<D, S>(g, P, A, fin, gin, gout, c0, i0, j, k);
}

// Block shape of the paired kernels: as many pairs of a row as fit in 64 threads.
static void pair_launch(const Geo& g, dim3& grid, dim3& block) {
    const int pairs = g.nx / 2;
    const int bx = pairs > 32 ? 64 : 32;
    const int by = 128 / bx;
    block = dim3(bx, by, 1);
    grid = dim3((pairs + bx - 1) / bx, (g.ny + by - 1) / by, g.nz);
}

// Row form of the two kernels (option LBM_OPT_ROWS): interior rows with the select-based x
// rule (flow_cell_row / thermal_cell_row), face rows with the full boundary rule; no
// division of a cell index, and no per-cell choice between a fixed-offset and a boundary
// path.  Same values as the one-cell kernels bit for bit.
template <int D, class S>
__global__ void __launch_bounds__(128, (OneCellBlocks<S, false>::value)) k_fast_flow_rows(Geo g, PhysF P, FastArgs<S> A,
                                                                                         const S* __restrict__ fin,
                                                                                         const S* __restrict__ gin,
                                                                                         S* __restrict__ fout) {
    long long c;
    int i, j, k;
    if (!row_interior_cell(g, c, i, j, k)) return;
    flow_cell_row<D, S>(g, P, A, fin, gin, fout, c, i);
}

template <int D, class S>
__global__ void __launch_bounds__(128, (OneCellBlocks<S, true>::value)) k_fast_thermal_rows(Geo g, PhysF P, FastArgs<S> A,
                                                                                           const S* __restrict__ fin,
                                                                                           const S* __restrict__ gin,
                                                                                           S* __restrict__ gout) {
    long long c;
    int i, j, k;
    if (!row_interior_cell(g, c, i, j, k)) return;
    thermal_cell_row<D, S>(g, P, A, fin, gin, gout, c, i);
}

template <int D, class S>
__global__ void __launch_bounds__(128) k_fast_flow_facerows(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fin,
                                                            const S* __restrict__ gin, S* __restrict__ fout) {
    long long c;
    int i, j, k;
    if (!row_face_cell(g, c, i, j, k)) return;
    flow_cell_2k<D, false, S, false>(g, P, A, fin, gin, fout, c, i, j, k);
}

template <int D, class S>
__global__ void __launch_bounds__(128) k_fast_thermal_facerows(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fin,
                                                               const S* __restrict__ gin, S* __restrict__ gout) {
    long long c;
    int i, j, k;
    if (!row_face_cell(g, c, i, j, k)) return;
    thermal_cell_2k<D, false, S, false>(g, P, A, fin, gin, gout, c, i, j, k);
}

// idx32: every array index fits in 32 bits.  Measured on GB300 (256^3 and 384^3): 32-bit
// indices speed up both FP16 kernels (2%) and the FP32 thermal kernel (1-1.5%); the FP32
// flow kernel takes 64 registers instead of 56 with them and runs 5-6% slower, so it keeps
// 64-bit indices.
template <int D, bool FIRST, class S>
static void one_cell_step(bool idx32, unsigned blocks, const Geo& g, const PhysF& pf, const FastArgs<S>& Af,
                          const FastArgs<S>& At, const S* fin, const S* gin, S* fout, S* gout, cudaStream_t s, bool fl,
                          bool th) {
    const bool flow32 = idx32 && sizeof(S) == 2;
    if (fl && flow32) k_fast_flow<D, FIRST, S, int><<<blocks, 128, 0, s>>>(g, pf, Af, fin, gin, fout);
    else if (fl) k_fast_flow<D, FIRST, S, long long><<<blocks, 128, 0, s>>>(g, pf, Af, fin, gin, fout);
    if (th && idx32) k_fast_thermal<D, FIRST, S, int><<<blocks, 128, 0, s>>>(g, pf, At, fout, gin, gout);
    else if (th) k_fast_thermal<D, FIRST, S, long long><<<blocks, 128, 0, s>>>(g, pf, At, fout, gin, gout);
}

template <int D, class S>
static void rows_step(const Geo& g, const PhysF& pf, const FastArgs<S>& Af, const FastArgs<S>& At, const S* fin,
                      const S* gin, S* fout, S* gout, cudaStream_t s, bool fl, bool th) {
    const unsigned bx = (unsigned)((g.nx + 127) / 128);
    const dim3 gin_grid(bx, (unsigned)(g.ny - 2), D == 3 ? (unsigned)(g.nz - 2) : 1u);
    const dim3 gface(bx, (unsigned)face_row_count(g), 1u);
    if (fl) {
        k_fast_flow_rows<D, S><<<gin_grid, 128, 0, s>>>(g, pf, Af, fin, gin, fout);
        k_fast_flow_facerows<D, S><<<gface, 128, 0, s>>>(g, pf, Af, fin, gin, fout);
    }
    if (th) {
        k_fast_thermal_rows<D, S><<<gin_grid, 128, 0, s>>>(g, pf, At, fout, gin, gout);
        k_fast_thermal_facerows<D, S><<<gface, 128, 0, s>>>(g, pf, At, fout, gin, gout);
    }
}

// Module arrays of step N from F[cur] = f_post_N, G[cur] = g_post_N, L[cur] (lag_in).
template <int D, class S>
__global__ void k_fast_materialize(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fin,
                                   const S* __restrict__ gin) {
    long long c;
    int i, j, k;
    if (!fcell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    float d[Q];
    auto lf = [&](int a, long long cc) { return ldS(fin, a * n + cc); };
    auto lg = [&](int a, long long cc) { return ldS(gin, a * n + cc); };
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        d[a] = pull_flow<Q, float>(g, a, i, j, k, c, lf);
        A.fref[a * n + c] = toS<S>(d[a]);
    }
    float ts = 0.0f;
#pragma unroll
    for (int a = 0; a < QT; ++a) {
        const float e = pull_thermal<QT, float>(g, a, i, j, k, c, lg);
        A.gref[a * n + c] = toS<S>(e);
        ts += e + wT<QT>(P, a) * P.Tref;
    }
    float dr, rho, u, v, w, Fy;
    fmacro<D>(d, A.lag_in[c], P, dr, rho, u, v, w, Fy);
    A.rho[c] = rho;
    A.u[c] = u;
    A.v[c] = v;
    if (D == 3) A.w[c] = w;
    A.T[c] = ts;
}

// export / import (FP64 Fortran layout)
template <int Q, class S>
__global__ void k_export_pop(const S* __restrict__ soa, double* __restrict__ out, long long n, int thermal, double w0,
                             double w1, int out_soa) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)Q * n) return;
    const long long c = e / Q;
    const int a = (int)(e - c * Q);
    const double rest = thermal ? (a == 0 ? w0 : w1) : wrest<(Q == 9 || Q == 5) ? 9 : 19>(a);
    out[out_soa ? (long long)a * n + c : e] = rest + (double)ldS(soa, (long long)a * n + c);
}

template <int Q, class S>
__global__ void k_import_pop(const double* __restrict__ in, S* __restrict__ soa, long long n, int thermal, double w0,
                             double w1, int in_soa) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)Q * n) return;
    const long long c = e / Q;
    const int a = (int)(e - c * Q);
    const double rest = thermal ? (a == 0 ? w0 : w1) : wrest<(Q == 9 || Q == 5) ? 9 : 19>(a);
    soa[(long long)a * n + c] = toS<S>((float)(in[in_soa ? (long long)a * n + c : e] - rest));
}

__global__ void k_f2d(const float* __restrict__ x, double* __restrict__ y, long long n) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) y[e] = x ? (double)x[e] : 0.0;
}

__global__ void k_d2f(const double* __restrict__ x, float* __restrict__ y, long long n) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) y[e] = (float)x[e];
}

__global__ void k_tick(unsigned long long* t) { *t += 1ULL; }

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
static inline unsigned nb(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

PhysF fast_physf(const FastState& F, const PhysC& P) {
    PhysF pf = to_physf(P);
    pf.sr = (F.sr && F.precision == LBM_FP16) ? 1 : 0;
    return pf;
}

void fast_tick(FastState& F, cudaStream_t s) { k_tick<<<1, 1, 0, s>>>(F.tick); }

int fast_allocate(FastState& F, const lbm_params& p, const Geo& g, const AllocFn& alloc) {
    F.precision = p.precision;
    // Measured on GB300 (3D cubes 128^3 and 384^3; 2D 256 x 128 to 4096 x 2048): with the
    // boundary tests confined to the face cells, one cell per thread is the fastest form
    // for 3D in both storage types (FP16 17.3 G cell updates/s at 384^3 against 13.0 G for
    // the staged rows) and for 2D FP16; 2D FP32 is fastest with two cells per thread.  The
    // staged and paired forms stay selectable (LBM_OPT_STAGED, LBM_OPT_PAIRS).
    F.tma = false;
    F.pairs = p.dim == 2 && p.precision == LBM_FP32;
    F.dim = p.dim;
    F.q = p.dim == 3 ? 19 : 9;
    F.qt = p.dim == 3 ? 7 : 5;
    F.esize = p.precision == LBM_FP16 ? 2 : 4;
    const long long n = g.ncell;
    F.aa = p.pattern == LBM_PATTERN_AA;
    F.AA = AAState{};
    int st;
    const int nbuf = F.aa ? 1 : 2;
    for (int b = 0; b < nbuf; ++b) {
        if ((st = alloc(&F.fbuf[b], F.esize * F.q * n)) != LBM_OK) return st;
        if ((st = alloc(&F.gbuf[b], F.esize * F.qt * n)) != LBM_OK) return st;
        for (int c = 0; c < (p.dim == 3 ? 3 : 2); ++c)
            if ((st = alloc((void**)&F.B[b][c], sizeof(float) * n)) != LBM_OK) return st;
        if ((st = alloc((void**)&F.L[b], sizeof(float) * n)) != LBM_OK) return st;
    }
    if ((st = alloc((void**)&F.err, sizeof(int))) != LBM_OK) return st;
    if (cudaMemset(F.err, 0, sizeof(int)) != cudaSuccess) return LBM_ERR_CUDA;
    if ((st = alloc((void**)&F.tick, sizeof(unsigned long long))) != LBM_OK) return st;
    if (cudaMemset(F.tick, 0, sizeof(unsigned long long)) != cudaSuccess) return LBM_ERR_CUDA;
    F.sr = p.precision == LBM_FP16;
    if (F.aa) {
        // one array each, which is also the module array; the lag fields are read and
        // written by the same thread, so one buffer serves both parities
        F.fref = F.fbuf[0];
        F.gref = F.gbuf[0];
        // in-place defaults (lbm_fast_aa.cu): one cell per thread except the even flow sweep
        F.pairs = false;
        F.tma = false;
        for (int c = 0; c < 3; ++c) F.B[1][c] = F.B[0][c];
        F.L[1] = F.L[0];
        for (int ax = 0; ax < 3; ++ax) {
            if (g.bcf[ax] == LBM_BC_PERIODIC && (st = alloc(&F.AA.face_f[ax], F.esize * F.q * aa_face_cells(g, ax))) != LBM_OK)
                return st;
            if (g.bct[ax] == LBM_BCT_PERIODIC && (st = alloc(&F.AA.face_g[ax], F.esize * F.qt * aa_face_cells(g, ax))) != LBM_OK)
                return st;
        }
    } else {
        if ((st = alloc(&F.fref, F.esize * F.q * n)) != LBM_OK) return st;
        if ((st = alloc(&F.gref, F.esize * F.qt * n)) != LBM_OK) return st;
    }
    float** scal[] = {&F.rho, &F.u, &F.v, &F.T, &F.up, &F.vp, &F.Tp};
    for (float** s : scal)
        if ((st = alloc((void**)s, sizeof(float) * n)) != LBM_OK) return st;
    if (p.dim == 3) {
        float** s3[] = {&F.w, &F.wp};
        for (float** s : s3)
            if ((st = alloc((void**)s, sizeof(float) * n)) != LBM_OK) return st;
    }
    F.fused_valid = false;
    F.ahead = false;
    F.cur = 0;
    return LBM_OK;
}

#define DISPATCH_S(F, ...)                    \
    do {                                      \
        if ((F).precision == LBM_FP16) {      \
            using S = __half;                 \
            __VA_ARGS__;                      \
        } else {                              \
            using S = float;                  \
            __VA_ARGS__;                      \
        }                                     \
    } while (0)

void fast_initial(FastState& F, const Geo& g, const PhysC& P, const InitC& I, int dim, cudaStream_t s) {
    const PhysF pf = to_physf(P);
    F.cur = 0;
    F.fused_valid = false;
    F.ahead = false;
    F.AA.fpar = F.AA.gpar = 0;  // the in-place arrays now hold module data
    F.AA.graw = false;
    cudaMemsetAsync(F.tick, 0, sizeof(unsigned long long), s);
    DISPATCH_S(F, {
        FastArgs<S> A = args_for<S>(F, 0, 0, 0, 0);
        if (dim == 2) k_fast_initial<2, S><<<nb(g.ncell, 256), 256, 0, s>>>(g, pf, I, A);
        else k_fast_initial<3, S><<<nb(g.ncell, 256), 256, 0, s>>>(g, pf, I, A);
    });
    cudaMemsetAsync(F.up, 0, sizeof(float) * g.ncell, s);
    cudaMemsetAsync(F.vp, 0, sizeof(float) * g.ncell, s);
    cudaMemsetAsync(F.Tp, 0, sizeof(float) * g.ncell, s);
    if (dim == 3) cudaMemsetAsync(F.wp, 0, sizeof(float) * g.ncell, s);
}

bool fast_step_tma(FastState& F, const Geo& g, const PhysF& pf, int dim, const void* Af, const void* At,
                   const void* fin, const void* gin, void* fout, void* gout, cudaStream_t s, int part);

int fast_take_error(FastState& F, cudaStream_t s) {
    if (!F.err) return LBM_OK;
    int h = 0;
    if (cudaMemcpyAsync(&h, F.err, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return LBM_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return LBM_ERR_CUDA;
    if (h == 0) return LBM_OK;
    cudaMemsetAsync(F.err, 0, sizeof(int), s);
    return LBM_ERR_TIMEOUT;
}

void fast_step(FastState& F, const Geo& g0, const PhysC& P, int dim, bool first, cudaStream_t s, int part) {
    const PhysF pf = fast_physf(F, P);
    const Geo g = dev_geo(g0, P);
    const int cur = F.cur, nxt = F.cur ^ 1;
    if (F.aa) {
        F.ahead = false;
        fast_step_aa(F, g, pf, dim, first, s, part);
        if (part != 0) {
            fast_tick(F, s);
            F.cur = nxt;
            F.fused_valid = true;
        }
        return;
    }
    const unsigned blocks = nb(g.ncell, 128);
    const bool paired = F.pairs && g.nx % 2 == 0;
    const bool rows = F.rows && !paired && row_launch_supported(g);
    const bool idx32 = !F.wide && (long long)F.q * g.ncell < (1LL << 31);
    dim3 pgrid, pblock;
    pair_launch(g, pgrid, pblock);
    F.ahead = false;
    DISPATCH_S(F, {
        const S* fin = (const S*)F.fbuf[cur];
        const S* gin = (const S*)F.gbuf[cur];
        S* fout = (S*)F.fbuf[nxt];
        S* gout = (S*)F.gbuf[nxt];
        FastArgs<S> Af = args_for<S>(F, cur, nxt, cur, nxt);  // flow: lag_in = L[cur], lag_out = L[nxt]
        FastArgs<S> At = args_for<S>(F, cur, nxt, nxt, nxt);  // thermal: 2D reads F_y,n from L[nxt]
        const bool fl = part != 1, th = part != 0;
        if (!first && F.tma && fast_step_tma(F, g, pf, dim, &Af, &At, fin, gin, fout, gout, s, part)) {
            // staged rows (lbm_fast_tma.cu)
        } else if (dim == 2) {
            if (first) {
                one_cell_step<2, true, S>(idx32, blocks, g, pf, Af, At, fin, gin, fout, gout, s, fl, th);
            } else if (paired) {
                if (fl) k_fast_flow_pair<2, S><<<pgrid, pblock, 0, s>>>(g, pf, Af, fin, gin, fout);
                if (th) k_fast_thermal_pair<2, S><<<pgrid, pblock, 0, s>>>(g, pf, At, fout, gin, gout);
            } else if (rows) {
                rows_step<2, S>(g, pf, Af, At, fin, gin, fout, gout, s, fl, th);
            } else {
                one_cell_step<2, false, S>(idx32, blocks, g, pf, Af, At, fin, gin, fout, gout, s, fl, th);
            }
        } else {
            if (first) {
                one_cell_step<3, true, S>(idx32, blocks, g, pf, Af, At, fin, gin, fout, gout, s, fl, th);
            } else if (paired) {
                if (fl) k_fast_flow_pair<3, S><<<pgrid, pblock, 0, s>>>(g, pf, Af, fin, gin, fout);
                if (th) k_fast_thermal_pair<3, S><<<pgrid, pblock, 0, s>>>(g, pf, At, fout, gin, gout);
            } else if (rows) {
                rows_step<3, S>(g, pf, Af, At, fin, gin, fout, gout, s, fl, th);
            } else {
                one_cell_step<3, false, S>(idx32, blocks, g, pf, Af, At, fin, gin, fout, gout, s, fl, th);
            }
        }
    });
    if (part != 0) {
        fast_tick(F, s);
        F.cur = nxt;
        F.fused_valid = true;
    }
}

void fast_enter(FastState& F, const Geo& g0, const PhysC& P, int dim, cudaStream_t s) {
    // one flow collision ahead: F[cur^1] = f_post_{N+1}, 2D L[cur^1] = F_y,N+1
    fast_step(F, g0, P, dim, false, s, 0);
    F.ahead = true;
}

void fast_materialize(FastState& F, const Geo& g0, const PhysC& P, int dim, cudaStream_t s) {
    if (!F.fused_valid) return;
    const PhysF pf = to_physf(P);
    const Geo g = dev_geo(g0, P);
    if (F.aa) {
        fast_materialize_aa(F, g, pf, dim, s);
        return;
    }
    DISPATCH_S(F, {
        const S* fin = (const S*)F.fbuf[F.cur];
        const S* gin = (const S*)F.gbuf[F.cur];
        FastArgs<S> A = args_for<S>(F, F.cur, F.cur, F.cur, F.cur);
        if (dim == 2) k_fast_materialize<2, S><<<nb(g.ncell, 128), 128, 0, s>>>(g, pf, A, fin, gin);
        else k_fast_materialize<3, S><<<nb(g.ncell, 128), 128, 0, s>>>(g, pf, A, fin, gin);
    });
}

DiagFields<float> fast_diag_fields(const FastState& F) {
    return DiagFields<float>{F.u, F.v, F.w, F.T, F.rho, F.up, F.vp, F.wp, F.Tp};
}

int fast_export(const FastState& F, const Geo& g, const PhysC& P, int dim, int field, double* out, cudaStream_t s,
                bool soa) {
    const long long n = g.ncell;
    const bool d3 = dim == 3;
    const double wt0 = P.omegaT0 * P.Tref, wt1 = P.omegaT1 * P.Tref;
    if (F.aa && (field == LBM_FIELD_F || field == LBM_FIELD_G)) {
        // the module view, read through the array's layout
        const bool th = field == LBM_FIELD_G;
        aa_module_view(dev_geo(g, P), th ? F.qt : F.q, th, F.precision, th ? F.gbuf[0] : F.fbuf[0],
                       th ? F.AA.gpar : F.AA.fpar, F.AA.graw, out, soa, true, wt0, wt1, s);
        return LBM_OK;
    }
    if (F.aa && (field == LBM_FIELD_F_POST || field == LBM_FIELD_G_POST)) return LBM_ERR_STATE;
    if (field == LBM_FIELD_F || field == LBM_FIELD_F_POST || field == LBM_FIELD_G || field == LBM_FIELD_G_POST) {
        const bool th = field == LBM_FIELD_G || field == LBM_FIELD_G_POST;
        const void* src = field == LBM_FIELD_F ? F.fref : field == LBM_FIELD_G ? F.gref
                        : field == LBM_FIELD_F_POST ? F.fbuf[F.cur] : F.gbuf[F.cur];
        const int q = th ? F.qt : F.q;
        DISPATCH_S(F, {
            if (d3) {
                if (th) k_export_pop<7, S><<<nb(q * n, 256), 256, 0, s>>>((const S*)src, out, n, 1, wt0, wt1, soa);
                else k_export_pop<19, S><<<nb(q * n, 256), 256, 0, s>>>((const S*)src, out, n, 0, 0, 0, soa);
            } else {
                if (th) k_export_pop<5, S><<<nb(q * n, 256), 256, 0, s>>>((const S*)src, out, n, 1, wt0, wt1, soa);
                else k_export_pop<9, S><<<nb(q * n, 256), 256, 0, s>>>((const S*)src, out, n, 0, 0, 0, soa);
            }
        });
        return LBM_OK;
    }
    const float* src = nullptr;
    const int c = F.cur;
    switch (field) {
        case LBM_FIELD_RHO: src = F.rho; break;
        case LBM_FIELD_U: src = F.u; break;
        case LBM_FIELD_V: src = F.v; break;
        case LBM_FIELD_W: if (!d3) return LBM_ERR_PARAM; src = F.w; break;
        case LBM_FIELD_T: src = F.T; break;
        case LBM_FIELD_BX_PREV: src = F.B[c][0]; break;
        case LBM_FIELD_BY_PREV: src = F.B[c][1]; break;
        case LBM_FIELD_BZ_PREV: if (!d3) return LBM_ERR_PARAM; src = F.B[c][2]; break;
        case LBM_FIELD_FX: if (d3) return LBM_ERR_PARAM; src = nullptr; break;
        case LBM_FIELD_FY: if (d3) return LBM_ERR_PARAM; src = F.L[c]; break;
        default: return LBM_ERR_PARAM;
    }
    k_f2d<<<nb(n, 256), 256, 0, s>>>(src, out, n);
    return LBM_OK;
}

int fast_import(FastState& F, const Geo& g, const PhysC& P, int dim, int field, const double* in, cudaStream_t s,
                bool soa) {
    const long long n = g.ncell;
    const bool d3 = dim == 3;
    const double wt0 = P.omegaT0 * P.Tref, wt1 = P.omegaT1 * P.Tref;
    if (field == LBM_FIELD_F || field == LBM_FIELD_G) {
        const bool th = field == LBM_FIELD_G;
        void* dst = th ? F.gref : F.fref;
        const int q = th ? F.qt : F.q;
        DISPATCH_S(F, {
            if (d3) {
                if (th) k_import_pop<7, S><<<nb(q * n, 256), 256, 0, s>>>(in, (S*)dst, n, 1, wt0, wt1, soa);
                else k_import_pop<19, S><<<nb(q * n, 256), 256, 0, s>>>(in, (S*)dst, n, 0, 0, 0, soa);
            } else {
                if (th) k_import_pop<5, S><<<nb(q * n, 256), 256, 0, s>>>(in, (S*)dst, n, 1, wt0, wt1, soa);
                else k_import_pop<9, S><<<nb(q * n, 256), 256, 0, s>>>(in, (S*)dst, n, 0, 0, 0, soa);
            }
        });
        F.fused_valid = false;
        F.ahead = false;
        if (th) {
            F.AA.gpar = 0;  // module data in the streamed layout
            F.AA.graw = false;
        } else {
            F.AA.fpar = 0;
        }
        return LBM_OK;
    }
    float* dst = nullptr;
    const int c = F.cur;
    switch (field) {
        case LBM_FIELD_RHO: dst = F.rho; break;
        case LBM_FIELD_U: dst = F.u; break;
        case LBM_FIELD_V: dst = F.v; break;
        case LBM_FIELD_W: if (!d3) return LBM_ERR_PARAM; dst = F.w; break;
        case LBM_FIELD_T: dst = F.T; break;
        case LBM_FIELD_BX_PREV: dst = F.B[c][0]; break;
        case LBM_FIELD_BY_PREV: dst = F.B[c][1]; break;
        case LBM_FIELD_BZ_PREV: if (!d3) return LBM_ERR_PARAM; dst = F.B[c][2]; break;
        case LBM_FIELD_FY: if (d3) return LBM_ERR_PARAM; dst = F.L[c]; break;
        default: return LBM_ERR_STATE;
    }
    k_d2f<<<nb(n, 256), 256, 0, s>>>(in, dst, n);
    F.fused_valid = false;
    F.ahead = false;
    return LBM_OK;
}

}  // namespace lbm
