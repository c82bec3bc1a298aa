// lbm_fixed.cu - kernels of the fixed arithmetic of FP64 handles (lbm_params.arith =
// LBM_ARITH_FIXED): the two-kernel fused step and the materialisation of the module arrays,
// with the per-cell bodies of lbm_fixed_cell.cuh (q60 integer arithmetic on the integer
// pipes, FP64 accuracy).  The fused buffers hold q60 deviations; the module arrays stay the
// plain method's FP64 arrays, so diagnostics, state transfer and restart files are shared
// with the plain method.
#include <cuda_runtime.h>

#include "lbm_fixed.h"
#include "lbm_fixed_cell.cuh"

namespace lbm {

using namespace fxa;

// Resident blocks per SM asked of the interior flow kernel: 5 (96 registers, no spill) ran
// the kernel 8% faster on GB300 than 4 (124 registers) at 256^3 and 384^3, where the warps
// wait on their loads (long-scoreboard stalls) at half the issue rate; 6 spills.
#ifndef LBM_XFLOW_MIN_BLOCKS
#define LBM_XFLOW_MIN_BLOCKS 5
#endif
// Resident blocks per SM asked of the interior thermal kernel: 7 (70 registers, no spill)
// ran it 4% faster on GB300 than 6 (80 registers) or 8 (64) at 256^3 and 384^3, at about
// the HBM copy rate on its measured traffic.
#ifndef LBM_XTHERMAL_MIN_BLOCKS
#define LBM_XTHERMAL_MIN_BLOCKS 7
#endif

__device__ __forceinline__ bool fixed_cell_of_thread(const Geo& g, long long& c, int& i, int& j, int& k) {
    c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return false;
    cell_coords(g, c, i, j, k);
    return true;
}

template <int D, bool FIRST>
__global__ void __launch_bounds__(128) k_xflow(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                                               const long long* __restrict__ gin, long long* __restrict__ fout) {
    long long c;
    int i, j, k;
    if (!fixed_cell_of_thread(g, c, i, j, k)) return;
    flow_cell<D, FIRST>(g, X, A, fin, gin, fout, c, i, j, k);
}

template <int D, bool FIRST>
__global__ void __launch_bounds__(128) k_xthermal(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                                                  const long long* __restrict__ gin, long long* __restrict__ gout) {
    long long c;
    int i, j, k;
    if (!fixed_cell_of_thread(g, c, i, j, k)) return;
    thermal_cell<D, FIRST>(g, X, A, fin, gin, gout, c, i, j, k);
}

// Interior rows and face rows of the steady-state step: row_interior_cell and
// row_face_cell (lbm_device.cuh).  Interior rows pull with selects for the x faces; the face
// kernels take the y- and z-face rows with the full boundary rule.
// I: int when q * ncell < 2^31 (every array index fits in 32 bits), else long long.
template <int D, class I>
__global__ void __launch_bounds__(128, LBM_XFLOW_MIN_BLOCKS) k_xflow_in(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                                                     const long long* __restrict__ gin, long long* __restrict__ fout) {
    long long c;
    int i, j, k;
    if (!row_interior_cell(g, c, i, j, k)) return;
    flow_cell<D, false, 3, I>(g, X, A, fin, gin, fout, c, i, j, k);
}

template <int D>
__global__ void __launch_bounds__(128) k_xflow_face(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                                                    const long long* __restrict__ gin, long long* __restrict__ fout) {
    long long c;
    int i, j, k;
    if (!row_face_cell(g, c, i, j, k)) return;
    flow_cell<D, false, 2>(g, X, A, fin, gin, fout, c, i, j, k);
}

template <int D, class I>
__global__ void __launch_bounds__(128, LBM_XTHERMAL_MIN_BLOCKS) k_xthermal_in(Geo g, PhysX X, FixedArrays A,
                                                        const long long* __restrict__ fin,
                                                        const long long* __restrict__ gin, long long* __restrict__ gout) {
    long long c;
    int i, j, k;
    if (!row_interior_cell(g, c, i, j, k)) return;
    thermal_cell<D, false, 3, I>(g, X, A, fin, gin, gout, c, i, j, k);
}

template <int D>
__global__ void __launch_bounds__(128) k_xthermal_face(Geo g, PhysX X, FixedArrays A,
                                                       const long long* __restrict__ fin,
                                                       const long long* __restrict__ gin, long long* __restrict__ gout) {
    long long c;
    int i, j, k;
    if (!row_face_cell(g, c, i, j, k)) return;
    thermal_cell<D, false, 2>(g, X, A, fin, gin, gout, c, i, j, k);
}

template <int D>
__global__ void k_xmaterialize(Geo g, PhysX X, FixedArrays A, const long long* __restrict__ fin,
                               const long long* __restrict__ gin) {
    long long c;
    int i, j, k;
    if (!fixed_cell_of_thread(g, c, i, j, k)) return;
    materialize_cell<D>(g, X, A, fin, gin, c, i, j, k);
}

// q60 deviations of a fused buffer -> the FP64 populations they stand for, in place.
__global__ void k_xpost_to_double(long long* buf, long long n, int q, PhysX X, int thermal) {
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)q * n) return;
    const int a = (int)(e / n);
    const long long rest = thermal ? X.wt[a] : X.w[a];
    const double v = to_double(Qb(buf[e]) + Qb(rest));
    buf[e] = __double_as_longlong(v);
}

static inline unsigned xblocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// ------------------------------------------------------------------------------------
// Fused step (3D): the thermal collision of step s and the flow collision of step s+1 in one
// pass over the lattice.  The two-kernel step reads the 19 flow populations twice per step
// (the thermal kernel pulls f_post again for u) and the thermal ones twice; here each is read
// once and written once.
//
// Order of the reference's step (3DRB.F90:227-241): the flow collision of step s+1 at x needs
// T_s(x) = sum_a pull_a(g_post_s)(x), i.e. the thermal collisions of step s at x and its six
// neighbours, and the thermal collision of step s at y needs u_{s+1}(y) = macro of
// pull(f_post_s)(y).  Both macro steps of a cell use the same pulled f and the same lag
// T_{s-1}(y) = sum_a pull_a(g_post_{s-1})(y), so one macro step serves both.  A block owns
// full x-rows j0..j1-1 of a z range and marches in z: at plane p it runs the thermal
// collision of every cell of rows j0-1..j1 (one halo row each side, recomputed by both
// neighbouring tiles), and each cell adds its seven post-collision values, by the pull's
// boundary rules read backwards, to the T_s accumulators of the cells that pull them (three
// planes of the tile in shared memory).  Integer addition is exact and associative, so the
// order of those additions does not matter and T_s equals the pull sum bit for bit.  The
// plane p-1 is then complete and its flow collisions run.
//
// State between launches: f_post_s and g_post_{s-1} (the thermal populations one step
// behind); lbm_step enters with a flow-only launch and leaves with a thermal-only one, so the
// handle is in the two-kernel state between calls.  B_prev is double-buffered, because halo
// cells read a neighbour tile's B_prev while that tile writes its new one.
// ------------------------------------------------------------------------------------
constexpr int kXfRows = 8;  // rows per tile

struct XFusedArgs {
    const long long* fin;  // f_post_s
    const long long* gin;  // g_post_{s-1}
    long long* fout;       // f_post_{s+1}
    long long* gout;       // g_post_s
    const long long *bin0, *bin1, *bin2;
    long long *bout0, *bout1, *bout2;
    int ntj, nzc, zc;      // row tiles, z chunks, planes per chunk
};

template <int NT>
struct XfBlocks {
    static constexpr int value = NT <= 128 ? 4 : (NT <= 256 ? 2 : 1);
};

template <int NT>
__global__ void __launch_bounds__(NT, XfBlocks<NT>::value) k_xfused(Geo g, PhysX X, XFusedArgs F) {
    constexpr int TY = kXfRows, Q = 19, QT = 7;
    extern __shared__ __align__(16) unsigned long long xsm[];
    unsigned long long* tacc = xsm;                    // [3][TY][NT]: T_s accumulators (deviations)
    long long* tst = (long long*)(xsm + 3 * TY * NT);  // [2][TY][NT]: T_{s-1} of the tile cells
    const int i = (int)threadIdx.x;
    const bool act = i < g.nx;
    const long long n = g.ncell;
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const bool xper = g.bct[0] == LBM_BCT_PERIODIC, zper = g.bct[2] == LBM_BCT_PERIODIC;
    auto lf = [&](int a, long long cc) { return ldq(F.fin, a * n + cc); };
    auto lg = [&](int a, long long cc) { return ldq(F.gin, a * n + cc); };
    for (int item = blockIdx.x; item < F.ntj * F.nzc; item += gridDim.x) {
        const int j0 = (item % F.ntj) * TY, j1 = min(j0 + TY, ny);
        const int z0 = (item / F.ntj) * F.zc, z1 = min(z0 + F.zc, nz);
        auto add_to = [&](int tj, int tp, int ti, q60 v) {
            if (tj < j0 || tj >= j1 || tp < z0 || tp >= z1) return;
            atomicAdd(&tacc[((tp % 3) * TY + (tj - j0)) * NT + ti], v.u);
        };
        for (int r = 0; r < TY; ++r)
            for (int sl = 0; sl < 3; ++sl) tacc[(sl * TY + r) * NT + i] = 0ULL;
        __syncthreads();
        for (int p = z0 - 1; p <= z1; ++p) {
            // the accumulators of plane p+1 receive their first values in this pass
            if (p + 1 < z1 && p + 1 > z0)
                for (int r = 0; r < TY; ++r) tacc[(((p + 1) % 3) * TY + r) * NT + i] = 0ULL;
            __syncthreads();
            // ---- thermal collisions of plane p (step s), rows j0-1 .. j1 ----
            const bool pin = p >= 0 && p < nz;
            if (act && (pin || zper)) {
                const int pp = pin ? p : (p < 0 ? p + nz : p - nz);
                for (int jt = j0 - 1; jt <= j1; ++jt) {
                    if (jt < 0 || jt >= ny) continue;
                    const long long c = (long long)i + (long long)nx * ((long long)jt + (long long)ny * pp);
                    q60 d[Q], e[QT], ep[QT], rho, P[3], U[3], B[3];
                    q60 tdev = Qb(0);
                    if (aa_inner(g, i, jt, pp)) {
#pragma unroll
                        for (int a = 0; a < Q; ++a) d[a] = ldq(F.fin, a * n + c - lat_off<Q>(g, a));
#pragma unroll
                        for (int a = 0; a < QT; ++a) {
                            e[a] = ldq(F.gin, a * n + c - lat_off<QT>(g, a));
                            tdev = tdev + e[a];
                        }
                    } else {
#pragma unroll
                        for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, q60>(g, a, i, jt, pp, c, lf);
#pragma unroll
                        for (int a = 0; a < QT; ++a) {
                            e[a] = pull_thermal<QT, q60>(g, a, i, jt, pp, c, lg);
                            tdev = tdev + e[a];
                        }
                    }
                    macro<3>(d, tdev, X, rho, P, U);
                    B[0] = Qb(F.bin0[c]);
                    B[1] = Qb(F.bin1[c]);
                    B[2] = Qb(F.bin2[c]);
                    collideT_3d(e, U, tdev, B, X, ep);
                    if (jt >= j0 && jt < j1 && p >= z0 && p < z1) {  // a cell of this tile
#pragma unroll
                        for (int a = 0; a < QT; ++a) F.gout[a * n + c] = ep[a].s();
                        F.bout0[c] = B[0].s();
                        F.bout1[c] = B[1].s();
                        F.bout2[c] = B[2].s();
                        tst[((p & 1) * TY + (jt - j0)) * NT + i] = tdev.s();
                    }
                    // each value to the accumulator of the cell that pulls it
                    add_to(jt, p, i, ep[0]);
#pragma unroll
                    for (int b = 1; b < QT; ++b) {
                        const int ex = Lat<QT>::ex(b), ey = Lat<QT>::ey(b), ez = Lat<QT>::ez(b);
                        const int tx = i + ex, ty = jt + ey, tz = pp + ez;
                        int axis = -1;
                        bool low = false;
                        if (ex != 0 && (tx < 0 || tx >= nx)) {
                            if (xper) {
                                add_to(jt, p, tx < 0 ? nx - 1 : 0, ep[b]);
                                continue;
                            }
                            axis = 0;
                            low = tx < 0;
                        } else if (ey != 0 && (ty < 0 || ty >= ny)) {
                            axis = 1;
                            low = ty < 0;
                        } else if (ez != 0 && (tz < 0 || tz >= nz) && !zper) {
                            axis = 2;
                            low = tz < 0;
                        }
                        if (axis < 0) {
                            add_to(ty, p + ez, tx, ep[b]);
                        } else if (pick3(g.bct, axis) == LBM_BCT_CONST) {
                            add_to(jt, p, i, -ep[b] + Qb(low ? pick3(X.bc_lo, axis) : pick3(X.bc_hi, axis)));
                        } else {
                            add_to(jt, p, i, ep[b]);
                        }
                    }
                }
            }
            __syncthreads();
            // ---- flow collisions of plane q = p - 1 (step s+1) ----
            const int q = p - 1;
            if (act && q >= z0 && q < z1) {
                for (int j = j0; j < j1; ++j) {
                    const long long c = (long long)i + (long long)nx * ((long long)j + (long long)ny * q);
                    q60 d[Q], dp[Q], rho, P[3], U[3];
                    if (aa_inner(g, i, j, q)) {
#pragma unroll
                        for (int a = 0; a < Q; ++a) d[a] = ldq(F.fin, a * n + c - lat_off<Q>(g, a));
                    } else {
#pragma unroll
                        for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, q60>(g, a, i, j, q, c, lf);
                    }
                    macro<3>(d, Qb(tst[((q & 1) * TY + (j - j0)) * NT + i]), X, rho, P, U);
                    const q60 tnew = Qb((long long)tacc[((q % 3) * TY + (j - j0)) * NT + i]);
                    collide_3d(d, rho, P, U, tnew, X, dp);
#pragma unroll
                    for (int a = 0; a < Q; ++a) F.fout[a * n + c] = dp[a].s();
                }
            }
            __syncthreads();
        }
    }
}

// Block width for the fused step: the smallest supported width holding a full x-row.
static int xfused_width(const Geo& g) {
    const int w[] = {128, 256, 384, 512};
    for (int x : w)
        if (g.nx <= x) return x;
    return 0;
}

bool fixed_fused_supported(const Geo& g, int dim) { return dim == 3 && xfused_width(g) > 0 && g.ny >= 3 && g.nz >= 3; }

static size_t xfused_smem(int nt) { return (size_t)5 * kXfRows * nt * sizeof(long long); }

template <int NT>
static void launch_xfused(const Geo& g, const PhysX& X, XFusedArgs F, cudaStream_t s) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_xfused<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)xfused_smem(NT));
        if (sms <= 0) sms = 1;
    }
    const int slots = XfBlocks<NT>::value * sms;
    // z chunks: enough items for about two waves of resident blocks, at least 16 planes each
    F.ntj = (g.ny + kXfRows - 1) / kXfRows;
    int nzc = (2 * slots + F.ntj - 1) / F.ntj;
    if (nzc > g.nz / 16) nzc = g.nz / 16;
    if (nzc < 1) nzc = 1;
    F.zc = (g.nz + nzc - 1) / nzc;
    F.nzc = (g.nz + F.zc - 1) / F.zc;
    const int items = F.ntj * F.nzc;
    const int grid = items < slots ? items : slots;
    k_xfused<NT><<<grid, NT, xfused_smem(NT), s>>>(g, X, F);
}

void fixed_fused_pass(const Geo& g, const PhysX& X, const long long* fin, const long long* gin, long long* fout,
                      long long* gout, const long long* const bin[3], long long* const bout[3], cudaStream_t s) {
    XFusedArgs F{};
    F.fin = fin;
    F.gin = gin;
    F.fout = fout;
    F.gout = gout;
    F.bin0 = bin[0];
    F.bin1 = bin[1];
    F.bin2 = bin[2];
    F.bout0 = bout[0];
    F.bout1 = bout[1];
    F.bout2 = bout[2];
    switch (xfused_width(g)) {
        case 128: launch_xfused<128>(g, X, F, s); break;
        case 256: launch_xfused<256>(g, X, F, s); break;
        case 384: launch_xfused<384>(g, X, F, s); break;
        default: launch_xfused<512>(g, X, F, s); break;
    }
}



// Steady-state step of one dimension: interior kernel and face kernel for each half.
template <int D>
static void steady_step(const Geo& g, const PhysX& X, const FixedArrays& A, const long long* fprev,
                        const long long* gprev, long long* fnext, long long* gnext, cudaStream_t s, bool fl, bool th,
                        bool wide) {
    const unsigned bx = (unsigned)((g.nx + 127) / 128);
    const dim3 bin(128), gin_grid(bx, (unsigned)(g.ny - 2), D == 3 ? (unsigned)(g.nz - 2) : 1u);
    const dim3 gface(bx, (unsigned)face_row_count(g), 1u);
    // a 3D lattice of two planes has no interior rows: the face rows hold every cell
    const bool interior = D == 2 || g.nz > 2;
    constexpr int Q = D == 3 ? 19 : 9;
    const bool idx32 = !wide && (long long)Q * g.ncell < (1LL << 31);
    if (fl) {
        if (interior && idx32) k_xflow_in<D, int><<<gin_grid, bin, 0, s>>>(g, X, A, fprev, gprev, fnext);
        else if (interior) k_xflow_in<D, long long><<<gin_grid, bin, 0, s>>>(g, X, A, fprev, gprev, fnext);
        k_xflow_face<D><<<gface, bin, 0, s>>>(g, X, A, fprev, gprev, fnext);
    }
    if (th) {
        if (interior && idx32) k_xthermal_in<D, int><<<gin_grid, bin, 0, s>>>(g, X, A, fnext, gprev, gnext);
        else if (interior) k_xthermal_in<D, long long><<<gin_grid, bin, 0, s>>>(g, X, A, fnext, gprev, gnext);
        k_xthermal_face<D><<<gface, bin, 0, s>>>(g, X, A, fnext, gprev, gnext);
    }
}

void fixed_fused_step(const Geo& g, const PhysX& X, const FixedArrays& A, int dim, bool first, const long long* fprev,
                      const long long* gprev, long long* fnext, long long* gnext, cudaStream_t s, int part, bool wide) {
    const int bs = 128;
    const unsigned nb = xblocks(g.ncell, bs);
    const bool fl = part != 1, th = part != 0;
    if (dim == 2) {
        if (first) {
            if (fl) k_xflow<2, true><<<nb, bs, 0, s>>>(g, X, A, fprev, gprev, fnext);
            if (th) k_xthermal<2, true><<<nb, bs, 0, s>>>(g, X, A, fnext, gprev, gnext);
        } else {
            steady_step<2>(g, X, A, fprev, gprev, fnext, gnext, s, fl, th, wide);
        }
    } else {
        if (first) {
            if (fl) k_xflow<3, true><<<nb, bs, 0, s>>>(g, X, A, fprev, gprev, fnext);
            if (th) k_xthermal<3, true><<<nb, bs, 0, s>>>(g, X, A, fnext, gprev, gnext);
        } else {
            steady_step<3>(g, X, A, fprev, gprev, fnext, gnext, s, fl, th, wide);
        }
    }
}

void fixed_materialize(const Geo& g, const PhysX& X, const FixedArrays& A, int dim, const long long* fcur,
                       const long long* gcur, cudaStream_t s) {
    const unsigned nb = xblocks(g.ncell, 128);
    if (dim == 2) k_xmaterialize<2><<<nb, 128, 0, s>>>(g, X, A, fcur, gcur);
    else k_xmaterialize<3><<<nb, 128, 0, s>>>(g, X, A, fcur, gcur);
}

void fixed_post_to_double(const PhysX& X, long long* fbuf, long long* gbuf, long long n, int q, int qt,
                          cudaStream_t s) {
    k_xpost_to_double<<<xblocks((long long)q * n, 256), 256, 0, s>>>(fbuf, n, q, X, 0);
    k_xpost_to_double<<<xblocks((long long)qt * n, 256), 256, 0, s>>>(gbuf, n, qt, X, 1);
}

}  // namespace lbm
