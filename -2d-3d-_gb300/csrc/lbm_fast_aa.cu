// lbm_fast_aa.cu - the in-place (AA) access pattern of the FP32/FP16 storage forms, and
// the pattern's helpers shared with the FP64 plain method (face snapshots, module view).
//
// One population array per lattice (fbuf[0], gbuf[0]) whose layout alternates between the
// streamed and the swapped form (lbm_device.cuh).  A step is the two-kernel step of
// lbm_fast.cu with the same per-cell arithmetic in the same order; only the slots a cell
// reads and writes change, so every state equals the two-buffer state bit for bit.  The
// population memory is half the two-buffer form's: the arrays are also the module arrays.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lbm_fast.h"
#include "lbm_fast_cells.cuh"
#include "lbm_fast_pairs.cuh"
#include "lbm_fast_aa.cuh"

namespace lbm {

// conversions of the generic helpers (S = double for the FP64 plain method)
template <class S> __device__ __forceinline__ double to_d(S x) { return (double)x; }
template <> __device__ __forceinline__ double to_d<__half>(__half x) { return (double)__half2float(x); }

// ------------------------------------------------------------------------------------
// face snapshots: slot (opp(a), source) of every cell on the far face of a periodic axis,
// stored at [a][face index of the destination cell] (the pull wraps along that axis only,
// so source and destination share their other indices)
// ------------------------------------------------------------------------------------
template <int Q, class S>
__global__ void k_aa_face(Geo g, const S* __restrict__ arr, S* __restrict__ face, int axis) {
    const long long nf = aa_face_cells(g, axis);
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)Q * nf) return;
    const int a = (int)(e / nf);
    const long long f = e - (long long)a * nf;
    const int ea = axis == 0 ? Lat<Q>::ex(a) : (axis == 1 ? Lat<Q>::ey(a) : Lat<Q>::ez(a));
    if (ea == 0) return;
    int i, j, k;
    if (axis == 0) {
        j = (int)(f % g.ny); k = (int)(f / g.ny); i = ea > 0 ? g.nx - 1 : 0;
    } else if (axis == 1) {
        i = (int)(f % g.nx); k = (int)(f / g.nx); j = ea > 0 ? g.ny - 1 : 0;
    } else {
        i = (int)(f % g.nx); j = (int)(f / g.nx); k = ea > 0 ? g.nz - 1 : 0;
    }
    face[e] = arr[(long long)Lat<Q>::opp(a) * g.ncell + cell_index(g, i, j, k)];
}

template <int Q, class S>
static void face_launch(const Geo& g, const void* arr, void* const face[3], cudaStream_t s) {
    for (int ax = 0; ax < 3; ++ax) {
        if (!face[ax]) continue;
        const long long cnt = (long long)Q * aa_face_cells(g, ax);
        k_aa_face<Q, S><<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>(g, (const S*)arr, (S*)face[ax], ax);
    }
}

template <class S>
static void face_dispatch(const Geo& g, int q, const void* arr, void* const face[3], cudaStream_t s) {
    switch (q) {
        case 19: face_launch<19, S>(g, arr, face, s); break;
        case 9: face_launch<9, S>(g, arr, face, s); break;
        case 7: face_launch<7, S>(g, arr, face, s); break;
        default: face_launch<5, S>(g, arr, face, s); break;
    }
}

void aa_snapshot(const Geo& g, int q, bool, int precision, const void* arr, void* const face[3], cudaStream_t s) {
    if (precision == LBM_FP64) face_dispatch<double>(g, q, arr, face, s);
    else if (precision == LBM_FP32) face_dispatch<float>(g, q, arr, face, s);
    else face_dispatch<__half>(g, q, arr, face, s);
}

// ------------------------------------------------------------------------------------
// module view: the streamed population of (cell, a) read through the array's layout
// ------------------------------------------------------------------------------------
template <int Q, bool THERMAL, class S, class T>
__global__ void k_aa_view(Geo g, const S* __restrict__ arr, int par, int raw, double* __restrict__ out, int soa,
                          int dev, double w0, double w1) {
    const long long n = g.ncell;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)Q * n) return;
    const long long c = e / Q;
    const int a = (int)(e - c * Q);
    int i, j, k;
    cell_coords(g, c, i, j, k);
    auto ld = [&](int b, long long cc) { return (T)to_d<S>(arr[(long long)(par ? Lat<Q>::opp(b) : b) * n + cc]); };
    T v;
    if (THERMAL) v = par ? pull_thermal<Q, T>(g, a, i, j, k, c, ld) : aa_local_thermal<Q, T>(g, a, i, j, k, c, raw != 0, ld);
    else v = par ? pull_flow<Q, T>(g, a, i, j, k, c, ld) : ld(a, c);
    double r = (double)v;
    if (dev) {
        const double rest = THERMAL ? (a == 0 ? w0 : w1) : wrest<(Q == 9 || Q == 5) ? 9 : 19>(a);
        r = rest + (double)roundS<S>((float)v);
    }
    out[soa ? (long long)a * n + c : e] = r;
}

template <class S, class T>
static void view_launch(const Geo& g, int q, bool thermal, const void* arr, int par, bool raw, double* out, bool soa,
                        bool dev, double w0, double w1, cudaStream_t s) {
    const unsigned nb = (unsigned)(((long long)q * g.ncell + 255) / 256);
    const S* p = (const S*)arr;
    const int r = raw ? 1 : 0, so = soa ? 1 : 0, dv = dev ? 1 : 0;
    if (thermal) {
        if (q == 7) k_aa_view<7, true, S, T><<<nb, 256, 0, s>>>(g, p, par, r, out, so, dv, w0, w1);
        else k_aa_view<5, true, S, T><<<nb, 256, 0, s>>>(g, p, par, r, out, so, dv, w0, w1);
    } else {
        if (q == 19) k_aa_view<19, false, S, T><<<nb, 256, 0, s>>>(g, p, par, r, out, so, dv, w0, w1);
        else k_aa_view<9, false, S, T><<<nb, 256, 0, s>>>(g, p, par, r, out, so, dv, w0, w1);
    }
}

void aa_module_view(const Geo& g, int q, bool thermal, int precision, const void* arr, int par, bool raw, double* out,
                    bool soa, bool dev, double w0, double w1, cudaStream_t s) {
    if (precision == LBM_FP64) view_launch<double, double>(g, q, thermal, arr, par, raw, out, soa, false, w0, w1, s);
    else if (precision == LBM_FP32) view_launch<float, float>(g, q, thermal, arr, par, raw, out, soa, dev, w0, w1, s);
    else view_launch<__half, float>(g, q, thermal, arr, par, raw, out, soa, dev, w0, w1, s);
}

// ------------------------------------------------------------------------------------
// FP32/FP16 step kernels, one cell per thread (the arithmetic of flow_cell_2k and
// thermal_cell_2k).  ODD: the kernel's own array is in the swapped layout.  FIRST is a
// template parameter as in the two-buffer kernels: with FMA contraction allowed, a value
// merged from two paths at run time could be rounded differently downstream.
// ------------------------------------------------------------------------------------
template <int D, class S, bool ODD, bool FIRST>
__global__ void __launch_bounds__(128, (OneCellBlocks<S, false>::value)) k_aa_flow_f(Geo g, PhysF P, FastArgs<S> A, S* f, const S* __restrict__ gs,
                                                   AAFace<S> wf, int gpar, int graw) {
    long long c;
    int i, j, k;
    // the FP16 odd sweep runs fastest with the x-face cells in warps of their own (its
    // boundary path, pulls and pushes, is the longest); every other one-cell kernel is
    // faster with cells in lattice order (row-aligned warps)
    if (ODD && sizeof(S) == 2 ? !split_cell(g, c, i, j, k) : !fcell(g, c, i, j, k)) return;
    aa_flow_cell<D, S, ODD, FIRST>(g, P, A, f, gs, wf, gpar, graw, c, i, j, k);
}

template <int D, class S, bool ODD, bool FIRST>
__global__ void __launch_bounds__(128, (OneCellBlocks<S, true>::value)) k_aa_thermal_f(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fs, S* gg,
                                                      AAFace<S> wg, int fpar, int graw) {
    long long c;
    int i, j, k;
    if (!fcell(g, c, i, j, k)) return;
    aa_thermal_cell<D, S, ODD, FIRST>(g, P, A, fs, gg, wg, fpar, graw, c, i, j, k);
}

// Module scalars (rho, u, v, w, T) of the current step, populations left in place.
template <int D, class S>
__global__ void k_aa_materialize_f(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fs,
                                   const S* __restrict__ gs, int fpar, int gpar, int graw) {
    long long c;
    int i, j, k;
    if (!fcell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    float d[Q];
    if (fpar) {
        auto lf = [&](int b, long long cc) { return ldS(fs, Lat<Q>::opp(b) * n + cc); };
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, float>(g, a, i, j, k, c, lf);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldS(fs, a * n + c);
    }
    float ts = 0.0f;
    if (gpar) {
        auto lg = [&](int b, long long cc) { return ldS(gs, Lat<QT>::opp(b) * n + cc); };
#pragma unroll
        for (int a = 0; a < QT; ++a) ts += pull_thermal<QT, float>(g, a, i, j, k, c, lg) + wT<QT>(P, a) * P.Tref;
    } else {
        auto lg = [&](int b, long long cc) { return ldS(gs, b * n + cc); };
#pragma unroll
        for (int a = 0; a < QT; ++a)
            ts += aa_local_thermal<QT, float>(g, a, i, j, k, c, graw != 0, lg) + wT<QT>(P, a) * P.Tref;
    }
    float dr, rho, u, v, w, Fy;
    fmacro<D>(d, A.lag_in[c], P, dr, rho, u, v, w, Fy);
    A.rho[c] = rho;
    A.u[c] = u;
    A.v[c] = v;
    if (D == 3) A.w[c] = w;
    A.T[c] = ts;
}

// ------------------------------------------------------------------------------------
// Paired form: cells (i0, j, k) and (i0+1, j, k) per thread (nx even), populations moved as
// 2-element vectors as in lbm_fast_pairs.cuh; the per-cell arithmetic is flow_pair_2k's and
// thermal_pair_2k's statement for statement.  Pushes whose target shifts along x, or
// leaves the lattice, are scalar stores through aa_push.
// ------------------------------------------------------------------------------------
// 2-element loads: CO = coherent (an array this kernel writes), otherwise the read-only path
template <class S, bool CO> __device__ __forceinline__ float2 ld2(const S* p, long long i);
template <> __device__ __forceinline__ float2 ld2<float, false>(const float* p, long long i) {
    return __ldg(reinterpret_cast<const float2*>(p + i));
}
template <> __device__ __forceinline__ float2 ld2<float, true>(const float* p, long long i) {
    return __ldg(reinterpret_cast<const float2*>(p + i));  // see ldA
}
__device__ __forceinline__ float2 h2f2(unsigned int w) {
    return __half22float2(__halves2half2(__ushort_as_half((unsigned short)(w & 0xFFFFu)),
                                         __ushort_as_half((unsigned short)(w >> 16))));
}
template <> __device__ __forceinline__ float2 ld2<__half, false>(const __half* p, long long i) {
    return h2f2(__ldg(reinterpret_cast<const unsigned int*>(p + i)));
}
template <> __device__ __forceinline__ float2 ld2<__half, true>(const __half* p, long long i) {
    return h2f2(__ldg(reinterpret_cast<const unsigned int*>(p + i)));  // see ldA
}

// Values at x = i0 - ex and i0 + 1 - ex of one row (both inside the lattice in x).
template <class S, bool CO>
__device__ __forceinline__ float2 row2(const Geo& g, const S* p, int ex, int i0, long long row) {
    if (ex == 0) return ld2<S, CO>(p, row + i0);
    if (ex == 1) {
        const float2 lo = ld2<S, CO>(p, row + (i0 > 0 ? i0 - 2 : 0));
        const float2 hi = ld2<S, CO>(p, row + i0);
        return make_float2(lo.y, hi.x);
    }
    const float2 lo = ld2<S, CO>(p, row + i0);
    const float2 hi = ld2<S, CO>(p, row + (i0 + 2 < g.nx ? i0 + 2 : i0));
    return make_float2(lo.y, hi.x);
}

// Pull of direction a into the pair from the swapped layout (dir d of cell s in plane
// opp(d)); sources outside the lattice take the scalar pull with its boundary rule.
template <int Q, bool TH, class S, bool CO, class LOAD, class W0, class W1>
__device__ __forceinline__ float2 swp_pull2(const Geo& g, const S* p, int a, int i0, int j, int k, long long c0,
                                           long long n, LOAD load, W0 w0, W1 w1) {
    const int ex = Lat<Q>::ex(a), ey = Lat<Q>::ey(a), ez = Lat<Q>::ez(a);
    const int sj = j - ey, sk = k - ez;
    const bool yz = (ey == 0 || (sj >= 0 && sj < g.ny)) && (ez == 0 || (sk >= 0 && sk < g.nz));
    float2 v = make_float2(0.0f, 0.0f);
    if (yz)
        v = row2<S, CO>(g, p, ex, i0, (long long)Lat<Q>::opp(a) * n + (long long)g.nx * ((long long)sj + (long long)g.ny * sk));
    if (!yz || (ex == 1 && i0 == 0))
        v.x = TH ? pull_thermal_w<Q, float>(g, a, i0, j, k, c0, load, w0) : pull_flow_w<Q, float>(g, a, i0, j, k, c0, load, w0);
    if (!yz || (ex == -1 && i0 + 2 >= g.nx))
        v.y = TH ? pull_thermal_w<Q, float>(g, a, i0 + 1, j, k, c0 + 1, load, w1)
                 : pull_flow_w<Q, float>(g, a, i0 + 1, j, k, c0 + 1, load, w1);
    return v;
}

// Thermal pair from the streamed layout, wall rule applied to pushed slots.
template <int QT, class S, bool CO>
__device__ __forceinline__ float2 loc_thermal2(const Geo& g, const S* p, int a, int i0, int j, int k, long long c0,
                                              long long n, bool raw) {
    float2 v = ld2<S, CO>(p, (long long)a * n + c0);
    if (raw && a != 0) {
        const float x = v.x, y = v.y;
        v.x = aa_local_thermal<QT, float>(g, a, i0, j, k, c0, true, [&](int, long long) { return x; });
        v.y = aa_local_thermal<QT, float>(g, a, i0 + 1, j, k, c0 + 1, true, [&](int, long long) { return y; });
    }
    return v;
}

// Push of the pair's post-collision values of direction a (odd sweep), already rounded to
// the storage type.
template <int Q, bool TH, class S>
__device__ __forceinline__ void push2(const Geo& g, S* p, int a, int i0, int j, int k, long long c0, long long n, S v0,
                                      S v1) {
    const int ex = Lat<Q>::ex(a), ey = Lat<Q>::ey(a), ez = Lat<Q>::ez(a);
    const int tj = j + ey, tk = k + ez;
    const bool yz = (ey == 0 || (tj >= 0 && tj < g.ny)) && (ez == 0 || (tk >= 0 && tk < g.nz));
    if (ex == 0 && yz) {
        Vec2<S>::st_raw(p, (long long)a * n + c0 + (long long)g.nx * ((long long)ey + (long long)g.ny * ez), v0, v1);
        return;
    }
    if (yz && i0 + ex >= 0 && i0 + 1 + ex < g.nx) {  // both targets inside: plain stores
        p[(long long)a * n + c0 + lat_off<Q>(g, a)] = v0;
        p[(long long)a * n + c0 + 1 + lat_off<Q>(g, a)] = v1;
        return;
    }
    auto st = [&](int b, long long cc, S v) { p[(long long)b * n + cc] = v; };
    aa_push<Q, TH, S>(g, a, i0, j, k, c0, v0, st);
    aa_push<Q, TH, S>(g, a, i0 + 1, j, k, c0 + 1, v1, st);
}

__device__ __forceinline__ bool aa_pair_cell(const Geo& g, long long& c0, int& i0, int& j, int& k) {
    i0 = 2 * (int)(blockIdx.x * blockDim.x + threadIdx.x);
    j = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    k = (int)blockIdx.z;
    if (i0 >= g.nx || j >= g.ny) return false;
    c0 = (long long)i0 + (long long)g.nx * ((long long)j + (long long)g.ny * (long long)k);
    return true;
}

template <int D, class S, bool ODD>
__global__ void __launch_bounds__(128) k_aa_flow_p(Geo g, PhysF P, FastArgs<S> A, S* f, const S* __restrict__ gs,
                                                   AAFace<S> wf, int gpar, int graw) {
    long long c0;
    int i0, j, k;
    if (!aa_pair_cell(g, c0, i0, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    float d0[Q], d1[Q];
    if (ODD) {
        auto lf = [&](int b, long long cc) { return ldA(f, Lat<Q>::opp(b) * n + cc); };
        auto w0 = [&](int ax, int b, long long) {
            return ldA(aa_face_ptr(wf, ax), b * aa_face_cells(g, ax) + aa_face_index(g, ax, i0, j, k));
        };
        auto w1 = [&](int ax, int b, long long) {
            return ldA(aa_face_ptr(wf, ax), b * aa_face_cells(g, ax) + aa_face_index(g, ax, i0 + 1, j, k));
        };
#pragma unroll
        for (int a = 0; a < Q; ++a) {
            const float2 v = swp_pull2<Q, false, S, true>(g, f, a, i0, j, k, c0, n, lf, w0, w1);
            d0[a] = v.x;
            d1[a] = v.y;
        }
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) {
            const float2 v = ld2<S, true>(f, a * n + c0);
            d0[a] = v.x;
            d1[a] = v.y;
        }
    }
    float ts0 = 0.0f, ts1 = 0.0f;
    if (gpar) {
        auto lg = [&](int b, long long cc) { return ldS(gs, Lat<QT>::opp(b) * n + cc); };
        auto wd = [&](int, int b, long long cc) { return lg(b, cc); };
#pragma unroll
        for (int a = 0; a < QT; ++a) {
            const float2 e = swp_pull2<QT, true, S, false>(g, gs, a, i0, j, k, c0, n, lg, wd, wd);
            ts0 += e.x;
            ts1 += e.y;
        }
    } else {
#pragma unroll
        for (int a = 0; a < QT; ++a) {
            const float2 e = loc_thermal2<QT, S, false>(g, gs, a, i0, j, k, c0, n, graw != 0);
            ts0 += e.x;
            ts1 += e.y;
        }
    }
    const float2 lag = ld2<float, true>(A.lag_in, c0);
    float dp0[Q], dp1[Q], Fy0, Fy1;
    {
        const float T = ts0 + P.Tref;
        float dr, rho, u, v, w = 0.0f, Fm;
        fmacro<D>(d0, lag.x, P, dr, rho, u, v, w, Fm);
        Fy0 = rho * P.gBeta * (T - P.Tref);
        if (D == 2) fcollide_2d(d0, dr, rho, u, v, Fy0, P, dp0);
        else fcollide_3d(d0, dr, rho, u, v, w, Fy0, P, dp0);
    }
    {
        const float T = ts1 + P.Tref;
        float dr, rho, u, v, w = 0.0f, Fm;
        fmacro<D>(d1, lag.y, P, dr, rho, u, v, w, Fm);
        Fy1 = rho * P.gBeta * (T - P.Tref);
        if (D == 2) fcollide_2d(d1, dr, rho, u, v, Fy1, P, dp1);
        else fcollide_3d(d1, dr, rho, u, v, w, Fy1, P, dp1);
    }
    if (D == 2) stf2(A.lag_out, c0, Fy0, Fy1);
    S h0[Q], h1[Q];
    round_pair<Q>(dp0, dp1, h0, h1, P.sr != 0, sr_seed(*A.tick, c0, 0), sr_seed(*A.tick, c0 + 1, 0));
    if (ODD) {
#pragma unroll
        for (int a = 0; a < Q; ++a) push2<Q, false, S>(g, f, a, i0, j, k, c0, n, h0[a], h1[a]);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) Vec2<S>::st_raw(f, Lat<Q>::opp(a) * n + c0, h0[a], h1[a]);
    }
}

template <int D, class S, bool ODD>
__global__ void __launch_bounds__(128) k_aa_thermal_p(Geo g, PhysF P, FastArgs<S> A, const S* __restrict__ fs, S* gg,
                                                      AAFace<S> wg, int fpar, int graw) {
    long long c0;
    int i0, j, k;
    if (!aa_pair_cell(g, c0, i0, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    float d0[Q], d1[Q], G0[QT], G1[QT];
    if (fpar) {
        auto lf = [&](int b, long long cc) { return ldS(fs, Lat<Q>::opp(b) * n + cc); };
        auto wd = [&](int, int b, long long cc) { return lf(b, cc); };
#pragma unroll
        for (int a = 0; a < Q; ++a) {
            const float2 v = swp_pull2<Q, false, S, false>(g, fs, a, i0, j, k, c0, n, lf, wd, wd);
            d0[a] = v.x;
            d1[a] = v.y;
        }
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) {
            const float2 v = ld2<S, false>(fs, a * n + c0);
            d0[a] = v.x;
            d1[a] = v.y;
        }
    }
    float ts0 = 0.0f, ts1 = 0.0f;
    if (ODD) {
        auto lg = [&](int b, long long cc) { return ldA(gg, Lat<QT>::opp(b) * n + cc); };
        auto w0 = [&](int ax, int b, long long) {
            return ldA(aa_face_ptr(wg, ax), b * aa_face_cells(g, ax) + aa_face_index(g, ax, i0, j, k));
        };
        auto w1 = [&](int ax, int b, long long) {
            return ldA(aa_face_ptr(wg, ax), b * aa_face_cells(g, ax) + aa_face_index(g, ax, i0 + 1, j, k));
        };
#pragma unroll
        for (int a = 0; a < QT; ++a) {
            const float2 e = swp_pull2<QT, true, S, true>(g, gg, a, i0, j, k, c0, n, lg, w0, w1);
            G0[a] = e.x + wT<QT>(P, a) * P.Tref;
            G1[a] = e.y + wT<QT>(P, a) * P.Tref;
            ts0 += G0[a];
            ts1 += G1[a];
        }
    } else {
#pragma unroll
        for (int a = 0; a < QT; ++a) {
            const float2 e = loc_thermal2<QT, S, true>(g, gg, a, i0, j, k, c0, n, graw != 0);
            G0[a] = e.x + wT<QT>(P, a) * P.Tref;
            G1[a] = e.y + wT<QT>(P, a) * P.Tref;
            ts0 += G0[a];
            ts1 += G1[a];
        }
    }
    const float2 bx = ld2<float, true>(A.Bin0, c0), by = ld2<float, true>(A.Bin1, c0);
    const float2 bz = D == 3 ? ld2<float, true>(A.Bin2, c0) : make_float2(0.0f, 0.0f);
    const float2 lag = D == 2 ? ld2<float, true>(A.lag_in, c0) : make_float2(0.0f, 0.0f);
    float GP0[QT], GP1[QT];
    float Bx0 = bx.x, By0 = by.x, Bz0 = bz.x, Bx1 = bx.y, By1 = by.y, Bz1 = bz.y;
    {
        float dr, rho, u, v, w, Fy;
        fmacro<D>(d0, D == 2 ? lag.x : ts0, P, dr, rho, u, v, w, Fy);
        if (D == 2) fcollideT_2d(G0, u, v, ts0, Bx0, By0, P, GP0);
        else fcollideT_3d(G0, u, v, w, ts0, Bx0, By0, Bz0, P, GP0);
    }
    {
        float dr, rho, u, v, w, Fy;
        fmacro<D>(d1, D == 2 ? lag.y : ts1, P, dr, rho, u, v, w, Fy);
        if (D == 2) fcollideT_2d(G1, u, v, ts1, Bx1, By1, P, GP1);
        else fcollideT_3d(G1, u, v, w, ts1, Bx1, By1, Bz1, P, GP1);
    }
    stf2(A.Bout0, c0, Bx0, Bx1);
    stf2(A.Bout1, c0, By0, By1);
    if (D == 3) {
        stf2(A.Bout2, c0, Bz0, Bz1);
        stf2(A.lag_out, c0, ts0, ts1);
    }
    float e0[QT], e1[QT];
    S h0[QT], h1[QT];
#pragma unroll
    for (int a = 0; a < QT; ++a) {
        e0[a] = GP0[a] - wT<QT>(P, a) * P.Tref;
        e1[a] = GP1[a] - wT<QT>(P, a) * P.Tref;
    }
    round_pair<QT>(e0, e1, h0, h1, P.sr != 0, sr_seed(*A.tick, c0, 1), sr_seed(*A.tick, c0 + 1, 1));
    if (ODD) {
#pragma unroll
        for (int a = 0; a < QT; ++a) push2<QT, true, S>(g, gg, a, i0, j, k, c0, n, h0[a], h1[a]);
    } else {
#pragma unroll
        for (int a = 0; a < QT; ++a) Vec2<S>::st_raw(gg, Lat<QT>::opp(a) * n + c0, h0[a], h1[a]);
    }
}

// ------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------
template <class S>
static FastArgs<S> aa_args(const FastState& F) {
    FastArgs<S> a;
    a.fref = (S*)F.fref;
    a.gref = (S*)F.gref;
    a.rho = F.rho; a.u = F.u; a.v = F.v; a.w = F.w; a.T = F.T;
    a.Bin0 = F.B[0][0]; a.Bin1 = F.B[0][1]; a.Bin2 = F.B[0][2];
    a.Bout0 = F.B[0][0]; a.Bout1 = F.B[0][1]; a.Bout2 = F.B[0][2];
    a.lag_in = F.L[0];
    a.lag_out = F.L[0];
    a.tick = F.tick;
    return a;
}

template <class S>
static AAFace<S> aa_faces(void* const face[3]) {
    return AAFace<S>{(const S*)face[0], (const S*)face[1], (const S*)face[2]};
}

static bool any_face(void* const face[3]) { return face[0] || face[1] || face[2]; }

bool fast_aa_tma_sweep(FastState& F, const Geo& g, const PhysF& pf, int dim, const void* A, int part, cudaStream_t s);

template <int D, class S, bool FIRST>
static void aa_step_launch(FastState& F, const Geo& g, const PhysF& pf, cudaStream_t s, int part) {
    AAState& st = F.AA;
    const FastArgs<S> A = aa_args<S>(F);
    S* f = (S*)F.fbuf[0];
    S* gg = (S*)F.gbuf[0];
    const unsigned nb = (unsigned)((g.ncell + 127) / 128);
    const int raw = st.graw ? 1 : 0;
    // Forms measured on GB300 (3D, 128^3 to 384^3): the even flow sweep, whose loads and
    // stores are all the cell's own slots, is fastest with two cells per thread; every other
    // sweep with one cell per thread (LBM_OPT_PAIRS / LBM_OPT_STAGED select the paired or
    // staged form for them).  The first step (module arrays) and odd nx take one cell per
    // thread.
    const bool paired = !FIRST && F.pairs && g.nx % 2 == 0;
    const bool paired_even_flow = !FIRST && g.nx % 2 == 0 && st.fpar == 0;
    const int pairs = g.nx / 2, bx = pairs > 32 ? 64 : 32, by = 128 / bx;
    const dim3 pgrid((pairs + bx - 1) / bx, (g.ny + by - 1) / by, g.nz), pblock(bx, by, 1);
    if (part != 1) {
        if (st.fpar && any_face(st.face_f)) aa_snapshot(g, F.q, false, F.precision, f, st.face_f, s);
        const AAFace<S> wf = aa_faces<S>(st.face_f);
        // the even flow sweep touches only the cell's own slots: staging buys nothing there
        if (!FIRST && F.tma && st.fpar && fast_aa_tma_sweep(F, g, pf, D, &A, 0, s)) {
            // staged rows (lbm_fast_tma.cu)
        } else if (paired || paired_even_flow) {
            if (st.fpar) k_aa_flow_p<D, S, true><<<pgrid, pblock, 0, s>>>(g, pf, A, f, gg, wf, st.gpar, raw);
            else k_aa_flow_p<D, S, false><<<pgrid, pblock, 0, s>>>(g, pf, A, f, gg, wf, st.gpar, raw);
        } else if (st.fpar) {
            k_aa_flow_f<D, S, true, FIRST><<<nb, 128, 0, s>>>(g, pf, A, f, gg, wf, st.gpar, raw);
        } else {
            k_aa_flow_f<D, S, false, FIRST><<<nb, 128, 0, s>>>(g, pf, A, f, gg, wf, st.gpar, raw);
        }
        st.fpar ^= 1;
    }
    if (part != 0) {
        if (st.gpar && any_face(st.face_g)) aa_snapshot(g, F.qt, true, F.precision, gg, st.face_g, s);
        const AAFace<S> wg = aa_faces<S>(st.face_g);
        if (!FIRST && F.tma && fast_aa_tma_sweep(F, g, pf, D, &A, 1, s)) {
            // staged rows (lbm_fast_tma.cu)
        } else if (paired) {
            if (st.gpar) k_aa_thermal_p<D, S, true><<<pgrid, pblock, 0, s>>>(g, pf, A, f, gg, wg, st.fpar, raw);
            else k_aa_thermal_p<D, S, false><<<pgrid, pblock, 0, s>>>(g, pf, A, f, gg, wg, st.fpar, raw);
        } else if (st.gpar) {
            k_aa_thermal_f<D, S, true, FIRST><<<nb, 128, 0, s>>>(g, pf, A, f, gg, wg, st.fpar, raw);
        } else {
            k_aa_thermal_f<D, S, false, FIRST><<<nb, 128, 0, s>>>(g, pf, A, f, gg, wg, st.fpar, raw);
        }
        if (st.gpar) st.graw = true;
        st.gpar ^= 1;
    }
}

template <int D, class S>
static void aa_step_first(FastState& F, const Geo& g, const PhysF& pf, bool first, cudaStream_t s, int part) {
    if (first) aa_step_launch<D, S, true>(F, g, pf, s, part);
    else aa_step_launch<D, S, false>(F, g, pf, s, part);
}

void fast_step_aa(FastState& F, const Geo& g, const PhysF& pf, int dim, bool first, cudaStream_t s, int part) {
    if (F.precision == LBM_FP16) {
        if (dim == 2) aa_step_first<2, __half>(F, g, pf, first, s, part);
        else aa_step_first<3, __half>(F, g, pf, first, s, part);
    } else {
        if (dim == 2) aa_step_first<2, float>(F, g, pf, first, s, part);
        else aa_step_first<3, float>(F, g, pf, first, s, part);
    }
}

void fast_materialize_aa(FastState& F, const Geo& g, const PhysF& pf, int dim, cudaStream_t s) {
    const unsigned nb = (unsigned)((g.ncell + 127) / 128);
    const AAState& st = F.AA;
    const int raw = st.graw ? 1 : 0;
    if (F.precision == LBM_FP16) {
        const FastArgs<__half> A = aa_args<__half>(F);
        const __half *f = (const __half*)F.fbuf[0], *gg = (const __half*)F.gbuf[0];
        if (dim == 2) k_aa_materialize_f<2, __half><<<nb, 128, 0, s>>>(g, pf, A, f, gg, st.fpar, st.gpar, raw);
        else k_aa_materialize_f<3, __half><<<nb, 128, 0, s>>>(g, pf, A, f, gg, st.fpar, st.gpar, raw);
    } else {
        const FastArgs<float> A = aa_args<float>(F);
        const float *f = (const float*)F.fbuf[0], *gg = (const float*)F.gbuf[0];
        if (dim == 2) k_aa_materialize_f<2, float><<<nb, 128, 0, s>>>(g, pf, A, f, gg, st.fpar, st.gpar, raw);
        else k_aa_materialize_f<3, float><<<nb, 128, 0, s>>>(g, pf, A, f, gg, st.fpar, st.gpar, raw);
    }
}

}  // namespace lbm
