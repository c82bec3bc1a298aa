// lbm_fast_pairs.cuh - two x-adjacent cells per thread for the FP32/FP16 two-kernel step.
//
// Populations move between HBM and registers as 2-element vectors (float2 / half2), so one
// warp request covers 64 cells of a direction plane (256 B FP32, 128 B FP16) instead of 32.
// With scalar FP16 loads each request carried 64 B while the collision arithmetic spread
// the requests out in time, and the loads waited about three times as long as FP32 loads
// for the same instruction count; vector requests give FP16 the FP32 request size.
//
// A pull along x shifts the pair by one element: it is assembled from the two aligned
// vectors that hold it.  Cells whose source lies outside the lattice (the x faces for the
// cell at the face, every direction with an out-of-range y or z source) take the scalar
// pull with the reference's boundary rule, so the values are those of the one-cell path.
// The per-cell arithmetic is the same inline functions in the same order.
#pragma once

#include "lbm_fast_cells.cuh"

namespace lbm {

template <class S> struct Vec2;
template <> struct Vec2<float> {
    __device__ static __forceinline__ float2 ld(const float* p, long long i) {
        return __ldg(reinterpret_cast<const float2*>(p + i));
    }
    __device__ static __forceinline__ void st(float* p, long long i, float a, float b) {
        *reinterpret_cast<float2*>(p + i) = make_float2(a, b);
    }
    // two values already in the storage type
    __device__ static __forceinline__ void st_raw(float* p, long long i, float a, float b) { st(p, i, a, b); }
};
template <> struct Vec2<__half> {
    __device__ static __forceinline__ float2 ld(const __half* p, long long i) {
        const unsigned int w = __ldg(reinterpret_cast<const unsigned int*>(p + i));
        return __half22float2(__halves2half2(__ushort_as_half((unsigned short)(w & 0xFFFFu)),
                                             __ushort_as_half((unsigned short)(w >> 16))));
    }
    __device__ static __forceinline__ void st(__half* p, long long i, float a, float b) {
        // each half rounds as __float2half_rn does in the one-cell path
        const unsigned int lo = __half_as_ushort(__float2half_rn(a)), hi = __half_as_ushort(__float2half_rn(b));
        *reinterpret_cast<unsigned int*>(p + i) = lo | (hi << 16);
    }
    // two values already in the storage type
    __device__ static __forceinline__ void st_raw(__half* p, long long i, __half a, __half b) {
        *reinterpret_cast<unsigned int*>(p + i) = (unsigned int)__half_as_ushort(a) | ((unsigned int)__half_as_ushort(b) << 16);
    }
};

__device__ __forceinline__ float2 ldf2(const float* p, long long i) { return __ldg(reinterpret_cast<const float2*>(p + i)); }
__device__ __forceinline__ void stf2(float* p, long long i, float a, float b) {
    *reinterpret_cast<float2*>(p + i) = make_float2(a, b);
}

// Values of direction a pulled into cells (i0, .) and (i0+1, .) from the source row that
// starts at `row` (the row of (sj, sk) in plane a), both sources inside the lattice in x.
template <int Q, class S>
__device__ __forceinline__ float2 vec_pull_row(const Geo& g, const S* __restrict__ p, int a, int i0, long long row) {
    const int ex = Lat<Q>::ex(a);
    if (ex == 0) return Vec2<S>::ld(p, row + i0);
    if (ex == 1) {  // sources i0-1 and i0
        const float2 lo = Vec2<S>::ld(p, row + (i0 > 0 ? i0 - 2 : 0));
        const float2 hi = Vec2<S>::ld(p, row + i0);
        return make_float2(lo.y, hi.x);
    }
    // ex == -1: sources i0+1 and i0+2
    const float2 lo = Vec2<S>::ld(p, row + i0);
    const float2 hi = Vec2<S>::ld(p, row + (i0 + 2 < g.nx ? i0 + 2 : i0));
    return make_float2(lo.y, hi.x);
}

template <int Q, class S, class LOAD>
__device__ __forceinline__ float2 pull_flow_pair(const Geo& g, const S* __restrict__ p, int a, int i0, int j, int k,
                                                 long long c0, long long n, LOAD load) {
    const int ex = Lat<Q>::ex(a), ey = Lat<Q>::ey(a), ez = Lat<Q>::ez(a);
    const int sj = j - ey, sk = k - ez;
    const bool yz = (ey == 0 || (sj >= 0 && sj < g.ny)) && (ez == 0 || (sk >= 0 && sk < g.nz));
    float2 v = make_float2(0.0f, 0.0f);
    if (yz) v = vec_pull_row<Q, S>(g, p, a, i0, (long long)a * n + (long long)g.nx * ((long long)sj + (long long)g.ny * sk));
    if (!yz || (ex == 1 && i0 == 0)) v.x = pull_flow<Q, float>(g, a, i0, j, k, c0, load);
    if (!yz || (ex == -1 && i0 + 2 >= g.nx)) v.y = pull_flow<Q, float>(g, a, i0 + 1, j, k, c0 + 1, load);
    return v;
}

template <int QT, class S, class LOAD>
__device__ __forceinline__ float2 pull_thermal_pair(const Geo& g, const S* __restrict__ p, int a, int i0, int j, int k,
                                                    long long c0, long long n, LOAD load) {
    const int ex = Lat<QT>::ex(a), ey = Lat<QT>::ey(a), ez = Lat<QT>::ez(a);
    const int sj = j - ey, sk = k - ez;
    const bool yz = (ey == 0 || (sj >= 0 && sj < g.ny)) && (ez == 0 || (sk >= 0 && sk < g.nz));
    float2 v = make_float2(0.0f, 0.0f);
    if (yz) v = vec_pull_row<QT, S>(g, p, a, i0, (long long)a * n + (long long)g.nx * ((long long)sj + (long long)g.ny * sk));
    if (!yz || (ex == 1 && i0 == 0)) v.x = pull_thermal<QT, float>(g, a, i0, j, k, c0, load);
    if (!yz || (ex == -1 && i0 + 2 >= g.nx)) v.y = pull_thermal<QT, float>(g, a, i0 + 1, j, k, c0 + 1, load);
    return v;
}

// flow_cell_2k (not FIRST) for the cells c0 = (i0, j, k) and c0 + 1.
template <int D, class S>
__device__ __forceinline__ void flow_pair_2k(const Geo& g, const PhysF& P, const FastArgs<S>& A, const S* __restrict__ fin,
                                             const S* __restrict__ gin, S* __restrict__ fout, long long c0, int i0, int j,
                                             int k) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    auto lf = [&](int a, long long cc) { return ldS(fin, a * n + cc); };
    auto lg = [&](int a, long long cc) { return ldS(gin, a * n + cc); };
    float d0[Q], d1[Q];
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        const float2 v = pull_flow_pair<Q, S>(g, fin, a, i0, j, k, c0, n, lf);
        d0[a] = v.x;
        d1[a] = v.y;
    }
    float ts0 = 0.0f, ts1 = 0.0f;
#pragma unroll
    for (int a = 0; a < QT; ++a) {
        const float2 e = pull_thermal_pair<QT, S>(g, gin, a, i0, j, k, c0, n, lg);
        ts0 += e.x;
        ts1 += e.y;
    }
    const float2 lag = ldf2(A.lag_in, c0);
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
#pragma unroll
    for (int a = 0; a < Q; ++a) Vec2<S>::st_raw(fout, a * n + c0, h0[a], h1[a]);
}

// thermal_cell_2k (not FIRST) for the cells c0 and c0 + 1.
template <int D, class S>
__device__ __forceinline__ void thermal_pair_2k(const Geo& g, const PhysF& P, const FastArgs<S>& A,
                                                const S* __restrict__ fin, const S* __restrict__ gin, S* __restrict__ gout,
                                                long long c0, int i0, int j, int k) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    auto lf = [&](int a, long long cc) { return ldS(fin, a * n + cc); };
    auto lg = [&](int a, long long cc) { return ldS(gin, a * n + cc); };
    float d0[Q], d1[Q], G0[QT], G1[QT];
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        const float2 v = pull_flow_pair<Q, S>(g, fin, a, i0, j, k, c0, n, lf);
        d0[a] = v.x;
        d1[a] = v.y;
    }
    float ts0 = 0.0f, ts1 = 0.0f;
#pragma unroll
    for (int a = 0; a < QT; ++a) {
        const float2 e = pull_thermal_pair<QT, S>(g, gin, a, i0, j, k, c0, n, lg);
        G0[a] = e.x + wT<QT>(P, a) * P.Tref;
        G1[a] = e.y + wT<QT>(P, a) * P.Tref;
        ts0 += G0[a];
        ts1 += G1[a];
    }
    const float2 bx = ldf2(A.Bin0, c0), by = ldf2(A.Bin1, c0);
    const float2 bz = D == 3 ? ldf2(A.Bin2, c0) : make_float2(0.0f, 0.0f);
    const float2 lag = D == 2 ? ldf2(A.lag_in, c0) : make_float2(0.0f, 0.0f);
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
#pragma unroll
    for (int a = 0; a < QT; ++a) Vec2<S>::st_raw(gout, a * n + c0, h0[a], h1[a]);
}

}  // namespace lbm
