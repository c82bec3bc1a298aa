// lbm_fast_aa.cuh - per-cell bodies of the in-place (AA) FP32/FP16 step, shared by the
// one-cell kernels (lbm_fast_aa.cu) and the face cells of the staged kernels
// (lbm_fast_tma.cu).  The arithmetic is flow_cell_2k's and thermal_cell_2k's; only the
// slots read and written differ (layouts in lbm_device.cuh).
#pragma once

#include "lbm_fast_cells.cuh"

namespace lbm {

// Loads from the array the sweep also writes.  They take the read-only path: in a sweep
// every slot is read only by the cell that owns it and written only by that cell after all
// of its reads (each stored value depends on every value the cell loaded, so no store can
// be moved above a load), and the face snapshot is a separate buffer.  No thread can see a
// value written earlier in the same sweep, which is the read-only path's one condition.
// Plain loads here would force the compiler to keep every load ordered against the
// stores of possibly aliasing pointers, doubling the register count of the odd sweep.
template <class S> __device__ __forceinline__ float ldA(const S* p, long long i) { return ldS<S>(p, i); }

// The value the module array of storage type S holds for an arithmetic value x.
template <class S> __device__ __forceinline__ float roundS(float x) { return x; }
template <> __device__ __forceinline__ float roundS<__half>(float x) { return __half2float(__float2half_rn(x)); }

// Flow collision of one cell.  ODD: f is in the swapped layout (pull, then push);
// otherwise streamed (own slots, written back swapped).  gpar: layout of g (read only).
template <int D, class S, bool ODD, bool FIRST>
__device__ __forceinline__ void aa_flow_cell(const Geo& g, const PhysF& P, const FastArgs<S>& A, S* f,
                                             const S* __restrict__ gs, const AAFace<S>& wf, int gpar, int graw,
                                             long long c, int i, int j, int k) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    float d[Q], dp[Q], dr, rho, u, v, w = 0.0f, T;
    const bool inner = aa_inner(g, i, j, k);  // no boundary rule on any pull or push
    if (ODD && inner) {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldA(f, Lat<Q>::opp(a) * n + c - lat_off<Q>(g, a));
    } else if (ODD) {
        auto lf = [&](int b, long long cc) { return ldA(f, Lat<Q>::opp(b) * n + cc); };
        auto wr = [&](int ax, int b, long long) {
            return ldA(aa_face_ptr(wf, ax), b * aa_face_cells(g, ax) + aa_face_index(g, ax, i, j, k));
        };
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow_w<Q, float>(g, a, i, j, k, c, lf, wr);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldA(f, a * n + c);
    }
    if (FIRST) {
        rho = A.rho[c];
        dr = rho - 1.0f;
        u = A.u[c];
        v = A.v[c];
        if (D == 3) w = A.w[c];
        T = A.T[c];
    } else {
        float ts = 0.0f;
        if (gpar && inner) {
#pragma unroll
            for (int a = 0; a < QT; ++a) ts += ldS(gs, Lat<QT>::opp(a) * n + c - lat_off<QT>(g, a));
        } else if (gpar) {
            auto lg = [&](int b, long long cc) { return ldS(gs, Lat<QT>::opp(b) * n + cc); };
#pragma unroll
            for (int a = 0; a < QT; ++a) ts += pull_thermal<QT, float>(g, a, i, j, k, c, lg);
        } else if (inner) {
#pragma unroll
            for (int a = 0; a < QT; ++a) ts += ldS(gs, a * n + c);
        } else {
            auto lg = [&](int b, long long cc) { return ldS(gs, b * n + cc); };
#pragma unroll
            for (int a = 0; a < QT; ++a) ts += aa_local_thermal<QT, float>(g, a, i, j, k, c, graw != 0, lg);
        }
        T = ts + P.Tref;
        float Fy;
        fmacro<D>(d, A.lag_in[c], P, dr, rho, u, v, w, Fy);
    }
    const float Fy = rho * P.gBeta * (T - P.Tref);
    if (D == 2) {
        A.lag_out[c] = Fy;
        fcollide_2d(d, dr, rho, u, v, Fy, P, dp);
    } else {
        fcollide_3d(d, dr, rho, u, v, w, Fy, P, dp);
    }
    // rounded by source cell and direction (the two-buffer kernels' bits); the push only
    // routes the stored value
    S hs[Q];
    round_cell<Q>(dp, hs, P.sr != 0, sr_seed(*A.tick, c, 0));
    if (ODD && inner) {
#pragma unroll
        for (int a = 0; a < Q; ++a) f[a * n + c + lat_off<Q>(g, a)] = hs[a];
    } else if (ODD) {
        auto st = [&](int b, long long cc, S val) { f[b * n + cc] = val; };
#pragma unroll
        for (int a = 0; a < Q; ++a) aa_push<Q, false, S>(g, a, i, j, k, c, hs[a], st);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) f[Lat<Q>::opp(a) * n + c] = hs[a];
    }
}

// Thermal collision of one cell.  ODD: g is in the swapped layout; fpar: layout of f.
template <int D, class S, bool ODD, bool FIRST>
__device__ __forceinline__ void aa_thermal_cell(const Geo& g, const PhysF& P, const FastArgs<S>& A,
                                                const S* __restrict__ fs, S* gg, const AAFace<S>& wg, int fpar,
                                                int graw, long long c, int i, int j, int k) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    float d[Q], G[QT], GP[QT];
    const bool inner = aa_inner(g, i, j, k);  // no boundary rule on any pull or push
    if (fpar && inner) {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldS(fs, Lat<Q>::opp(a) * n + c - lat_off<Q>(g, a));
    } else if (fpar) {
        auto lf = [&](int b, long long cc) { return ldS(fs, Lat<Q>::opp(b) * n + cc); };
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, float>(g, a, i, j, k, c, lf);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldS(fs, a * n + c);
    }
    float e[QT];
    if (ODD && inner) {
#pragma unroll
        for (int a = 0; a < QT; ++a) e[a] = ldA(gg, Lat<QT>::opp(a) * n + c - lat_off<QT>(g, a));
    } else if (ODD) {
        auto lg = [&](int b, long long cc) { return ldA(gg, Lat<QT>::opp(b) * n + cc); };
        auto wr = [&](int ax, int b, long long) {
            return ldA(aa_face_ptr(wg, ax), b * aa_face_cells(g, ax) + aa_face_index(g, ax, i, j, k));
        };
#pragma unroll
        for (int a = 0; a < QT; ++a) e[a] = pull_thermal_w<QT, float>(g, a, i, j, k, c, lg, wr);
    } else if (inner) {
#pragma unroll
        for (int a = 0; a < QT; ++a) e[a] = ldA(gg, a * n + c);
    } else {
        auto lg = [&](int b, long long cc) { return ldA(gg, b * n + cc); };
#pragma unroll
        for (int a = 0; a < QT; ++a) e[a] = aa_local_thermal<QT, float>(g, a, i, j, k, c, graw != 0, lg);
    }
    float Tprev;
    if (FIRST) {
        // the module array holds each value rounded to the storage type
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = roundS<S>(e[a]) + wT<QT>(P, a) * P.Tref;
        Tprev = A.T[c];
    } else {
        float ts = 0.0f;
#pragma unroll
        for (int a = 0; a < QT; ++a) {
            G[a] = e[a] + wT<QT>(P, a) * P.Tref;
            ts += G[a];
        }
        Tprev = ts;
    }
    float dr, rho, u, v, w, Fy;
    fmacro<D>(d, D == 2 ? A.lag_in[c] : Tprev, P, dr, rho, u, v, w, Fy);
    if (D == 2) {
        float Bx = A.Bin0[c], By = A.Bin1[c];
        fcollideT_2d(G, u, v, Tprev, Bx, By, P, GP);
        A.Bout0[c] = Bx;
        A.Bout1[c] = By;
    } else {
        float Bx = A.Bin0[c], By = A.Bin1[c], Bz = A.Bin2[c];
        fcollideT_3d(G, u, v, w, Tprev, Bx, By, Bz, P, GP);
        A.Bout0[c] = Bx;
        A.Bout1[c] = By;
        A.Bout2[c] = Bz;
        A.lag_out[c] = Tprev;
    }
    float ev[QT];
    S hs[QT];
#pragma unroll
    for (int a = 0; a < QT; ++a) ev[a] = GP[a] - wT<QT>(P, a) * P.Tref;
    round_cell<QT>(ev, hs, P.sr != 0, sr_seed(*A.tick, c, 1));
    if (ODD && inner) {
#pragma unroll
        for (int a = 0; a < QT; ++a) gg[a * n + c + lat_off<QT>(g, a)] = hs[a];
    } else if (ODD) {
        auto st = [&](int b, long long cc, S val) { gg[b * n + cc] = val; };
#pragma unroll
        for (int a = 0; a < QT; ++a) aa_push<QT, true, S>(g, a, i, j, k, c, hs[a], st);
    } else {
#pragma unroll
        for (int a = 0; a < QT; ++a) gg[Lat<QT>::opp(a) * n + c] = hs[a];
    }
}

}  // namespace lbm
