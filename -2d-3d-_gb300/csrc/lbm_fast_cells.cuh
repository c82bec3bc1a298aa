// lbm_fast_cells.cuh - per-cell bodies of the two-kernel FP32/FP16 step, shared by the
// single-lattice kernels (lbm_fast.cu) and the batched many-lattice kernels
// (lbm_ensemble.cu), so both run the same arithmetic.
#pragma once

#include "lbm_fast_math.cuh"

namespace lbm {

// Resident blocks per SM requested from the one-cell kernels (128 threads).  Measured on
// GB300: the FP16 kernels and the FP32 thermal kernels run faster with 10 (48 registers,
// a few bytes of spill) than with the compiler's own choice (56-64 registers, 8 blocks),
// which keeps more loads in flight; the FP32 flow kernels run slower with it.
template <class S, bool THERMAL>
struct OneCellBlocks {
    static constexpr int value = (sizeof(S) == 2 || THERMAL) ? 10 : 0;  // 0: no minimum
};

// Pointers of one launch: module arrays plus the B_prev / lag buffers to read and write.
template <class S>
struct FastArgs {
    S *fref, *gref;
    float *rho, *u, *v, *w, *T;
    const float *Bin0, *Bin1, *Bin2;
    float *Bout0, *Bout1, *Bout2;
    const float* lag_in;
    float* lag_out;
    const unsigned long long* tick;  // the lattice's step counter (stochastic rounding)
};

// Flow collision of step n: f_post_n from f_post_{n-1} (or the module arrays when FIRST).
// Reads lag_in (3D: T_{n-2}; 2D: F_y,n-1); writes lag_out (2D: F_y,n).  INNER: cells off
// the lattice's faces pull at fixed offsets without the boundary tests (the batched kernels
// leave it off: their persistent loops would carry both paths' registers).
// I: index type of the cell's own accesses and of the fixed-offset pulls (int where every
// array index fits in 32 bits; the values do not depend on it).
template <int D, bool FIRST, class S, bool INNER = true, class I = long long>
__device__ __forceinline__ void flow_cell_2k(const Geo& g, const PhysF& P, const FastArgs<S>& A, const S* __restrict__ fin,
                                             const S* __restrict__ gin, S* __restrict__ fout, long long c, int i, int j,
                                             int k) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    const I ni = (I)g.ncell, ci = (I)c;
    float d[Q], dp[Q], dr, rho, u, v, w = 0.0f, T;
    if (FIRST) {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldS(A.fref, a * ni + ci);
        rho = A.rho[ci];
        dr = rho - 1.0f;
        u = A.u[ci];
        v = A.v[ci];
        if (D == 3) w = A.w[ci];
        T = A.T[ci];
    } else {
        // loads only in the branch: the arithmetic after it is one sequence for every cell,
        // so FMA contraction rounds it as in the paired and staged kernels
        float ts = 0.0f;
        if (INNER && aa_inner(g, i, j, k)) {  // no pull off the faces needs a boundary rule
#pragma unroll
            for (int a = 0; a < Q; ++a) d[a] = ldS(fin, a * ni + ci - (I)lat_off<Q>(g, a));
#pragma unroll
            for (int a = 0; a < QT; ++a) ts += ldS(gin, a * ni + ci - (I)lat_off<QT>(g, a));
        } else {
            auto lf = [&](int a, long long cc) { return ldS(fin, a * n + cc); };
            auto lg = [&](int a, long long cc) { return ldS(gin, a * n + cc); };
#pragma unroll
            for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, float>(g, a, i, j, k, c, lf);
#pragma unroll
            for (int a = 0; a < QT; ++a) ts += pull_thermal<QT, float>(g, a, i, j, k, c, lg);
        }
        T = ts + P.Tref;  // sum of deviations + Tref * sum(wT)
        float Fy;
        fmacro<D>(d, A.lag_in[ci], P, dr, rho, u, v, w, Fy);
    }
    const float Fy = rho * P.gBeta * (T - P.Tref);
    if (D == 2) {
        A.lag_out[ci] = Fy;
        fcollide_2d(d, dr, rho, u, v, Fy, P, dp);
    } else {
        fcollide_3d(d, dr, rho, u, v, w, Fy, P, dp);
    }
    S hs[Q];
    round_cell<Q>(dp, hs, P.sr != 0, sr_seed(*A.tick, c, 0));
#pragma unroll
    for (int a = 0; a < Q; ++a) fout[a * ni + ci] = hs[a];
}

// Streaming, boundary and macro of the flow, and thermal collision of step n.
// 2D reads lag_in = F_y,n; 3D writes lag_out = T_{n-1}.
template <int D, bool FIRST, class S, bool INNER = true, class I = long long>
__device__ __forceinline__ void thermal_cell_2k(const Geo& g, const PhysF& P, const FastArgs<S>& A, const S* __restrict__ fin,
                                             const S* __restrict__ gin, S* __restrict__ gout, long long c, int i, int j,
                                             int k) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    const I ni = (I)g.ncell, ci = (I)c;
    float d[Q], G[QT], GP[QT];
    const bool inner = INNER && aa_inner(g, i, j, k);  // no pull needs a boundary rule
    auto lf = [&](int a, long long cc) { return ldS(fin, a * n + cc); };
    if (inner) {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldS(fin, a * ni + ci - (I)lat_off<Q>(g, a));
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, float>(g, a, i, j, k, c, lf);
    }
    float Tprev;
    if (FIRST) {
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = ldS(A.gref, a * ni + ci) + wT<QT>(P, a) * P.Tref;
        Tprev = A.T[ci];
    } else if (inner) {
        float ts = 0.0f;
#pragma unroll
        for (int a = 0; a < QT; ++a) {
            G[a] = ldS(gin, a * ni + ci - (I)lat_off<QT>(g, a)) + wT<QT>(P, a) * P.Tref;
            ts += G[a];
        }
        Tprev = ts;
    } else {
        auto lg = [&](int a, long long cc) { return ldS(gin, a * n + cc); };
        float ts = 0.0f;
#pragma unroll
        for (int a = 0; a < QT; ++a) {
            G[a] = pull_thermal<QT, float>(g, a, i, j, k, c, lg) + wT<QT>(P, a) * P.Tref;
            ts += G[a];
        }
        Tprev = ts;
    }
    float dr, rho, u, v, w, Fy;
    fmacro<D>(d, D == 2 ? A.lag_in[ci] : Tprev, P, dr, rho, u, v, w, Fy);
    if (D == 2) {
        float Bx = A.Bin0[ci], By = A.Bin1[ci];
        fcollideT_2d(G, u, v, Tprev, Bx, By, P, GP);
        A.Bout0[ci] = Bx;
        A.Bout1[ci] = By;
    } else {
        float Bx = A.Bin0[ci], By = A.Bin1[ci], Bz = A.Bin2[ci];
        fcollideT_3d(G, u, v, w, Tprev, Bx, By, Bz, P, GP);
        A.Bout0[ci] = Bx;
        A.Bout1[ci] = By;
        A.Bout2[ci] = Bz;
        A.lag_out[ci] = Tprev;
    }
    float ev[QT];
    S hs[QT];
#pragma unroll
    for (int a = 0; a < QT; ++a) ev[a] = GP[a] - wT<QT>(P, a) * P.Tref;
    round_cell<QT>(ev, hs, P.sr != 0, sr_seed(*A.tick, c, 1));
#pragma unroll
    for (int a = 0; a < QT; ++a) gout[a * ni + ci] = hs[a];
}

// The steady-state bodies above for a cell of an interior row (0 < j < ny-1 and, in 3D,
// 0 < k < nz-1): only the x axis can take a pull source outside the lattice, which the row
// pulls resolve with selects (pull_flow_xrow / pull_thermal_xrow: the same sources and
// rules), so a warp runs one instruction stream whatever its lanes' x positions.  The
// arithmetic after the pulls is flow_cell_2k's / thermal_cell_2k's, statement for
// statement.
template <int D, class S>
__device__ __forceinline__ void flow_cell_row(const Geo& g, const PhysF& P, const FastArgs<S>& A,
                                              const S* __restrict__ fin, const S* __restrict__ gin,
                                              S* __restrict__ fout, long long c, int i) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    auto lf = [&](int a, long long cc) { return ldS(fin, a * n + cc); };
    auto lg = [&](int a, long long cc) { return ldS(gin, a * n + cc); };
    float d[Q], dp[Q], dr, rho, u, v, w = 0.0f, T;
    {
        float ts = 0.0f;
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow_xrow<Q, float>(g, a, i, c, lf);
#pragma unroll
        for (int a = 0; a < QT; ++a) ts += pull_thermal_xrow<QT, float>(g, a, i, c, lg);
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
    S hs[Q];
    round_cell<Q>(dp, hs, P.sr != 0, sr_seed(*A.tick, c, 0));
#pragma unroll
    for (int a = 0; a < Q; ++a) fout[a * n + c] = hs[a];
}

template <int D, class S>
__device__ __forceinline__ void thermal_cell_row(const Geo& g, const PhysF& P, const FastArgs<S>& A,
                                                 const S* __restrict__ fin, const S* __restrict__ gin,
                                                 S* __restrict__ gout, long long c, int i) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    auto lf = [&](int a, long long cc) { return ldS(fin, a * n + cc); };
    auto lg = [&](int a, long long cc) { return ldS(gin, a * n + cc); };
    float d[Q], G[QT], GP[QT];
#pragma unroll
    for (int a = 0; a < Q; ++a) d[a] = pull_flow_xrow<Q, float>(g, a, i, c, lf);
    float Tprev;
    {
        float ts = 0.0f;
#pragma unroll
        for (int a = 0; a < QT; ++a) {
            G[a] = pull_thermal_xrow<QT, float>(g, a, i, c, lg) + wT<QT>(P, a) * P.Tref;
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
#pragma unroll
    for (int a = 0; a < QT; ++a) gout[a * n + c] = hs[a];
}

}  // namespace lbm
