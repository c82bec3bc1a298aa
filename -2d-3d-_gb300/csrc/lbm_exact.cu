// lbm_exact.cu - the plain method: FP64 kernels that reproduce the reference's arithmetic.
//
// Compiled with -fmad=false (no multiply-add contraction) and IEEE division/sqrt, with
// every expression in the reference's left-to-right order, so each kernel returns the
// same bits as the reference's loop body on the same inputs.
//
//  * Stage kernels: one per reference subroutine (collision .. macroT), operating on the
//    reference's module arrays (f, f_post, rho, u, v, w, T, ...), for stage-by-stage parity.
//  * Fused step: two kernels per time step over SoA population buffers:
//      k_flow    : pull f_post_{n-1} + boundary rule -> f_{n-1}; pull g_post_{n-1} ->
//                  T_{n-1}; MRT collision -> f_post_n, with rho, u and the momentum sums
//                  of f_{n-1} from the previous thermal kernel's macro step (same values,
//                  not recomputed).
//      k_thermal : pull f_post_n -> f_n, macro -> rho_n, u_n (stored with the sums);
//                  pull g_post_{n-1} -> g_{n-1} (T_{n-1} from the flow kernel); thermal MRT
//                  collision with the M1G term -> g_post_n, B_prev, T lag.
//    The reference's step order (collision, streaming, bounceback, macro, collisionT,
//    streamingT, bouncebackT, macroT, 3DRB.F90:227-241) couples flow step n+1 to the
//    thermal streaming of step n (a dependency cone of radius 2), so one pass per step
//    cannot pull both; the split keeps each kernel a radius-1 pull.
#include <cuda_runtime.h>

#include "lbm_device.cuh"
#include "lbm_exact_cell.cuh"
#include "lbm_internal.h"

namespace lbm {

__device__ __forceinline__ bool thread_cell(const Geo& g, long long& c, int& i, int& j, int& k) {
    c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return false;
    cell_coords(g, c, i, j, k);
    return true;
}

// ------------------------------------------------------------------------------------
// initial (2DRB.F90:460-617, 3DRB.F90:445-603), loadInitField = 0
// ------------------------------------------------------------------------------------
template <int D>
__global__ void k_initial(Geo g, PhysC P, InitC I, ExactArrays A) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    // xp(i) = (i - 0.5)/lengthUnit, xp(0) = 0, xp(nx+1) = nx/lengthUnit (1-based Fortran i)
    const double xpi = ((double)(i + 1) - 0.5) / I.L, yp_j = ((double)(j + 1) - 0.5) / I.L;
    const double xp0 = 0.0 / I.L, xpe = (double)g.nx / I.L, yp0 = 0.0 / I.L, ype = (double)g.ny / I.L;
    double T = 0.0;
    if (g.bct[0] == LBM_BCT_CONST) T = I.Thot + (xpi - xp0) / (xpe - xp0) * (I.Tcold - I.Thot);
    if (g.bct[1] == LBM_BCT_CONST) {
        T = I.Thot + (yp_j - yp0) / (ype - yp0) * (I.Tcold - I.Thot);
        if (I.perturb) T = T + I.pert_amp * I.sx[i] * I.sy[j];
    }
    if (I.noise_amp != 0.0) T = T + I.noise_amp * (2.0 * noise_xi(I.seed, (uint64_t)c) - 1.0);
    const double rho = 1.0, u = 0.0, v = 0.0, w = 0.0;
    A.rho[c] = rho;
    A.u[c] = u;
    A.v[c] = v;
    A.T[c] = T;
    if (D == 3) A.w[c] = w;
    const long long n = g.ncell;
    if (D == 2) {
        const double us2 = u * u + v * v;
#pragma unroll
        for (int a = 0; a < 9; ++a) {
            const double un = u * (double)Lat<9>::ex(a) + v * (double)Lat<9>::ey(a);
            const double om = (a == 0) ? 4.0 / 9.0 : (a <= 4 ? 1.0 / 9.0 : 1.0 / 36.0);
            A.f[a * n + c] = rho * om * (1.0 + 3.0 * un + 4.5 * un * un - 1.5 * us2);
        }
#pragma unroll
        for (int a = 0; a < 5; ++a) {
            const double un = u * (double)Lat<9>::ex(a) + v * (double)Lat<9>::ey(a);
            const double omT = (a == 0) ? P.omegaT0 : P.omegaT1;
            A.g[a * n + c] = omT * T * (1.0 + P.geqc * un);
        }
    } else {
        const double u2Loc = u * u + v * v + w * w;
#pragma unroll
        for (int a = 0; a < 19; ++a) {
            const double eu = (double)Lat<19>::ex(a) * u + (double)Lat<19>::ey(a) * v + (double)Lat<19>::ez(a) * w;
            const double om = (a == 0) ? 1.0 / 3.0 : (a <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
            A.f[a * n + c] = om * rho * (1.0 + 3.0 * eu + 4.5 * eu * eu - 1.5 * u2Loc);
        }
#pragma unroll
        for (int a = 0; a < 7; ++a) {
            const double eu = (double)Lat<7>::ex(a) * u + (double)Lat<7>::ey(a) * v + (double)Lat<7>::ez(a) * w;
            const double omT = (a == 0) ? P.omegaT0 : P.omegaT1;
            A.g[a * n + c] = omT * T * (1.0 + P.geqc * eu);
        }
    }
    A.Bx[c] = P.use_g ? u * T : 0.0;
    A.By[c] = P.use_g ? v * T : 0.0;
    if (D == 3) A.Bz[c] = P.use_g ? w * T : 0.0;
    if (D == 2) {
        A.Fx[c] = 0.0;
        A.Fy[c] = 0.0;
    }
    A.up[c] = 0.0;
    A.vp[c] = 0.0;
    A.Tp[c] = 0.0;
    if (D == 3) A.wp[c] = 0.0;
    // the in-place pattern has no post-collision arrays (null pointers)
    if (A.fpost) {
#pragma unroll
        for (int a = 0; a < Q; ++a) A.fpost[a * n + c] = 0.0;
    }
    if (A.gpost) {
#pragma unroll
        for (int a = 0; a < QT; ++a) A.gpost[a * n + c] = 0.0;
    }
}

// ------------------------------------------------------------------------------------
// Stage kernels: one per reference subroutine
// ------------------------------------------------------------------------------------
template <int D>
__global__ void k_collision(Geo g, PhysC P, ExactArrays A) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    const long long n = g.ncell;
    if (D == 2) {
        double F[9], FP[9], Fx, Fy;
#pragma unroll
        for (int a = 0; a < 9; ++a) F[a] = A.f[a * n + c];
        collide_2d(F, A.rho[c], A.u[c], A.v[c], A.T[c], P, FP, Fx, Fy);
        A.Fx[c] = Fx;
        A.Fy[c] = Fy;
#pragma unroll
        for (int a = 0; a < 9; ++a) A.fpost[a * n + c] = FP[a];
    } else {
        double F[19], FP[19];
#pragma unroll
        for (int a = 0; a < 19; ++a) F[a] = A.f[a * n + c];
        collide_3d(F, A.rho[c], A.u[c], A.v[c], A.w[c], A.T[c], P, FP);
#pragma unroll
        for (int a = 0; a < 19; ++a) A.fpost[a * n + c] = FP[a];
    }
}

// streaming: pull from the ghost-padded f_post; ghost cells are zero (2DRB.F90:787-795).
template <int Q>
__global__ void k_streaming(Geo g, const double* __restrict__ src, double* __restrict__ dst) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    const long long n = g.ncell;
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        const int si = i - Lat<Q>::ex(a), sj = j - Lat<Q>::ey(a), sk = k - Lat<Q>::ez(a);
        double val = 0.0;
        if (si >= 0 && si < g.nx && sj >= 0 && sj < g.ny && sk >= 0 && sk < g.nz) val = src[a * n + cell_index(g, si, sj, sk)];
        dst[a * n + c] = val;
    }
}

// bounceback / bouncebackT: the face rules applied in the reference's order to the
// cells of the boundary faces only.
template <int Q>
__global__ void k_bounceback(Geo g, const double* __restrict__ fpost, double* __restrict__ f) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    const bool onface = i == 0 || i == g.nx - 1 || j == 0 || j == g.ny - 1 || (Lat<Q>::D == 3 && (k == 0 || k == g.nz - 1));
    if (!onface) return;
    const long long n = g.ncell;
    auto load = [&](int a, long long cc) { return fpost[a * n + cc]; };
#pragma unroll
    for (int a = 1; a < Q; ++a) {
        const int si = i - Lat<Q>::ex(a), sj = j - Lat<Q>::ey(a), sk = k - Lat<Q>::ez(a);
        const bool out = si < 0 || si >= g.nx || sj < 0 || sj >= g.ny || sk < 0 || sk >= g.nz;
        if (out) f[a * n + c] = pull_flow<Q, double>(g, a, i, j, k, c, load);
    }
}

template <int QT>
__global__ void k_bouncebackT(Geo g, const double* __restrict__ gpost, double* __restrict__ gg) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    const bool onface = i == 0 || i == g.nx - 1 || j == 0 || j == g.ny - 1 || (Lat<QT>::D == 3 && (k == 0 || k == g.nz - 1));
    if (!onface) return;
    const long long n = g.ncell;
    auto load = [&](int a, long long cc) { return gpost[a * n + cc]; };
#pragma unroll
    for (int a = 1; a < QT; ++a) {
        const int si = i - Lat<QT>::ex(a), sj = j - Lat<QT>::ey(a), sk = k - Lat<QT>::ez(a);
        const bool out = si < 0 || si >= g.nx || sj < 0 || sj >= g.ny || sk < 0 || sk >= g.nz;
        if (out) gg[a * n + c] = pull_thermal<QT, double>(g, a, i, j, k, c, load);
    }
}

template <int D>
__global__ void k_macro(Geo g, PhysC P, ExactArrays A) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    const long long n = g.ncell;
    if (D == 2) {
        double F[9], rho, u, v;
#pragma unroll
        for (int a = 0; a < 9; ++a) F[a] = A.f[a * n + c];
        macro_2d(F, A.Fx[c], A.Fy[c], rho, u, v);
        A.rho[c] = rho;
        A.u[c] = u;
        A.v[c] = v;
    } else {
        double F[19], rho, u, v, w;
#pragma unroll
        for (int a = 0; a < 19; ++a) F[a] = A.f[a * n + c];
        macro_3d(F, A.T[c], P, rho, u, v, w);
        A.rho[c] = rho;
        A.u[c] = u;
        A.v[c] = v;
        A.w[c] = w;
    }
}

template <int D>
__global__ void k_collisionT(Geo g, PhysC P, ExactArrays A) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    const long long n = g.ncell;
    if (D == 2) {
        double G[5], GP[5], Bx, By;
#pragma unroll
        for (int a = 0; a < 5; ++a) G[a] = A.g[a * n + c];
        collideT_2d(G, A.u[c], A.v[c], A.T[c], A.Bx[c], A.By[c], P, GP, Bx, By);
        if (P.use_g) {
            A.Bx[c] = Bx;
            A.By[c] = By;
        }
#pragma unroll
        for (int a = 0; a < 5; ++a) A.gpost[a * n + c] = GP[a];
    } else {
        double G[7], GP[7], Bx, By, Bz;
#pragma unroll
        for (int a = 0; a < 7; ++a) G[a] = A.g[a * n + c];
        collideT_3d(G, A.u[c], A.v[c], A.w[c], A.T[c], A.Bx[c], A.By[c], A.Bz[c], P, GP, Bx, By, Bz);
        if (P.use_g) {
            A.Bx[c] = Bx;
            A.By[c] = By;
            A.Bz[c] = Bz;
        }
#pragma unroll
        for (int a = 0; a < 7; ++a) A.gpost[a * n + c] = GP[a];
    }
}

template <int QT>
__global__ void k_macroT(Geo g, const double* __restrict__ gg, double* __restrict__ T) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    const long long n = g.ncell;
    double G[QT];
#pragma unroll
    for (int a = 0; a < QT; ++a) G[a] = gg[a * n + c];
    T[c] = sumT<QT>(G);
}

// ------------------------------------------------------------------------------------
// Fused step kernels
// ------------------------------------------------------------------------------------
// Macro step of f_n (with the 2D force F_n or the 3D lag T_{n-1}) and the thermal
// collision of one cell.  The macro results (rho, u and the momentum sums) go to the module
// arrays: the next flow kernel pulls the same f_n and uses them instead of repeating the
// macro step (three IEEE divisions and 45 additions per cell in 3D, on GB300's narrow FP64
// pipe), and the module rho and u are those of step n as the reference's macro leaves them.
template <int D, bool KNOWN>
__device__ __forceinline__ void thermal_cell(const PhysC& P, const ExactArrays& A, long long c, const double* F,
                                             const double* G, double Tprev, double* GP) {
    if (D == 2) {
        double rho, u, v, jx, jy, Bx, By;
        macro_2d(F, A.Fx[c], A.Fy[c], rho, u, v, jx, jy);
        collideT_2d<KNOWN>(G, u, v, Tprev, A.Bx[c], A.By[c], P, GP, Bx, By);
        if (P.use_g) {
            A.Bx[c] = Bx;
            A.By[c] = By;
        }
        A.rho[c] = rho;
        A.u[c] = u;
        A.v[c] = v;
        A.jx[c] = jx;
        A.jy[c] = jy;
    } else {
        double rho, u, v, w, jx, jy, jz, Bx, By, Bz;
        macro_3d(F, Tprev, P, rho, u, v, w, jx, jy, jz);
        collideT_3d<KNOWN>(G, u, v, w, Tprev, A.Bx[c], A.By[c], A.Bz[c], P, GP, Bx, By, Bz);
        if (P.use_g) {
            A.Bx[c] = Bx;
            A.By[c] = By;
            A.Bz[c] = Bz;
        }
        A.Tlag[c] = Tprev;
        A.rho[c] = rho;
        A.u[c] = u;
        A.v[c] = v;
        A.w[c] = w;
        A.jx[c] = jx;
        A.jy[c] = jy;
        A.jz[c] = jz;
    }
}

// Flow collision of step n (A_n in the reference's order).  FIRST: the inputs are the
// reference's module arrays after `initial` or after a materialisation; otherwise they
// are rebuilt from the fused buffers: f_{n-1} = pull(f_post_{n-1}), T_{n-1} =
// sum pull(g_post_{n-1}) (stored for the thermal kernel), and rho, u_{n-1} and the momentum
// sums from the previous thermal kernel, which computed them from the same f_{n-1} with the
// lag (3D: T_{n-2}; 2D: the force F_{n-1} stored by the previous flow collision).
template <int D, bool FIRST>
__global__ void __launch_bounds__(128) k_flow(Geo g, PhysC P, ExactArrays A, const double* __restrict__ fin,
                                              const double* __restrict__ gin, double* __restrict__ fout) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    double F[Q], FP[Q], T, jx = 0.0, jy = 0.0, jz = 0.0;
    // rho and u: the module arrays after initial / a materialisation, otherwise the thermal
    // kernel's macro step of the same f_{n-1} (with the same lag), stored with its sums
    const double rho = A.rho[c], u = A.u[c], v = A.v[c], w = D == 3 ? A.w[c] : 0.0;
    if (FIRST) {
#pragma unroll
        for (int a = 0; a < Q; ++a) F[a] = A.f[a * n + c];
        T = A.T[c];
    } else {
        auto lf = [&](int a, long long cc) { return fin[a * n + cc]; };
        auto lg = [&](int a, long long cc) { return gin[a * n + cc]; };
#pragma unroll
        for (int a = 0; a < Q; ++a) F[a] = pull_flow<Q, double>(g, a, i, j, k, c, lf);
        double G[QT];
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = pull_thermal<QT, double>(g, a, i, j, k, c, lg);
        T = sumT<QT>(G);
        A.T[c] = T;  // T_{n-1}, the thermal kernel's n0 of the same pulled populations
        jx = A.jx[c];
        jy = A.jy[c];
        if (D == 3) jz = A.jz[c];
    }
    if (D == 2) {
        double Fx, Fy;
        collide_2d<!FIRST>(F, rho, u, v, T, P, FP, Fx, Fy, jx, jy);
        A.Fx[c] = Fx;
        A.Fy[c] = Fy;
    } else {
        collide_3d<!FIRST>(F, rho, u, v, w, T, P, FP, jx, jy, jz);
    }
#pragma unroll
    for (int a = 0; a < Q; ++a) fout[a * n + c] = FP[a];
}

// Streaming + boundary + macro of the flow and thermal collision of step n
// (B_n .. D_n).  FIRST: g_{n-1} and T_{n-1} are the module arrays; otherwise T_{n-1} is the
// flow kernel's sum of the same pulled g_{n-1}.
template <int D, bool FIRST>
__global__ void __launch_bounds__(128) k_thermal(Geo g, PhysC P, ExactArrays A, const double* __restrict__ fin,
                                                 const double* __restrict__ gin, double* __restrict__ gout) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    double F[Q], G[QT], GP[QT];
    auto lf = [&](int a, long long cc) { return fin[a * n + cc]; };
#pragma unroll
    for (int a = 0; a < Q; ++a) F[a] = pull_flow<Q, double>(g, a, i, j, k, c, lf);
    // T_{n-1}: the module T, or the flow kernel's sum of the same pulled g_{n-1}
    const double Tprev = A.T[c];
    if (FIRST) {
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = A.g[a * n + c];
    } else {
        auto lg = [&](int a, long long cc) { return gin[a * n + cc]; };
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = pull_thermal<QT, double>(g, a, i, j, k, c, lg);
    }
    thermal_cell<D, !FIRST>(P, A, c, F, G, Tprev, GP);
#pragma unroll
    for (int a = 0; a < QT; ++a) gout[a * n + c] = GP[a];
}

// Rebuild the reference's module arrays after fused step N: f_N, g_N (streamed, with
// boundaries), rho_N, u_N (with the lag), T_N.
template <int D>
__global__ void k_materialize(Geo g, PhysC P, ExactArrays A, const double* __restrict__ fin,
                              const double* __restrict__ gin) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    double F[Q], G[QT];
    auto lf = [&](int a, long long cc) { return fin[a * n + cc]; };
    auto lg = [&](int a, long long cc) { return gin[a * n + cc]; };
#pragma unroll
    for (int a = 0; a < Q; ++a) F[a] = pull_flow<Q, double>(g, a, i, j, k, c, lf);
#pragma unroll
    for (int a = 0; a < QT; ++a) G[a] = pull_thermal<QT, double>(g, a, i, j, k, c, lg);
    double rho, u, v, w;
    if (D == 2) {
        macro_2d(F, A.Fx[c], A.Fy[c], rho, u, v);
    } else {
        macro_3d(F, A.Tlag[c], P, rho, u, v, w);
        A.w[c] = w;
    }
    A.rho[c] = rho;
    A.u[c] = u;
    A.v[c] = v;
    A.T[c] = sumT<QT>(G);
#pragma unroll
    for (int a = 0; a < Q; ++a) A.f[a * n + c] = F[a];
#pragma unroll
    for (int a = 0; a < QT; ++a) A.g[a * n + c] = G[a];
}

// ------------------------------------------------------------------------------------
// In-place (AA) form of the two fused kernels: one array per lattice, the layout parity
// of each array selects where a cell reads and writes (lbm_device.cuh).  The arithmetic
// is k_flow / k_thermal's, on the same values, so each state equals the two-buffer one.
// ODD: this kernel's own array is in the swapped layout (odd sweep: pull, then push).
// gpar / fpar: layout of the other array, which the kernel only reads.  graw: the thermal
// array's streamed slots were filled by pushes.  The own array is read through the
// read-only path although the sweep writes it: every slot is read only by the cell that
// owns it and written only by that cell after all of its reads (lbm_fast_aa.cu, ldA).
// ------------------------------------------------------------------------------------
// FIRST is a template parameter as in k_flow: with rho and u known to come from the macro
// step, the compiler reuses its sums in the collision's moment transform (a run-time
// choice repeats 45 additions on the FP64 pipe, 8% of the step on GB300).
template <int D, bool ODD, bool FIRST>
__global__ void __launch_bounds__(128) k_aa_flow(Geo g, PhysC P, ExactArrays A, double* f,
                                                 const double* __restrict__ gs, AAFace<double> wf, int gpar,
                                                 int graw) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    double F[Q], FP[Q], rho, u, v, w = 0.0, T;
    if (ODD) {
        auto lf = [&](int b, long long cc) { return __ldg(f + Lat<Q>::opp(b) * n + cc); };
        auto wr = [&](int ax, int b, long long) {
            return __ldg(aa_face_ptr(wf, ax) + b * aa_face_cells(g, ax) + aa_face_index(g, ax, i, j, k));
        };
#pragma unroll
        for (int a = 0; a < Q; ++a) F[a] = pull_flow_w<Q, double>(g, a, i, j, k, c, lf, wr);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) F[a] = __ldg(f + a * n + c);
    }
    double jx = 0.0, jy = 0.0, jz = 0.0;
    rho = A.rho[c];  // the module arrays, or the thermal kernel's macro step of the same f
    u = A.u[c];
    v = A.v[c];
    if (D == 3) w = A.w[c];
    if (FIRST) {
        T = A.T[c];
    } else {
        double G[QT];
        if (gpar) {
            auto lg = [&](int b, long long cc) { return gs[Lat<QT>::opp(b) * n + cc]; };
#pragma unroll
            for (int a = 0; a < QT; ++a) G[a] = pull_thermal<QT, double>(g, a, i, j, k, c, lg);
        } else {
            auto lg = [&](int b, long long cc) { return gs[b * n + cc]; };
#pragma unroll
            for (int a = 0; a < QT; ++a) G[a] = aa_local_thermal<QT, double>(g, a, i, j, k, c, graw != 0, lg);
        }
        T = sumT<QT>(G);
        A.T[c] = T;  // T_{n-1}, the thermal sweep's n0 of the same populations
        jx = A.jx[c];
        jy = A.jy[c];
        if (D == 3) jz = A.jz[c];
    }
    if (D == 2) {
        double Fx, Fy;
        collide_2d<!FIRST>(F, rho, u, v, T, P, FP, Fx, Fy, jx, jy);
        A.Fx[c] = Fx;
        A.Fy[c] = Fy;
    } else {
        collide_3d<!FIRST>(F, rho, u, v, w, T, P, FP, jx, jy, jz);
    }
    if (ODD) {
        auto st = [&](int b, long long cc, double val) { f[b * n + cc] = val; };
#pragma unroll
        for (int a = 0; a < Q; ++a) aa_push<Q, false, double>(g, a, i, j, k, c, FP[a], st);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) f[Lat<Q>::opp(a) * n + c] = FP[a];
    }
}

template <int D, bool ODD, bool FIRST>
__global__ void __launch_bounds__(128) k_aa_thermal(Geo g, PhysC P, ExactArrays A, const double* __restrict__ fs,
                                                    double* gg, AAFace<double> wg, int fpar, int graw) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    double F[Q], G[QT], GP[QT];
    if (fpar) {
        auto lf = [&](int b, long long cc) { return fs[Lat<Q>::opp(b) * n + cc]; };
#pragma unroll
        for (int a = 0; a < Q; ++a) F[a] = pull_flow<Q, double>(g, a, i, j, k, c, lf);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) F[a] = fs[a * n + c];
    }
    if (ODD) {
        auto lg = [&](int b, long long cc) { return __ldg(gg + Lat<QT>::opp(b) * n + cc); };
        auto wr = [&](int ax, int b, long long) {
            return __ldg(aa_face_ptr(wg, ax) + b * aa_face_cells(g, ax) + aa_face_index(g, ax, i, j, k));
        };
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = pull_thermal_w<QT, double>(g, a, i, j, k, c, lg, wr);
    } else {
        auto lg = [&](int b, long long cc) { return __ldg(gg + b * n + cc); };
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = aa_local_thermal<QT, double>(g, a, i, j, k, c, graw != 0, lg);
    }
    const double Tprev = A.T[c];  // the module T, or the flow sweep's sum of the same g_{n-1}
    thermal_cell<D, !FIRST>(P, A, c, F, G, Tprev, GP);
    if (ODD) {
        auto st = [&](int b, long long cc, double val) { gg[b * n + cc] = val; };
#pragma unroll
        for (int a = 0; a < QT; ++a) aa_push<QT, true, double>(g, a, i, j, k, c, GP[a], st);
    } else {
#pragma unroll
        for (int a = 0; a < QT; ++a) gg[Lat<QT>::opp(a) * n + c] = GP[a];
    }
}

// Module scalars of step N from the in-place arrays (k_materialize without the population
// copies: the arrays already are the module populations, read through their layout).
template <int D>
__global__ void k_aa_materialize(Geo g, PhysC P, ExactArrays A, const double* __restrict__ fs,
                                 const double* __restrict__ gs, int fpar, int gpar, int graw) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    double F[Q], G[QT];
    if (fpar) {
        auto lf = [&](int b, long long cc) { return fs[Lat<Q>::opp(b) * n + cc]; };
#pragma unroll
        for (int a = 0; a < Q; ++a) F[a] = pull_flow<Q, double>(g, a, i, j, k, c, lf);
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) F[a] = fs[a * n + c];
    }
    if (gpar) {
        auto lg = [&](int b, long long cc) { return gs[Lat<QT>::opp(b) * n + cc]; };
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = pull_thermal<QT, double>(g, a, i, j, k, c, lg);
    } else {
        auto lg = [&](int b, long long cc) { return gs[b * n + cc]; };
#pragma unroll
        for (int a = 0; a < QT; ++a) G[a] = aa_local_thermal<QT, double>(g, a, i, j, k, c, graw != 0, lg);
    }
    double rho, u, v, w;
    if (D == 2) {
        macro_2d(F, A.Fx[c], A.Fy[c], rho, u, v);
    } else {
        macro_3d(F, A.Tlag[c], P, rho, u, v, w);
        A.w[c] = w;
    }
    A.rho[c] = rho;
    A.u[c] = u;
    A.v[c] = v;
    A.T[c] = sumT<QT>(G);
}

// ------------------------------------------------------------------------------------
// restart reconstruction (reconstruct_macro_from_fg, 2DRB.F90:1144-1200,
// 3DRB.F90:1392-1463): T = sum g (the macroT call), rho = sum f, u = (mom + F/2)/rho with
// F = rho gBeta (T - Tref).  The reference iterates that assignment three times; without
// the magnetic force the right-hand side does not depend on u, so one pass gives the same
// value.
// ------------------------------------------------------------------------------------
template <int D>
__global__ void k_reconstruct(Geo g, PhysC P, ExactArrays A, unsigned int* bad) {
    long long c;
    int i, j, k;
    if (!thread_cell(g, c, i, j, k)) return;
    const long long n = g.ncell;
    constexpr int QT = (D == 2) ? 5 : 7;
    double G[QT];
#pragma unroll
    for (int a = 0; a < QT; ++a) G[a] = A.g[a * n + c];
    const double T = sumT<QT>(G);
    A.T[c] = T;
    if (D == 2) {
        double F[9];
#pragma unroll
        for (int a = 0; a < 9; ++a) F[a] = A.f[a * n + c];
        const double rho = F[0] + F[1] + F[2] + F[3] + F[4] + F[5] + F[6] + F[7] + F[8];
        const double momx = F[1] - F[3] + F[5] - F[6] - F[7] + F[8];
        const double momy = F[2] - F[4] + F[5] + F[6] - F[7] - F[8];
        double u = 0.0, v = 0.0, Fx = 0.0, Fy = 0.0;
        if (rho > 0.0) {
            u = momx / rho;
            v = momy / rho;
            // three fixed-point passes (2DRB.F90:1165-1177); with the magnetic force F depends on u
            for (int iter = 0; iter < (P.ha ? 3 : 1); ++iter) {
                Fx = 0.0;
                Fy = rho * P.gBeta * (T - P.Tref);
                if (P.ha) {
                    Fx = P.B2 * (v * P.sinphi * P.cosphi - u * P.sinphi * P.sinphi);
                    Fy = rho * P.gBeta * (T - P.Tref) + rho * P.B2 * (u * P.sinphi * P.cosphi - v * P.cosphi * P.cosphi);
                }
                u = (momx + 0.5 * Fx) / rho;
                v = (momy + 0.5 * Fy) / rho;
            }
        } else {
            *bad = 1u;
        }
        A.rho[c] = rho;
        A.u[c] = u;
        A.v[c] = v;
        A.Fx[c] = Fx;
        A.Fy[c] = Fy;
        if (P.use_g) {  // without EnableUseG the 2D reconstruction leaves B_prev as it is
            A.Bx[c] = u * T;
            A.By[c] = v * T;
        }
    } else {
        double f[19];
#pragma unroll
        for (int a = 0; a < 19; ++a) f[a] = A.f[a * n + c];
        const double rho = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11] + f[12]
                           + f[13] + f[14] + f[15] + f[16] + f[17] + f[18];
        const double momx = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
        const double momy = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
        const double momz = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
        double u = 0.0, v = 0.0, w = 0.0;
        if (rho > 0.0) {
            const double FxLoc = 0.0, FyLoc = rho * P.gBeta * (T - P.Tref), FzLoc = 0.0;
            u = (momx + 0.5 * FxLoc) / rho;
            v = (momy + 0.5 * FyLoc) / rho;
            w = (momz + 0.5 * FzLoc) / rho;
        } else {
            *bad = 1u;
        }
        A.rho[c] = rho;
        A.u[c] = u;
        A.v[c] = v;
        A.w[c] = w;
        A.Bx[c] = P.use_g ? u * T : 0.0;
        A.By[c] = P.use_g ? v * T : 0.0;
        A.Bz[c] = P.use_g ? w * T : 0.0;
    }
}

// ------------------------------------------------------------------------------------
// host launchers
// ------------------------------------------------------------------------------------
static inline unsigned nblocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

void exact_initial(const Geo& g, const PhysC& P, const InitC& I, const ExactArrays& A, int dim, cudaStream_t s) {
    if (dim == 2) k_initial<2><<<nblocks(g.ncell, 256), 256, 0, s>>>(g, P, I, A);
    else k_initial<3><<<nblocks(g.ncell, 256), 256, 0, s>>>(g, P, I, A);
}

void exact_stage(int stage, const Geo& g, const PhysC& P, const ExactArrays& A, int dim, cudaStream_t s) {
    const unsigned nb = nblocks(g.ncell, 128);
    const bool d3 = dim == 3;
    switch (stage) {
        case STAGE_COLLISION:
            if (d3) k_collision<3><<<nb, 128, 0, s>>>(g, P, A); else k_collision<2><<<nb, 128, 0, s>>>(g, P, A);
            break;
        case STAGE_STREAMING:
            if (d3) k_streaming<19><<<nb, 128, 0, s>>>(g, A.fpost, A.f); else k_streaming<9><<<nb, 128, 0, s>>>(g, A.fpost, A.f);
            break;
        case STAGE_BOUNCEBACK:
            if (d3) k_bounceback<19><<<nb, 128, 0, s>>>(g, A.fpost, A.f); else k_bounceback<9><<<nb, 128, 0, s>>>(g, A.fpost, A.f);
            break;
        case STAGE_MACRO:
            if (d3) k_macro<3><<<nb, 128, 0, s>>>(g, P, A); else k_macro<2><<<nb, 128, 0, s>>>(g, P, A);
            break;
        case STAGE_COLLISIONT:
            if (d3) k_collisionT<3><<<nb, 128, 0, s>>>(g, P, A); else k_collisionT<2><<<nb, 128, 0, s>>>(g, P, A);
            break;
        case STAGE_STREAMINGT:
            if (d3) k_streaming<7><<<nb, 128, 0, s>>>(g, A.gpost, A.g); else k_streaming<5><<<nb, 128, 0, s>>>(g, A.gpost, A.g);
            break;
        case STAGE_BOUNCEBACKT:
            if (d3) k_bouncebackT<7><<<nb, 128, 0, s>>>(g, A.gpost, A.g); else k_bouncebackT<5><<<nb, 128, 0, s>>>(g, A.gpost, A.g);
            break;
        case STAGE_MACROT:
            if (d3) k_macroT<7><<<nb, 128, 0, s>>>(g, A.g, A.T); else k_macroT<5><<<nb, 128, 0, s>>>(g, A.g, A.T);
            break;
        default: break;
    }
}

// Threads per block of the fused step kernels: 128, or 32 on lattices below 65,536 cells,
// where 128-thread blocks leave a few blocks per SM and the step waits for the SMs that
// hold one block more than the others (the FP64 kernels are bound by each SM's FP64 pipe).
static inline int step_block(const Geo& g) { return g.ncell < 65536 ? 32 : 128; }

void exact_fused_step(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, bool first, const double* fprev,
                      const double* gprev, double* fnext, double* gnext, cudaStream_t s, int part) {
    const int bs = step_block(g);
    const unsigned nb = nblocks(g.ncell, bs);
    const bool fl = part != 1, th = part != 0;
    if (dim == 2) {
        if (first) {
            if (fl) k_flow<2, true><<<nb, bs, 0, s>>>(g, P, A, fprev, gprev, fnext);
            if (th) k_thermal<2, true><<<nb, bs, 0, s>>>(g, P, A, fnext, gprev, gnext);
        } else {
            if (fl) k_flow<2, false><<<nb, bs, 0, s>>>(g, P, A, fprev, gprev, fnext);
            if (th) k_thermal<2, false><<<nb, bs, 0, s>>>(g, P, A, fnext, gprev, gnext);
        }
    } else {
        if (first) {
            if (fl) k_flow<3, true><<<nb, bs, 0, s>>>(g, P, A, fprev, gprev, fnext);
            if (th) k_thermal<3, true><<<nb, bs, 0, s>>>(g, P, A, fnext, gprev, gnext);
        } else {
            if (fl) k_flow<3, false><<<nb, bs, 0, s>>>(g, P, A, fprev, gprev, fnext);
            if (th) k_thermal<3, false><<<nb, bs, 0, s>>>(g, P, A, fnext, gprev, gnext);
        }
    }
}

static AAFace<double> aa_faces(void* const face[3]) {
    return AAFace<double>{(const double*)face[0], (const double*)face[1], (const double*)face[2]};
}

static bool any_face(void* const face[3]) { return face[0] || face[1] || face[2]; }

template <int D, bool FIRST>
static void aa_step_d(const Geo& g, const PhysC& P, const ExactArrays& A, AAState& S, cudaStream_t s, int part) {
    const int bs = step_block(g);
    const unsigned nb = nblocks(g.ncell, bs);
    const int raw = S.graw ? 1 : 0;
    if (part != 1) {
        if (S.fpar && any_face(S.face_f)) aa_snapshot(g, D == 3 ? 19 : 9, false, LBM_FP64, A.f, S.face_f, s);
        const AAFace<double> wf = aa_faces(S.face_f);
        if (S.fpar) k_aa_flow<D, true, FIRST><<<nb, bs, 0, s>>>(g, P, A, A.f, A.g, wf, S.gpar, raw);
        else k_aa_flow<D, false, FIRST><<<nb, bs, 0, s>>>(g, P, A, A.f, A.g, wf, S.gpar, raw);
        S.fpar ^= 1;
    }
    if (part != 0) {
        if (S.gpar && any_face(S.face_g)) aa_snapshot(g, D == 3 ? 7 : 5, true, LBM_FP64, A.g, S.face_g, s);
        const AAFace<double> wg = aa_faces(S.face_g);
        if (S.gpar) k_aa_thermal<D, true, FIRST><<<nb, bs, 0, s>>>(g, P, A, A.f, A.g, wg, S.fpar, raw);
        else k_aa_thermal<D, false, FIRST><<<nb, bs, 0, s>>>(g, P, A, A.f, A.g, wg, S.fpar, raw);
        if (S.gpar) S.graw = true;
        S.gpar ^= 1;
    }
}

void exact_aa_step(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, bool first, AAState& S,
                   cudaStream_t s, int part) {
    if (dim == 2) {
        if (first) aa_step_d<2, true>(g, P, A, S, s, part);
        else aa_step_d<2, false>(g, P, A, S, s, part);
    } else {
        if (first) aa_step_d<3, true>(g, P, A, S, s, part);
        else aa_step_d<3, false>(g, P, A, S, s, part);
    }
}

void exact_aa_materialize(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, const AAState& S,
                          cudaStream_t s) {
    const unsigned nb = nblocks(g.ncell, 128);
    const int raw = S.graw ? 1 : 0;
    if (dim == 2) k_aa_materialize<2><<<nb, 128, 0, s>>>(g, P, A, A.f, A.g, S.fpar, S.gpar, raw);
    else k_aa_materialize<3><<<nb, 128, 0, s>>>(g, P, A, A.f, A.g, S.fpar, S.gpar, raw);
}

void exact_reconstruct(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, unsigned int* bad,
                       cudaStream_t s) {
    const unsigned nb = nblocks(g.ncell, 128);
    if (dim == 2) k_reconstruct<2><<<nb, 128, 0, s>>>(g, P, A, bad);
    else k_reconstruct<3><<<nb, 128, 0, s>>>(g, P, A, bad);
}

void exact_materialize(const Geo& g, const PhysC& P, const ExactArrays& A, int dim, const double* fcur,
                       const double* gcur, cudaStream_t s) {
    const unsigned nb = nblocks(g.ncell, 128);
    if (dim == 2) k_materialize<2><<<nb, 128, 0, s>>>(g, P, A, fcur, gcur);
    else k_materialize<3><<<nb, 128, 0, s>>>(g, P, A, fcur, gcur);
}

}  // namespace lbm

// ------------------------------------------------------------------------------------
// self-test of divc against CUDA's IEEE double division
// ------------------------------------------------------------------------------------
namespace lbm {

__constant__ double kDivisors[19] = {3.0, 6.0, 7.0, 9.0, 10.0, 12.0, 18.0, 19.0, 21.0, 24.0,
                                     36.0, 40.0, 42.0, 63.0, 72.0, 252.0, 399.0, 1197.0, 2394.0};

__global__ void k_selftest_divc(long long n, uint64_t seed, unsigned long long* mismatches) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    // random sign, normal exponent in [2^-923, 2^900], random 52-bit significand; every
    // 8th sample is an exact multiple c*k so that exact quotients are covered too
    uint64_t z = (seed ^ (uint64_t)i) + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    const uint64_t expo = 100 + (z >> 52) % 1824;
    const uint64_t bits = (z & 0x8000000000000000ULL) | (expo << 52) | (z & 0x000FFFFFFFFFFFFFULL);
    double x = __longlong_as_double((long long)bits);
    unsigned long long bad = 0;
#pragma unroll 1
    for (int d = 0; d < 19; ++d) {
        const double c = kDivisors[d];
        double xx = x;
        if ((i & 7) == 0) xx = c * (double)(long long)((z >> 11) & 0xFFFFFFFFFFULL);
        const double q_ieee = xx / c;
        const double rc = 1.0 / c;
        const double q = __dmul_rn(xx, rc);
        const double r = __fma_rn(-q, c, xx);
        const double q_fast = __fma_rn(r, rc, q);
        if (q_fast != q_ieee) bad += 1;
    }
    if (bad) atomicAdd(mismatches, bad);
}

}  // namespace lbm

// ------------------------------------------------------------------------------------
// self-test of the integer-pipe scalings and the shared divisions against the FP64 pipe
// ------------------------------------------------------------------------------------
namespace lbm {

__device__ __forceinline__ uint64_t st_mix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

__device__ __forceinline__ bool same_bits(double a, double b) {
    return (a != a && b != b) || __double_as_longlong(a) == __double_as_longlong(b);
}

// Sample i: a random bit pattern, paired with (by i mod 4) a random pattern, one within 32
// binades, one sharing leading significand bits, or two values near the bottom of the normal
// range (subnormal results of the scalings).
__global__ void k_selftest_int(long long n, uint64_t seed, unsigned long long* mismatches) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t a = st_mix(seed ^ (2 * (uint64_t)i)), b = st_mix(seed ^ (2 * (uint64_t)i + 1));
    const int mode = (int)(i & 3);
    if (mode >= 1) {
        const long long ea = (long long)((a >> 52) & 0x7FF);
        long long eb = ea + (long long)((b >> 58) & 63) - 32;
        eb = eb < 0 ? 0 : (eb > 2046 ? 2046 : eb);
        b = (b & ~(0x7FFULL << 52)) | ((uint64_t)eb << 52);
    }
    if (mode == 2) {
        const uint64_t keep = st_mix(a) % 53;
        b = (b & ~i64f::kMant) | ((a & i64f::kMant) ^ (st_mix(b) & ((1ULL << keep) - 1)));
    }
    if (mode == 3) {
        a = (a & ~(0x7F0ULL << 52)) | (0x010ULL << 52);
        b = (b & ~(0x7F0ULL << 52)) | (0x010ULL << 52);
    }
    const double x = __longlong_as_double((long long)a), y = __longlong_as_double((long long)b);
    unsigned long long bad = 0;
    bad += !same_bits(iscale<1>(x), __dmul_rn(x, 2.0));
    bad += !same_bits(iscale<2>(y), __dmul_rn(y, 4.0));
    bad += !same_bits(iscale<3>(x), __dmul_rn(x, 8.0));
    bad += !same_bits(iscale<-1>(y), __dmul_rn(y, 0.5));
    bad += !same_bits(iscale<-2>(x), __dmul_rn(x, 0.25));
    bad += !same_bits(iscale<-3>(y), __dmul_rn(y, 0.125));
    // a quotient by c 2^k as the quotient by c scaled (normal quotients): the divisor pairs
    // of the collisions' inverse transforms
    const unsigned ex = (unsigned)((a >> 52) & 0x7FF);
    if (ex >= 64 && ex <= 1984) {
        bad += !same_bits(iscale<-2>(__ddiv_rn(x, 10.0)), __ddiv_rn(x, 40.0));
        bad += !same_bits(iscale<-1>(__ddiv_rn(x, 18.0)), __ddiv_rn(x, 36.0));
        bad += !same_bits(iscale<-2>(__ddiv_rn(x, 18.0)), __ddiv_rn(x, 72.0));
        bad += !same_bits(iscale<-1>(__ddiv_rn(x, 12.0)), __ddiv_rn(x, 24.0));
        bad += !same_bits(iscale<-2>(__ddiv_rn(x, 63.0)), __ddiv_rn(x, 252.0));
        bad += !same_bits(iscale<-1>(__ddiv_rn(x, 6.0)), __ddiv_rn(x, 12.0));
        bad += !same_bits(iscale<-1>(__ddiv_rn(x, 9.0)), __ddiv_rn(x, 18.0));
        bad += !same_bits(iscale<-2>(__ddiv_rn(x, 9.0)), __ddiv_rn(x, 36.0));
    }
    // quotients through a shared correctly rounded reciprocal (div_rcp) against IEEE
    // division: divisors across the whole normal range and near 1 (densities), numerators
    // within 40 binades of them
    {
        const uint64_t bb = st_mix(a ^ 0x5555ULL);
        const uint64_t ebits = (i & 1) ? (1021ULL + ((bb >> 60) & 3)) : (64 + (bb >> 52) % 1900);
        const double den = __longlong_as_double((long long)((ebits << 52) | (bb & i64f::kMant)));  // positive
        const uint64_t en = ebits + ((b >> 56) % 80) - 40;
        const double num = __longlong_as_double((long long)((b & i64f::kSign) | (en << 52) | (a & i64f::kMant)));
        const double yr = __drcp_rn(den);
        bad += !same_bits(div_rcp(num, den, yr), __ddiv_rn(num, den));
        bad += !same_bits(div_rcp(-0.0, den, yr), __ddiv_rn(-0.0, den));
    }
    if (bad) atomicAdd(mismatches, bad);
}

}  // namespace lbm

extern "C" int lbm_selftest_int_arith(int64_t n, uint64_t seed, int64_t* mismatches) {
    if (n <= 0 || !mismatches) return LBM_ERR_PARAM;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return LBM_ERR_OOM;
    cudaMemset(d, 0, sizeof(*d));
    lbm::k_selftest_int<<<(unsigned)((n + 255) / 256), 256>>>((long long)n, seed, d);
    unsigned long long h = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return LBM_ERR_CUDA;
    *mismatches = (int64_t)h;
    return LBM_OK;
}

extern "C" int lbm_selftest_const_division(int64_t n, uint64_t seed, int64_t* mismatches) {
    if (n <= 0 || !mismatches) return LBM_ERR_PARAM;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return LBM_ERR_OOM;
    cudaMemset(d, 0, sizeof(*d));
    lbm::k_selftest_divc<<<(unsigned)((n + 255) / 256), 256>>>((long long)n, seed, d);
    unsigned long long h = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return LBM_ERR_CUDA;
    *mismatches = (int64_t)h;
    return LBM_OK;
}
