// Host build of the plain method's per-cell FP64 arithmetic (csrc/lbm_exact_cell.cuh) for
// test_cpu_exact_cell.py: the collision, macro and thermal-collision functions of the GPU
// kernels, compiled for the CPU without floating-point contraction, applied to every cell of
// arrays in the reference's Fortran layout (population a of cell c at a + q*c).  The rounding
// intrinsics of the device code map to the CPU's IEEE operations: __dmul_rn to *, __fma_rn
// to std::fma, __drcp_rn to 1.0/x (each correctly rounded).
#include <cuda_runtime.h>

#include <cmath>

inline double __dmul_rn(double a, double b) { return a * b; }
inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
inline double __drcp_rn(double x) { return 1.0 / x; }

#include "lbm_exact_cell.cuh"

using namespace lbm;

// collision: f_post of every cell from f, rho, u, v[, w], T.  known != 0: the conserved
// moments come from the macro sums of the same f (the fused flow kernel's form).
extern "C" int cell_collide(int dim, const lbm_params* p, const lbm_constants* c, long long n, const double* f,
                            const double* rho, const double* u, const double* v, const double* w, const double* T,
                            int known, double* fp, double* Fx, double* Fy) {
    const PhysC P = make_physc(*p, *c);
    for (long long x = 0; x < n; ++x) {
        if (dim == 2) {
            double F[9], FP[9], fx, fy, r, uu, vv, jx, jy;
            for (int a = 0; a < 9; ++a) F[a] = f[a + 9 * x];
            if (known) {
                macro_2d(F, 0.0, 0.0, r, uu, vv, jx, jy);
                collide_2d<true>(F, rho[x], u[x], v[x], T[x], P, FP, fx, fy, jx, jy);
            } else {
                collide_2d<false>(F, rho[x], u[x], v[x], T[x], P, FP, fx, fy);
            }
            for (int a = 0; a < 9; ++a) fp[a + 9 * x] = FP[a];
            Fx[x] = fx;
            Fy[x] = fy;
        } else {
            double F[19], FP[19], r, uu, vv, ww, jx, jy, jz;
            for (int a = 0; a < 19; ++a) F[a] = f[a + 19 * x];
            if (known) {
                macro_3d(F, 0.0, P, r, uu, vv, ww, jx, jy, jz);
                collide_3d<true>(F, rho[x], u[x], v[x], w[x], T[x], P, FP, jx, jy, jz);
            } else {
                collide_3d<false>(F, rho[x], u[x], v[x], w[x], T[x], P, FP);
            }
            for (int a = 0; a < 19; ++a) fp[a + 19 * x] = FP[a];
        }
    }
    return 0;
}

// macro: rho, u, v[, w] of every cell from the streamed f and the lag (2D: the stored force
// Fx, Fy; 3D: T, from which the macro step recomputes F_y).
extern "C" int cell_macro(int dim, const lbm_params* p, const lbm_constants* c, long long n, const double* f,
                          const double* lag0, const double* lag1, double* rho, double* u, double* v, double* w) {
    const PhysC P = make_physc(*p, *c);
    for (long long x = 0; x < n; ++x) {
        if (dim == 2) {
            double F[9];
            for (int a = 0; a < 9; ++a) F[a] = f[a + 9 * x];
            macro_2d(F, lag0[x], lag1[x], rho[x], u[x], v[x]);
        } else {
            double F[19];
            for (int a = 0; a < 19; ++a) F[a] = f[a + 19 * x];
            macro_3d(F, lag0[x], P, rho[x], u[x], v[x], w[x]);
        }
    }
    return 0;
}

// collisionT: g_post and the new B of every cell.  known != 0: n0 is passed in as T, which
// the caller sets to the sum of the same g (the fused thermal kernel's form).
extern "C" int cell_collideT(int dim, const lbm_params* p, const lbm_constants* c, long long n, const double* g,
                             const double* u, const double* v, const double* w, const double* T, const double* Bx,
                             const double* By, const double* Bz, int known, double* gp, double* BxOut, double* ByOut,
                             double* BzOut) {
    const PhysC P = make_physc(*p, *c);
    for (long long x = 0; x < n; ++x) {
        if (dim == 2) {
            double G[5], GP[5];
            for (int a = 0; a < 5; ++a) G[a] = g[a + 5 * x];
            if (known) collideT_2d<true>(G, u[x], v[x], sumT<5>(G), Bx[x], By[x], P, GP, BxOut[x], ByOut[x]);
            else collideT_2d<false>(G, u[x], v[x], T[x], Bx[x], By[x], P, GP, BxOut[x], ByOut[x]);
            for (int a = 0; a < 5; ++a) gp[a + 5 * x] = GP[a];
        } else {
            double G[7], GP[7];
            for (int a = 0; a < 7; ++a) G[a] = g[a + 7 * x];
            if (known)
                collideT_3d<true>(G, u[x], v[x], w[x], sumT<7>(G), Bx[x], By[x], Bz[x], P, GP, BxOut[x], ByOut[x],
                                  BzOut[x]);
            else
                collideT_3d<false>(G, u[x], v[x], w[x], T[x], Bx[x], By[x], Bz[x], P, GP, BxOut[x], ByOut[x],
                                   BzOut[x]);
            for (int a = 0; a < 7; ++a) gp[a + 7 * x] = GP[a];
        }
    }
    return 0;
}
