// lbm_exact_cell.cuh - per-cell arithmetic of the plain method (FP64): the reference's
// collision, thermal collision and macro steps for one cell, shared by the stage kernels and
// the fused kernels of lbm_exact.cu.
//
// The functions are host-compilable (the device qualifiers and the rounding intrinsics
// __dmul_rn, __fma_rn, __drcp_rn map to the host's IEEE operations, with floating-point
// contraction off), so the CPU tests compare them cell by cell with the oracle's stages.
#pragma once

#include "lbm_fp64_int.cuh"
#include "lbm_internal.h"

namespace lbm {

// Products with exact powers of two (x*2, x/4, -0.5*x, ...) are exponent adds on the
// integer pipes (i64f::iscale), the same bits as the FP64 multiply, which on GB300 is the
// step's bottleneck; IEEE multiplication is sign-symmetric, so -(2^k x) = (-2^k) x.
using i64f::iscale;

// ------------------------------------------------------------------------------------
// Per-cell arithmetic in the reference's expression order.  Every rounded operation of the
// reference happens once, on the same operands; only operations that give the same bits by
// another route take it (exact power-of-two products on the integer pipes, rate-only
// factors rounded on the host, shared divisions and reciprocals, macro sums handed between
// the kernels).
// ------------------------------------------------------------------------------------

// Division by one of the reference's integer constants c (all below 2^12), as the
// reference writes it (x / c), rounded exactly like IEEE division but in 3 FP64
// operations: q = x*rc with rc = RN(1/c), the exact remainder r = x - q*c (one fma),
// then RN(q + r*rc) (Markstein's correction).  For an integer divisor c < 2^12 the exact
// quotient is never closer than ulp/(2c) to a rounding midpoint, while the corrected
// value differs from it by less than 1.5 ulp * 2^-53, so the result is the correctly
// rounded quotient for every normal x (checked against CUDA's division by
// lbm_selftest_const_division).
__device__ __forceinline__ double divc(double x, double c) {
    const double rc = 1.0 / c;  // folded at compile time
    const double q = __dmul_rn(x, rc);
    const double r = __fma_rn(-q, c, x);
    return __fma_rn(r, rc, q);
}

// x / b from y = RN(1/b) (CUDA's correctly rounded reciprocal) by Markstein's correction:
// q = RN(x y), r = x - b q in one fma, RN(q + r y) is the correctly rounded x / b for every
// normal quotient (Markstein 1990; checked exhaustively for 5- to 11-bit significands with
// the remainder rounded as the fma rounds it, and against CUDA's division by
// lbm_selftest_int_arith).  A zero numerator keeps q = RN(x y), which has the IEEE sign.
// Several quotients by one b share the reciprocal: 3 FP64 operations each instead of a
// full division.
__device__ __forceinline__ double div_rcp(double x, double b, double y) {
    const double q = __dmul_rn(x, y);
    const double r = __fma_rn(-q, b, x);
    const double qc = __fma_rn(r, y, q);
    return (i64f::bits(x) & i64f::kAbs) == 0 ? q : qc;
}

// collision (2DRB.F90:688-759).  Writes f_post and the stored body force (Fx, Fy).
// KNOWN: rho, jx, jy are the macro step's sums of these populations (m0, m3, m5 in the
// same order), passed in instead of summed again.
template <bool KNOWN = false>
__device__ __forceinline__ void collide_2d(const double* F, double rho, double u, double v, double T,
                                           const PhysC& P, double* FP, double& FxOut, double& FyOut,
                                           double jx = 0.0, double jy = 0.0) {
    double m[9], meq[9], s[9], fSource[9], m_post[9];
    m[0] = KNOWN ? rho : F[0] + F[1] + F[2] + F[3] + F[4] + F[5] + F[6] + F[7] + F[8];
    m[1] = -iscale<2>(F[0]) - F[1] - F[2] - F[3] - F[4] + iscale<1>(F[5] + F[6] + F[7] + F[8]);
    m[2] = iscale<2>(F[0]) - iscale<1>(F[1] + F[2] + F[3] + F[4]) + F[5] + F[6] + F[7] + F[8];
    m[3] = KNOWN ? jx : F[1] - F[3] + F[5] - F[6] - F[7] + F[8];
    m[4] = -iscale<1>(F[1]) + iscale<1>(F[3]) + F[5] - F[6] - F[7] + F[8];
    m[5] = KNOWN ? jy : F[2] - F[4] + F[5] + F[6] - F[7] - F[8];
    m[6] = -iscale<1>(F[2]) + iscale<1>(F[4]) + F[5] + F[6] - F[7] - F[8];
    m[7] = F[1] - F[2] + F[3] - F[4];
    m[8] = F[5] - F[6] + F[7] - F[8];

    meq[0] = rho;
    meq[1] = rho * (-2.0 + 3.0 * (u * u + v * v));
    meq[2] = rho * (1.0 - 3.0 * (u * u + v * v));
    meq[3] = rho * u;
    meq[4] = -(rho * u);
    meq[5] = rho * v;
    meq[6] = -(rho * v);
    meq[7] = rho * (u * u - v * v);
    meq[8] = rho * (u * v);

    s[0] = 0.0; s[1] = P.Snu; s[2] = P.Snu; s[3] = 0.0; s[4] = P.Sq;
    s[5] = 0.0; s[6] = P.Sq;  s[7] = P.Snu; s[8] = P.Snu;

    double Fx = 0.0;
    double Fy = rho * P.gBeta * (T - P.Tref);
    if (P.ha) {  // SideHeatedHa (2DRB.F90:722-726): buoyancy plus the magnetic force
        Fx = 0.0 + P.B2 * (v * P.sinphi * P.cosphi - u * P.sinphi * P.sinphi);
        Fy = rho * P.gBeta * (T - P.Tref) + rho * P.B2 * (u * P.sinphi * P.cosphi - v * P.cosphi * P.cosphi);
    }
    FxOut = Fx;
    FyOut = Fy;

    // (6 - 3 s1) = (6 - 3 s2) = h6Snu, (1 - s/2) = 1 for s3, s5 = 0, hSq for s4, s6,
    // (2 - s7) = h2Snu, (1 - s8/2) = hSnu: the rates' factors rounded once on the host
    fSource[0] = 0.0;
    fSource[1] = P.h6Snu * (u * Fx + v * Fy);
    fSource[2] = -(P.h6Snu * (u * Fx + v * Fy));
    fSource[3] = Fx;
    fSource[4] = -(P.hSq * Fx);
    fSource[5] = Fy;
    fSource[6] = -(P.hSq * Fy);
    fSource[7] = P.h2Snu * (u * Fx - v * Fy);
    fSource[8] = P.hSnu * (u * Fy + v * Fx);

    // conserved moments (zero rates s0, s3, s5): m - 0*(m - meq) + source is m + source for
    // every finite m but -0 (a zero rate only subtracts a zero; m0 = rho, and a sum of
    // populations is never -0), as in collide_3d; fSource[0] = 0
    m_post[0] = m[0];
    m_post[3] = m[3] + fSource[3];
    m_post[5] = m[5] + fSource[5];
    m_post[1] = m[1] - s[1] * (m[1] - meq[1]) + fSource[1];
    m_post[2] = m[2] - s[2] * (m[2] - meq[2]) + fSource[2];
    m_post[4] = m[4] - s[4] * (m[4] - meq[4]) + fSource[4];
    m_post[6] = m[6] - s[6] * (m[6] - meq[6]) + fSource[6];
    m_post[7] = m[7] - s[7] * (m[7] - meq[7]) + fSource[7];
    m_post[8] = m[8] - s[8] * (m[8] - meq[8]) + fSource[8];

    // m/4 as exponent adds; x/(c 2^k) = RN(x/c) 2^-k, one exact multiply, for a normal quotient
    const double q7 = iscale<-2>(m_post[7]), q8 = iscale<-2>(m_post[8]);
    const double e1 = divc(m_post[1], 9.0), e2 = divc(m_post[2], 9.0), e4 = divc(m_post[4], 6.0),
                 e6 = divc(m_post[6], 6.0);
    FP[0] = divc(m_post[0], 9.0) - e1 + e2;
    FP[1] = divc(m_post[0], 9.0) - __dmul_rn(e1, 0.25) - __dmul_rn(e2, 0.5) + divc(m_post[3], 6.0) - e4 + q7;
    FP[2] = divc(m_post[0], 9.0) - __dmul_rn(e1, 0.25) - __dmul_rn(e2, 0.5) + divc(m_post[5], 6.0) - e6 - q7;
    FP[3] = divc(m_post[0], 9.0) - __dmul_rn(e1, 0.25) - __dmul_rn(e2, 0.5) - divc(m_post[3], 6.0) + e4 + q7;
    FP[4] = divc(m_post[0], 9.0) - __dmul_rn(e1, 0.25) - __dmul_rn(e2, 0.5) - divc(m_post[5], 6.0) + e6 - q7;
    FP[5] = divc(m_post[0], 9.0) + __dmul_rn(e1, 0.5) + __dmul_rn(e2, 0.25) + divc(m_post[3], 6.0) + __dmul_rn(e4, 0.5)
            + divc(m_post[5], 6.0) + __dmul_rn(e6, 0.5) + q8;
    FP[6] = divc(m_post[0], 9.0) + __dmul_rn(e1, 0.5) + __dmul_rn(e2, 0.25) - divc(m_post[3], 6.0) - __dmul_rn(e4, 0.5)
            + divc(m_post[5], 6.0) + __dmul_rn(e6, 0.5) - q8;
    FP[7] = divc(m_post[0], 9.0) + __dmul_rn(e1, 0.5) + __dmul_rn(e2, 0.25) - divc(m_post[3], 6.0) - __dmul_rn(e4, 0.5)
            - divc(m_post[5], 6.0) - __dmul_rn(e6, 0.5) + q8;
    FP[8] = divc(m_post[0], 9.0) + __dmul_rn(e1, 0.5) + __dmul_rn(e2, 0.25) + divc(m_post[3], 6.0) + __dmul_rn(e4, 0.5)
            - divc(m_post[5], 6.0) - __dmul_rn(e6, 0.5) - q8;
}

// collision (3DRB.F90:704-943).  KNOWN: rhoLoc, jx, jy, jz are the macro step's sums of
// these populations (m0, m3, m5, m7 in the same order), passed in instead of summed again.
template <bool KNOWN = false>
__device__ __forceinline__ void collide_3d(const double* f, double rhoLoc, double uLoc, double vLoc, double wLoc,
                                           double Tc, const PhysC& P, double* fp, double jx = 0.0, double jy = 0.0,
                                           double jz = 0.0) {
    double m[19], meq[19], s[19], fSource[19], mp[19];
    const double u2 = uLoc * uLoc + vLoc * vLoc + wLoc * wLoc;
    m[0] = KNOWN ? rhoLoc
                 : f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13]
                       + f[14] + f[15] + f[16] + f[17] + f[18];
    m[1] = -30.0 * f[0] - 11.0 * (f[1] + f[2] + f[3] + f[4] + f[5] + f[6])
           + iscale<3>(f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18]);
    m[2] = 12.0 * f[0] - iscale<2>(f[1] + f[2] + f[3] + f[4] + f[5] + f[6])
           + (f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14] + f[15] + f[16] + f[17] + f[18]);
    m[3] = KNOWN ? jx : f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    m[4] = -iscale<2>(f[1]) + iscale<2>(f[2]) + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    m[5] = KNOWN ? jy : f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    m[6] = -iscale<2>(f[3]) + iscale<2>(f[4]) + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    m[7] = KNOWN ? jz : f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    m[8] = -iscale<2>(f[5]) + iscale<2>(f[6]) + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    m[9] = iscale<1>(f[1] + f[2]) - (f[3] + f[4] + f[5] + f[6]) + (f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14])
           - iscale<1>(f[15] + f[16] + f[17] + f[18]);
    m[10] = -iscale<2>(f[1] + f[2]) + iscale<1>(f[3] + f[4] + f[5] + f[6])
            + (f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14]) - iscale<1>(f[15] + f[16] + f[17] + f[18]);
    m[11] = (f[3] + f[4]) - (f[5] + f[6]) + (f[7] + f[8] + f[9] + f[10]) - (f[11] + f[12] + f[13] + f[14]);
    m[12] = -iscale<1>(f[3] + f[4]) + iscale<1>(f[5] + f[6]) + (f[7] + f[8] + f[9] + f[10]) - (f[11] + f[12] + f[13] + f[14]);
    m[13] = f[7] - f[8] - f[9] + f[10];
    m[14] = f[15] - f[16] - f[17] + f[18];
    m[15] = f[11] - f[12] - f[13] + f[14];
    m[16] = f[7] - f[8] + f[9] - f[10] - f[11] + f[12] - f[13] + f[14];
    m[17] = -f[7] - f[8] + f[9] + f[10] + f[15] - f[16] + f[17] - f[18];
    m[18] = f[11] + f[12] - f[13] - f[14] - f[15] - f[16] + f[17] + f[18];

    const double m2rho = -iscale<1>(rhoLoc);  // -2.0 * rhoLoc
    meq[0] = rhoLoc;
    meq[1] = rhoLoc * (-11.0 + 19.0 * u2);
    meq[2] = rhoLoc * (3.0 - iscale<-1>(11.0 * u2));
    meq[3] = rhoLoc * uLoc;
    meq[4] = divc(m2rho * uLoc, 3.0);
    meq[5] = rhoLoc * vLoc;
    meq[6] = divc(m2rho * vLoc, 3.0);
    meq[7] = rhoLoc * wLoc;
    meq[8] = divc(m2rho * wLoc, 3.0);
    meq[9] = rhoLoc * (iscale<1>(uLoc) * uLoc - vLoc * vLoc - wLoc * wLoc);
    meq[10] = -iscale<-1>(meq[9]);
    meq[11] = rhoLoc * (vLoc * vLoc - wLoc * wLoc);
    meq[12] = -iscale<-1>(meq[11]);
    meq[13] = rhoLoc * uLoc * vLoc;
    meq[14] = rhoLoc * vLoc * wLoc;
    meq[15] = rhoLoc * uLoc * wLoc;
    meq[16] = 0.0;
    meq[17] = 0.0;
    meq[18] = 0.0;

    s[0] = 0.0;    s[1] = P.Se;   s[2] = P.Seps; s[3] = 0.0;    s[4] = P.Sq;
    s[5] = 0.0;    s[6] = P.Sq;   s[7] = 0.0;    s[8] = P.Sq;   s[9] = P.Snu;
    s[10] = P.Spi; s[11] = P.Snu; s[12] = P.Spi; s[13] = P.Snu; s[14] = P.Snu;
    s[15] = P.Snu; s[16] = P.Sm;  s[17] = P.Sm;  s[18] = P.Sm;

    // Guo source (3DRB.F90:826-849) with the body force F = (0, F_y, 0).  Terms that the
    // reference multiplies by F_x = F_z = 0 or by a zero rate are left out: they only add
    // or subtract a zero, so every value is unchanged (at most the sign of a zero result
    // differs, and no result is ever divided by it).
    const double FyLoc = rhoLoc * P.gBeta * (Tc - P.Tref);
    const double uDotF = vLoc * FyLoc;

    // (1 - s/2) factors: s1 = Se, s2 = Seps, s6 = Sq, s9 = s11 = s13 = s14 = Snu, s10 = s12 = Spi,
    // with the constant multiplied in first as the reference's left-to-right order does
    const double vF2 = iscale<1>(vLoc) * FyLoc;  // 2.0 * vLoc * FyLoc
    fSource[1] = P.hSe38 * uDotF;
    fSource[2] = P.hSeps11 * uDotF;
    fSource[6] = P.hSq23 * FyLoc;
    fSource[9] = P.hSnu * (-vF2);
    fSource[10] = P.hSpi * (vLoc * FyLoc);
    fSource[11] = P.hSnu * vF2;
    fSource[12] = P.hSpi * (-(vLoc * FyLoc));
    fSource[13] = P.hSnu * (uLoc * FyLoc);
    fSource[14] = P.hSnu * (wLoc * FyLoc);

    // m_post = m - S(m - meq) + source; conserved moments (s = 0) keep m plus the force.
    mp[0] = m[0];
    mp[3] = m[3];
    mp[5] = m[5] + FyLoc;
    mp[7] = m[7];
    mp[1] = m[1] - s[1] * (m[1] - meq[1]) + fSource[1];
    mp[2] = m[2] - s[2] * (m[2] - meq[2]) + fSource[2];
    mp[4] = m[4] - s[4] * (m[4] - meq[4]);
    mp[6] = m[6] - s[6] * (m[6] - meq[6]) + fSource[6];
    mp[8] = m[8] - s[8] * (m[8] - meq[8]);
#pragma unroll
    for (int a = 9; a <= 14; ++a) mp[a] = m[a] - s[a] * (m[a] - meq[a]) + fSource[a];
    mp[15] = m[15] - s[15] * (m[15] - meq[15]);
#pragma unroll
    for (int a = 16; a <= 18; ++a) mp[a] = m[a] - s[a] * m[a];

    // m/4 and m/8 as exponent adds.  A moment divided by c and by c 2^k shares the division:
    // RN(x / (c 2^k)) = RN(x / c) 2^-k whenever the quotient is normal (as divc itself
    // assumes), so the second quotient is one exact FP64 multiply instead of three
    // operations.  (An exponent add there measured slower: its rare-case branch sits
    // between two FP64 operations of every reconstruction sum.)
    const double d2 = divc(mp[2], 63.0), d4 = divc(mp[4], 10.0), d6 = divc(mp[6], 10.0), d8 = divc(mp[8], 10.0);
    const double d9 = divc(mp[9], 18.0), d10 = divc(mp[10], 18.0), d12 = divc(mp[12], 12.0);
    const double d1b = divc(iscale<2>(mp[1]), 1197.0);  // (4 mp1) / 1197
    const double q13 = iscale<-2>(mp[13]), q14 = iscale<-2>(mp[14]), q15 = iscale<-2>(mp[15]);
    const double q16 = iscale<-3>(mp[16]), q17 = iscale<-3>(mp[17]), q18 = iscale<-3>(mp[18]);
    fp[0] = divc(mp[0], 19.0) - divc(5.0 * mp[1], 399.0) + divc(mp[2], 21.0);
    fp[1] = divc(mp[0], 19.0) - divc(11.0 * mp[1], 2394.0) - d2 + divc(mp[3], 10.0) - d4 + d9 - d10;
    fp[2] = divc(mp[0], 19.0) - divc(11.0 * mp[1], 2394.0) - d2 - divc(mp[3], 10.0) + d4 + d9 - d10;
    fp[3] = divc(mp[0], 19.0) - divc(11.0 * mp[1], 2394.0) - d2 + divc(mp[5], 10.0) - d6 - __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.5)
            + divc(mp[11], 12.0) - d12;
    fp[4] = divc(mp[0], 19.0) - divc(11.0 * mp[1], 2394.0) - d2 - divc(mp[5], 10.0) + d6 - __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.5)
            + divc(mp[11], 12.0) - d12;
    fp[5] = divc(mp[0], 19.0) - divc(11.0 * mp[1], 2394.0) - d2 + divc(mp[7], 10.0) - d8 - __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.5)
            - divc(mp[11], 12.0) + d12;
    fp[6] = divc(mp[0], 19.0) - divc(11.0 * mp[1], 2394.0) - d2 - divc(mp[7], 10.0) + d8 - __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.5)
            - divc(mp[11], 12.0) + d12;
    fp[7] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) + divc(mp[3], 10.0) + __dmul_rn(d4, 0.25) + divc(mp[5], 10.0) + __dmul_rn(d6, 0.25)
            + __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.25) + divc(mp[11], 12.0) + __dmul_rn(d12, 0.5) + q13 + q16 - q17;
    fp[8] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) - divc(mp[3], 10.0) - __dmul_rn(d4, 0.25) + divc(mp[5], 10.0) + __dmul_rn(d6, 0.25)
            + __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.25) + divc(mp[11], 12.0) + __dmul_rn(d12, 0.5) - q13 - q16 - q17;
    fp[9] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) + divc(mp[3], 10.0) + __dmul_rn(d4, 0.25) - divc(mp[5], 10.0) - __dmul_rn(d6, 0.25)
            + __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.25) + divc(mp[11], 12.0) + __dmul_rn(d12, 0.5) - q13 + q16 + q17;
    fp[10] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) - divc(mp[3], 10.0) - __dmul_rn(d4, 0.25) - divc(mp[5], 10.0) - __dmul_rn(d6, 0.25)
             + __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.25) + divc(mp[11], 12.0) + __dmul_rn(d12, 0.5) + q13 - q16 + q17;
    fp[11] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) + divc(mp[3], 10.0) + __dmul_rn(d4, 0.25) + divc(mp[7], 10.0) + __dmul_rn(d8, 0.25)
             + __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.25) - divc(mp[11], 12.0) - __dmul_rn(d12, 0.5) + q15 - q16 + q18;
    fp[12] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) - divc(mp[3], 10.0) - __dmul_rn(d4, 0.25) + divc(mp[7], 10.0) + __dmul_rn(d8, 0.25)
             + __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.25) - divc(mp[11], 12.0) - __dmul_rn(d12, 0.5) - q15 + q16 + q18;
    fp[13] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) + divc(mp[3], 10.0) + __dmul_rn(d4, 0.25) - divc(mp[7], 10.0) - __dmul_rn(d8, 0.25)
             + __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.25) - divc(mp[11], 12.0) - __dmul_rn(d12, 0.5) - q15 - q16 - q18;
    fp[14] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) - divc(mp[3], 10.0) - __dmul_rn(d4, 0.25) - divc(mp[7], 10.0) - __dmul_rn(d8, 0.25)
             + __dmul_rn(d9, 0.5) + __dmul_rn(d10, 0.25) - divc(mp[11], 12.0) - __dmul_rn(d12, 0.5) + q15 + q16 - q18;
    fp[15] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) + divc(mp[5], 10.0) + __dmul_rn(d6, 0.25) + divc(mp[7], 10.0) + __dmul_rn(d8, 0.25)
             - d9 - __dmul_rn(d10, 0.5) + q14 + q17 - q18;
    fp[16] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) - divc(mp[5], 10.0) - __dmul_rn(d6, 0.25) + divc(mp[7], 10.0) + __dmul_rn(d8, 0.25)
             - d9 - __dmul_rn(d10, 0.5) - q14 - q17 - q18;
    fp[17] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) + divc(mp[5], 10.0) + __dmul_rn(d6, 0.25) - divc(mp[7], 10.0) - __dmul_rn(d8, 0.25)
             - d9 - __dmul_rn(d10, 0.5) - q14 + q17 + q18;
    fp[18] = divc(mp[0], 19.0) + d1b + __dmul_rn(d2, 0.25) - divc(mp[5], 10.0) - __dmul_rn(d6, 0.25) - divc(mp[7], 10.0) - __dmul_rn(d8, 0.25)
             - d9 - __dmul_rn(d10, 0.5) + q14 - q17 + q18;
}

// collisionT (2DRB.F90:921-974).  B = (u T, v T); returns g_post and the new B.  KNOWN: T is
// the sum of these populations in the same order (n0), passed in instead of summed again.
template <bool KNOWN = false>
__device__ __forceinline__ void collideT_2d(const double* G, double u, double v, double T, double Bxp, double Byp,
                                            const PhysC& P, double* GP, double& BxOut, double& ByOut) {
    double n[5], neq[5], q[5], n_post[5];
    const double Bx = u * T;
    const double By = v * T;
    double dBx, dBy;
    if (P.use_g) {
        dBx = Bx - Bxp;
        dBy = By - Byp;
    } else {
        dBx = 0.0;
        dBy = 0.0;
    }
    BxOut = Bx;
    ByOut = By;
    n[0] = KNOWN ? T : G[0] + G[1] + G[2] + G[3] + G[4];
    n[1] = G[1] - G[3];
    n[2] = G[2] - G[4];
    n[3] = -iscale<2>(G[0]) + G[1] + G[2] + G[3] + G[4];
    n[4] = G[1] - G[2] + G[3] - G[4];
    neq[0] = T;
    neq[1] = T * u;
    neq[2] = T * v;
    neq[3] = P.legacy ? T * P.paraA : T * (-2.0 / 3.0);
    neq[4] = 0.0;
    q[0] = 0.0; q[1] = P.Qk; q[2] = P.Qk; q[3] = P.Qnu; q[4] = P.Qnu;
    n_post[0] = n[0];  // zero rate q0: n0 - 0*(n0 - T) is n0 (never -0, a sum of populations)
    n_post[1] = n[1] - q[1] * (n[1] - neq[1]) + P.SG * dBx;
    n_post[2] = n[2] - q[2] * (n[2] - neq[2]) + P.SG * dBy;
    n_post[3] = n[3] - q[3] * (n[3] - neq[3]);
    n_post[4] = n[4] - q[4] * (n[4] - neq[4]);
    const double h1 = iscale<-1>(n_post[1]), h2 = iscale<-1>(n_post[2]), q4 = iscale<-2>(n_post[4]);
    GP[0] = 0.2 * n_post[0] - 0.2 * n_post[3];
    GP[1] = 0.2 * n_post[0] + h1 + 0.05 * n_post[3] + q4;
    GP[2] = 0.2 * n_post[0] + h2 + 0.05 * n_post[3] - q4;
    GP[3] = 0.2 * n_post[0] - h1 + 0.05 * n_post[3] + q4;
    GP[4] = 0.2 * n_post[0] - h2 + 0.05 * n_post[3] - q4;
}

// collisionT (3DRB.F90:1121-1191).  KNOWN as in collideT_2d.
template <bool KNOWN = false>
__device__ __forceinline__ void collideT_3d(const double* g, double u, double v, double w, double T, double Bxp,
                                            double Byp, double Bzp, const PhysC& P, double* gp, double& BxOut,
                                            double& ByOut, double& BzOut) {
    double n[7], neq[7], q[7], n_post[7];
    const double Bx = u * T, By = v * T, Bz = w * T;
    double dBx, dBy, dBz;
    if (P.use_g) {
        dBx = Bx - Bxp;
        dBy = By - Byp;
        dBz = Bz - Bzp;
    } else {
        dBx = 0.0;
        dBy = 0.0;
        dBz = 0.0;
    }
    BxOut = Bx;
    ByOut = By;
    BzOut = Bz;
    n[0] = KNOWN ? T : g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6];
    n[1] = g[1] - g[2];
    n[2] = g[3] - g[4];
    n[3] = g[5] - g[6];
    n[4] = -6.0 * g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6];
    n[5] = iscale<1>(g[1]) + iscale<1>(g[2]) - g[3] - g[4] - g[5] - g[6];
    n[6] = g[3] + g[4] - g[5] - g[6];
    neq[0] = T;
    neq[1] = Bx;
    neq[2] = By;
    neq[3] = Bz;
    neq[4] = P.legacy ? P.paraA * T : -0.75 * T;
    neq[5] = 0.0;
    neq[6] = 0.0;
    q[0] = 0.0; q[1] = P.Qk; q[2] = P.Qk; q[3] = P.Qk; q[4] = P.Qnu; q[5] = P.Qnu; q[6] = P.Qnu;
    n_post[0] = n[0];  // zero rate q0: n0 - 0*(n0 - T) is n0 (never -0, a sum of populations)
    n_post[1] = n[1] - q[1] * (n[1] - neq[1]) + P.SG * dBx;
    n_post[2] = n[2] - q[2] * (n[2] - neq[2]) + P.SG * dBy;
    n_post[3] = n[3] - q[3] * (n[3] - neq[3]) + P.SG * dBz;
    n_post[4] = n[4] - q[4] * (n[4] - neq[4]);
    n_post[5] = n[5] - q[5] * (n[5] - neq[5]);
    n_post[6] = n[6] - q[6] * (n[6] - neq[6]);
    const double h1 = iscale<-1>(n_post[1]), h2 = iscale<-1>(n_post[2]), h3 = iscale<-1>(n_post[3]);
    const double q6 = iscale<-2>(n_post[6]), s5 = divc(n_post[5], 6.0);  // x/12 = RN(x/6) * 0.5
    gp[0] = divc(n_post[0], 7.0) - divc(n_post[4], 7.0);
    gp[1] = divc(n_post[0], 7.0) + h1 + divc(n_post[4], 42.0) + s5;
    gp[2] = divc(n_post[0], 7.0) - h1 + divc(n_post[4], 42.0) + s5;
    gp[3] = divc(n_post[0], 7.0) + h2 + divc(n_post[4], 42.0) - __dmul_rn(s5, 0.5) + q6;
    gp[4] = divc(n_post[0], 7.0) - h2 + divc(n_post[4], 42.0) - __dmul_rn(s5, 0.5) + q6;
    gp[5] = divc(n_post[0], 7.0) + h3 + divc(n_post[4], 42.0) - __dmul_rn(s5, 0.5) - q6;
    gp[6] = divc(n_post[0], 7.0) - h3 + divc(n_post[4], 42.0) - __dmul_rn(s5, 0.5) - q6;
}

// macro (2DRB.F90:884-889): u = (sum e f + Fx/2)/rho with the force stored by collision.
// jx, jy: the momentum sums before the force term (the reference's left-to-right order
// adds it last).
__device__ __forceinline__ void macro_2d(const double* F, double Fx, double Fy, double& rho, double& u, double& v,
                                         double& jx, double& jy) {
    rho = F[0] + F[1] + F[2] + F[3] + F[4] + F[5] + F[6] + F[7] + F[8];
    jx = F[1] - F[3] + F[5] - F[6] - F[7] + F[8];
    jy = F[2] - F[4] + F[5] + F[6] - F[7] - F[8];
    const double y = __drcp_rn(rho);
    u = div_rcp(jx + iscale<-1>(Fx), rho, y);
    v = div_rcp(jy + iscale<-1>(Fy), rho, y);
}

__device__ __forceinline__ void macro_2d(const double* F, double Fx, double Fy, double& rho, double& u, double& v) {
    double jx, jy;
    macro_2d(F, Fx, Fy, rho, u, v, jx, jy);
}

// macro (3DRB.F90:1077-1092): F_y recomputed with the new rho and the lagged T.
__device__ __forceinline__ void macro_3d(const double* f, double Tlag, const PhysC& P, double& rho, double& u,
                                         double& v, double& w, double& jx, double& jy, double& jz) {
    rho = f[0] + f[1] + f[2] + f[3] + f[4] + f[5] + f[6] + f[7] + f[8] + f[9] + f[10] + f[11] + f[12] + f[13] + f[14]
          + f[15] + f[16] + f[17] + f[18];
    const double FyLoc = rho * P.gBeta * (Tlag - P.Tref);
    jx = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    jy = f[3] - f[4] + f[7] + f[8] - f[9] - f[10] + f[15] - f[16] + f[17] - f[18];
    jz = f[5] - f[6] + f[11] + f[12] - f[13] - f[14] + f[15] + f[16] - f[17] - f[18];
    const double y = __drcp_rn(rho);
    u = div_rcp(jx, rho, y);
    v = div_rcp(jy + iscale<-1>(FyLoc), rho, y);
    w = div_rcp(jz, rho, y);
}

__device__ __forceinline__ void macro_3d(const double* f, double Tlag, const PhysC& P, double& rho, double& u,
                                         double& v, double& w) {
    double jx, jy, jz;
    macro_3d(f, Tlag, P, rho, u, v, w, jx, jy, jz);
}

template <int QT>
__device__ __forceinline__ double sumT(const double* g) {
    double T = g[0] + g[1] + g[2] + g[3] + g[4];
    if (QT == 7) T = T + g[5] + g[6];
    return T;
}

}  // namespace lbm
