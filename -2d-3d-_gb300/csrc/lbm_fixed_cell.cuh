// lbm_fixed_cell.cuh - the fixed arithmetic of FP64 handles (lbm_params.arith =
// LBM_ARITH_FIXED): the coupled MRT step to FP64 accuracy on the integer pipes.
//
// GB300 issues FP64 operations at 2 per clock per SM, against 64 or more 32-bit integer
// operations.  The plain method's reference-order FP64 arithmetic is therefore bound by the
// FP64 pipe at about 6% of HBM bandwidth.  This form keeps FP64-grade accuracy without the
// FP64 pipe:
//
//  * Number format "q60": a population, moment or scalar x is held as the int64
//    round(x * 2^60).  Range |x| < 8, resolution 2^-60 = 8.7e-19: finer than an FP64 ulp for
//    every value above 2^-8 (all flow populations; thermal populations are compared to their
//    largest magnitude, about 0.1).
//  * Populations are deviations from the rest state, d_a = f_a - w_a and e_a = g_a - wT_a Tref,
//    as in the FP32/FP16 forms; moments of deviations are the reference's moments minus those
//    of the rest state.
//  * Additions and integer multiples are exact two's-complement integer operations (done on
//    unsigned 64-bit words, so an intermediate that wraps is still exact: every value that
//    enters a product is in range).  The moment transforms are the reference's integer
//    matrices, so they round nothing.
//  * Products are 64 x 64 -> 128-bit integer multiplies: of two q60 values (equilibria, the
//    force, B = u T, 1/rho by Newton's iteration), or of a q60 value with a constant scaled by
//    2^64 (relaxation rates over the row norms).  Each rounds once, down, by < 2^-60.
//  * The collision adds the relaxation update in moment space to the populations:
//      f_post = f + M^-1 delta,  delta_i = -s_i (m_i - meq_i) + source_i,
//    with M^-1 = M^T D^-1 because the rows of the reference's moment matrices are orthogonal
//    (D holds their squared norms: the reference's divisors 19, 2394, 252, 10, 40, 36, 72, 12,
//    24, 4, 8 in 3D; 9, 36, 36, 6, 12, 4 in 2D; 7, 2, 42, 12, 4 and 5, 2, 20, 4 for the
//    thermal sets).  c_i = delta_i / D_i is one product per term; f_post - f = M^T c is exact.
//    Since every row but the first has zero sum, mass is conserved exactly.
//
// The operations, their order and the lag structure (which T and which force each macro step
// uses) are those of the two-kernel fused step of the plain method (lbm_exact.cu), which are
// the reference's (3DRB.F90:227-241).  The results differ from the reference's by rounding
// only: the tests bound them at 1e-12 relative in the populations after 1000 steps and 1e-10
// in Nu.
//
// Every function here is host-compilable (g++ with the CUDA headers): the CPU tests run the
// same cell bodies through a host stepper and compare them with the oracle, and the GPU tests
// compare the kernels with that stepper bit for bit (integer arithmetic rounds identically on
// both).
#pragma once

#include <cstdint>
#include <cmath>

#include "lbm_internal.h"

namespace lbm {
namespace fxa {

constexpr int kFrac = 60;

// A q60 number: two's-complement bits of round(x * 2^60).  Arithmetic on the unsigned word
// is exact modulo 2^64.
struct q60 {
    unsigned long long u;
    q60() = default;
    // round(x * 2^60), ties to even (the scaling by 2^60 is exact)
    __device__ __forceinline__ explicit q60(double x) {
#ifdef __CUDA_ARCH__
        u = (unsigned long long)__double2ll_rn(x * 0x1p60);
#else
        u = (unsigned long long)std::llrint(x * 0x1p60);
#endif
    }
    __device__ __forceinline__ long long s() const { return (long long)u; }
};
__device__ __forceinline__ q60 Qb(long long v) {
    q60 r;
    r.u = (unsigned long long)v;
    return r;
}
__device__ __forceinline__ q60 operator+(q60 a, q60 b) { return Qb((long long)(a.u + b.u)); }
__device__ __forceinline__ q60 operator-(q60 a, q60 b) { return Qb((long long)(a.u - b.u)); }
__device__ __forceinline__ q60 operator-(q60 a) { return Qb((long long)(0ULL - a.u)); }
__device__ __forceinline__ q60 operator*(int k, q60 a) { return Qb((long long)((unsigned long long)(long long)k * a.u)); }
// floor(x / 2)
__device__ __forceinline__ q60 half(q60 a) { return Qb(a.s() >> 1); }

// The nearest double to x (one rounding; the scaling by 2^-60 is exact).
__device__ __forceinline__ double to_double(q60 a) {
#ifdef __CUDA_ARCH__
    return __ll2double_rn(a.s()) * 0x1p-60;
#else
    return (double)a.s() * 0x1p-60;
#endif
}

constexpr long long kOne = 1LL << kFrac;

// Product of two q60 numbers, rounded down to q60: bits 60..123 of the 128-bit product.  On
// the GPU the high word is one signed 64 x 64 high multiply (mul.hi.s64) and the low word a
// 64-bit multiply; the host uses a 128-bit integer.  Both give the same bits.
__device__ __forceinline__ q60 mul(q60 a, q60 b) {
#ifdef __CUDA_ARCH__
    const unsigned long long hi = (unsigned long long)__mul64hi(a.s(), b.s());
    const unsigned long long lo = a.u * b.u;
    return Qb((long long)((hi << (64 - kFrac)) | (lo >> kFrac)));
#else
    return Qb((long long)(((__int128)a.s() * (__int128)b.s()) >> kFrac));
#endif
}
// Product with a non-negative constant k given as an even K = round(k * 2^(64-S)) (k < 2^(S-1)),
// rounded down: floor(a k).  Constants are stored as magnitudes and their signs written into
// the formulas, because an unsigned high multiply needs no sign correction: with
// a' = a + 2^63 (the top bit flipped, a' >= 0), floor(a' K / 2^64) = floor(a K / 2^64) + K/2
// for an even K, and for S = 1, floor(a' K / 2^63) = floor(a K / 2^63) + K.
template <int S>
__device__ __forceinline__ q60 mulk(q60 a, long long K) {
#ifdef __CUDA_ARCH__
    const unsigned long long ab = a.u ^ 0x8000000000000000ULL;
    const unsigned long long Ku = (unsigned long long)K;
    const unsigned long long hi = __umul64hi(ab, Ku);
    if constexpr (S == 0) {
        return Qb((long long)(hi - (Ku >> 1)));
    } else {
        const unsigned long long lo = ab * Ku;
        return Qb((long long)(((hi << S) | (lo >> (64 - S))) - Ku));
    }
#else
    return Qb((long long)(((__int128)a.s() * (__int128)K) >> (64 - S)));
#endif
}

// 1/rho for rho in (1/2, 4): an FP32 reciprocal of the leading bits (24 correct bits), then
// two Newton steps r <- r + r (1 - rho r) in q60 (48, then beyond 60 bits).
__device__ __forceinline__ q60 recip(q60 rho) {
    float x = (float)(int)(rho.s() >> 32) * 0x1p-28f;
    x = x < 0.5f ? 0.5f : (x > 4.0f ? 4.0f : x);
#ifdef __CUDA_ARCH__
    const float r0 = __frcp_rn(x);
    q60 r = Qb((long long)__float2int_rz(r0 * 0x1p30f) << 30);
#else
    const float r0 = 1.0f / x;
    q60 r = Qb((long long)(int)(r0 * 0x1p30f) << 30);
#endif
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const q60 e = Qb(kOne) - mul(rho, r);
        r = r + mul(r, e);
    }
    return r;
}

__device__ __forceinline__ double quiet_nan() {
#ifdef __CUDA_ARCH__
    return __longlong_as_double(0x7FF8000000000000LL);
#else
    return std::nan("");
#endif
}

// Read-only loads of population buffers (the read-only data path on the GPU).
__device__ __forceinline__ q60 ldq(const long long* p, long long idx) {
#ifdef __CUDA_ARCH__
    return Qb(__ldg(p + idx));
#else
    return Qb(p[idx]);
#endif
}

}  // namespace fxa

// Constants of the fixed arithmetic for one run, from the commondata constants.  Each is the
// magnitude of a constant as an even K = round(|k| 2^64) (|k| < 1/2), or 2^63 where noted
// (|k| < 1); the comments give the signed constant and the formulas apply its sign.
struct PhysX {
    long long w[19];     // flow rest weights w_a (q60): D2Q9 in the first 9, or D3Q19
    long long wt[7];     // thermal rest populations wT_a Tref (q60)
    long long tref;      // sum_a wT_a Tref (q60): T = sum_a e_a + tref exactly
    long long gb;        // gBeta
    // 3D flow: c_i = k_n n_i + k_s (source product), n_i the non-equilibrium moment
    long long e_n, e_s;        // -Se/2394, (1 - Se/2) 38/2394 (times u.F)
    long long p_n, p_s;        // -Seps/252, -(1 - Seps/2) 11/252
    long long q_n, q_p, q_s;   // -Sq/40, -Sq/60 (the -2/3 rho u of meq_q), -(1 - Sq/2)(2/3)/40 (times F_y)
    long long j_f;             // 1/10 (F_y on the j_y moment)
    long long x9_n, x9_s;      // -Snu/36, -(1 - Snu/2) 2/36
    long long x10_n, x10_s;    // -Spi/72, (1 - Spi/2)/72
    long long x11_n, x11_s;    // -Snu/12, (1 - Snu/2) 2/12
    long long x12_n, x12_s;    // -Spi/24, -(1 - Spi/2)/24
    long long x13_n, x13_s;    // -Snu/4, (1 - Snu/2)/4 (times u F_y, w F_y)
    long long m_n;             // -Sm/8
    // 2D flow
    long long e2_n, e2_s;      // -Snu/36, (6 - 3 Snu)/36
    long long q2_n, q2_s;      // -Sq/12, -(1 - Sq/2)/12
    long long j2_f;            // 1/6
    long long x7_n, x7_s;      // -Snu/4, -(2 - Snu)/4
    long long x8_s;            // (1 - Snu/2)/4
    // thermal (3D: n4 row norm 42, n5 12, n6 4; 2D: n3 20, n4 4)
    long long qk2;             // -Qk/2, scale 2^63
    long long sg2;             // SG/2
    long long t_n, t_a;        // -Qnu/norm; Qnu a_T/norm of the a_T T moment, of sign t_a_neg
    long long t5_n, t6_n;      // 3D: -Qnu/12, -Qnu/4; 2D: t5_n = -Qnu/4
    long long bc_lo[3], bc_hi[3];  // constant-T wall terms of deviations (q60), per axis
    int t_a_neg;               // 1 when Qnu a_T < 0 (a_T = -3/4, -2/3; the legacy paraA may be either)
    int use_g;
};

// Magnitude k >= 0 as an even round(k * 2^(64-S)); false when k leaves [0, 2^(S-1)).
inline bool fx_const(long double k, int S, long long& K) {
    const long double lim = S == 0 ? 0.5L : 1.0L;
    if (!(k >= 0 && k < lim)) return false;
    K = (long long)std::llround(k * (S == 0 ? 0x1p64L : 0x1p63L)) & ~1LL;
    return true;
}

// The constants of one run; false when a constant leaves its range (a relaxation rate
// outside the stable range).  Host code.
inline bool make_physx(const lbm_params& p, const lbm_constants& c, PhysX& X) {
    X = PhysX{};
    const bool d3 = p.dim == 3;
    const long double w3[19] = {1.0L / 3, 1.0L / 18, 1.0L / 18, 1.0L / 18, 1.0L / 18, 1.0L / 18, 1.0L / 18,
                                1.0L / 36, 1.0L / 36, 1.0L / 36, 1.0L / 36, 1.0L / 36, 1.0L / 36,
                                1.0L / 36, 1.0L / 36, 1.0L / 36, 1.0L / 36, 1.0L / 36, 1.0L / 36};
    const long double w2[9] = {4.0L / 9, 1.0L / 9, 1.0L / 9, 1.0L / 9, 1.0L / 9,
                               1.0L / 36, 1.0L / 36, 1.0L / 36, 1.0L / 36};
    for (int a = 0; a < 19; ++a) X.w[a] = (long long)std::llround((d3 ? w3[a] : (a < 9 ? w2[a] : 0.0L)) * 0x1p60L);
    const int qt = d3 ? 7 : 5;
    X.tref = 0;
    for (int a = 0; a < 7; ++a) {
        const long double wt = a == 0 ? c.omegaT0 : c.omegaT1;
        X.wt[a] = a < qt ? (long long)std::llround(wt * (long double)c.Tref * 0x1p60L) : 0;
        X.tref += X.wt[a];
    }
    bool ok = fx_const(c.gBeta, 0, X.gb);
    const long double Se = c.Se, Seps = c.Seps, Sq = c.Sq, Snu = c.Snu, Spi = c.Spi, Sm = c.Sm;
    if (d3) {
        ok = ok && fx_const(Se / 2394, 0, X.e_n) && fx_const((1 - Se / 2) * 38 / 2394, 0, X.e_s);
        ok = ok && fx_const(Seps / 252, 0, X.p_n) && fx_const((1 - Seps / 2) * 11 / 252, 0, X.p_s);
        ok = ok && fx_const(Sq / 40, 0, X.q_n) && fx_const(Sq / 60, 0, X.q_p) &&
             fx_const((1 - Sq / 2) * (2.0L / 3) / 40, 0, X.q_s);
        ok = ok && fx_const(1.0L / 10, 0, X.j_f);
        ok = ok && fx_const(Snu / 36, 0, X.x9_n) && fx_const((1 - Snu / 2) * 2 / 36, 0, X.x9_s);
        ok = ok && fx_const(Spi / 72, 0, X.x10_n) && fx_const((1 - Spi / 2) / 72, 0, X.x10_s);
        ok = ok && fx_const(Snu / 12, 0, X.x11_n) && fx_const((1 - Snu / 2) * 2 / 12, 0, X.x11_s);
        ok = ok && fx_const(Spi / 24, 0, X.x12_n) && fx_const((1 - Spi / 2) / 24, 0, X.x12_s);
        ok = ok && fx_const(Snu / 4, 0, X.x13_n) && fx_const((1 - Snu / 2) / 4, 0, X.x13_s);
        ok = ok && fx_const(Sm / 8, 0, X.m_n);
    } else {
        ok = ok && fx_const(Snu / 36, 0, X.e2_n) && fx_const((6 - 3 * Snu) / 36, 0, X.e2_s);
        ok = ok && fx_const(Sq / 12, 0, X.q2_n) && fx_const((1 - Sq / 2) / 12, 0, X.q2_s);
        ok = ok && fx_const(1.0L / 6, 0, X.j2_f);
        ok = ok && fx_const(Snu / 4, 0, X.x7_n) && fx_const((2 - Snu) / 4, 0, X.x7_s);
        ok = ok && fx_const((1 - Snu / 2) / 4, 0, X.x8_s);
    }
    const long double Qk = c.Qk, Qnu = c.Qnu, SG = c.SG;
    // a_T of the thermal equilibrium moment: -3/4 (3D), -2/3 (2D), paraA in the legacy scheme
    const long double aT = p.legacy_thermal ? (long double)c.paraA : (d3 ? -0.75L : -2.0L / 3);
    const long double nrm = d3 ? 42 : 20;
    const long double ta = Qnu * aT / nrm;
    X.t_a_neg = ta < 0 ? 1 : 0;
    ok = ok && fx_const(Qk / 2, 1, X.qk2) && fx_const(SG / 2, 0, X.sg2);
    ok = ok && fx_const(Qnu / nrm, 0, X.t_n) && fx_const(ta < 0 ? -ta : ta, 0, X.t_a);
    ok = ok && fx_const(d3 ? Qnu / 12 : Qnu / 4, 0, X.t5_n) && fx_const(Qnu / 4, 0, X.t6_n);
    X.use_g = p.use_g ? 1 : 0;
    const Geo dg = deviation_geo(make_geo(p, c), c);
    for (int a = 0; a < 3; ++a) {
        // round(x 2^60) ties to even, as the device conversion q60(double) rounds
        X.bc_lo[a] = (long long)std::llrint(dg.bcT_lo[a] * 0x1p60);
        X.bc_hi[a] = (long long)std::llrint(dg.bcT_hi[a] * 0x1p60);
    }
    return ok;
}

namespace fxa {

// ------------------------------------------------------------------------------------
// macro (3DRB.F90:1066-1098, 2DRB.F90:878-894) on q60 deviations: rho = 1 + sum d,
// P = rho u = sum e d + F/2 (3D: F_y = rho gBeta (T_lag - Tref), lag = T_lag - Tref;
// 2D: the force stored by the collision, lag = F_y), u = P / rho.
// ------------------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void macro(const q60* d, q60 lag, const PhysX& X, q60& rho, q60* P, q60* U) {
    if (D == 2) {
        rho = Qb(kOne) + d[0] + d[1] + d[2] + d[3] + d[4] + d[5] + d[6] + d[7] + d[8];
        P[0] = d[1] - d[3] + d[5] - d[6] - d[7] + d[8];
        P[1] = d[2] - d[4] + d[5] + d[6] - d[7] - d[8] + half(lag);
        P[2] = Qb(0);
    } else {
        q60 s = d[0];
#pragma unroll
        for (int a = 1; a < 19; ++a) s = s + d[a];
        rho = Qb(kOne) + s;
        const q60 Fy = mul(rho, mulk<0>(lag, X.gb));
        P[0] = d[1] - d[2] + d[7] - d[8] + d[9] - d[10] + d[11] - d[12] + d[13] - d[14];
        P[1] = d[3] - d[4] + d[7] + d[8] - d[9] - d[10] + d[15] - d[16] + d[17] - d[18] + half(Fy);
        P[2] = d[5] - d[6] + d[11] + d[12] - d[13] - d[14] + d[15] + d[16] - d[17] - d[18];
    }
    const q60 r = recip(rho);
    U[0] = mul(P[0], r);
    U[1] = mul(P[1], r);
    U[2] = D == 3 ? mul(P[2], r) : Qb(0);
}

// ------------------------------------------------------------------------------------
// D2Q9 MRT collision with Guo forcing (2DRB.F90:688-759), F = (0, F_y).  rho, P = rho u, U,
// tdev = T - Tref; returns F_y (the force the reference stores, 2DRB.F90:718-719).
// ------------------------------------------------------------------------------------
__device__ __forceinline__ q60 collide_2d(const q60* d, q60 rho, const q60* P, const q60* U, q60 tdev, const PhysX& X,
                                          q60* dp) {
    const q60 dr = rho - Qb(kOne);
    const q60 Fy = mul(rho, mulk<0>(tdev, X.gb));
    const q60 ruu = mul(P[0], U[0]), rvv = mul(P[1], U[1]), ruv = mul(P[0], U[1]);
    const q60 vF = mul(U[1], Fy), uF = mul(U[0], Fy);
    const q60 s14 = d[1] + d[2] + d[3] + d[4], s58 = d[5] + d[6] + d[7] + d[8];
    const q60 m1 = -4 * d[0] - s14 + 2 * s58;
    const q60 m2 = 4 * d[0] - 2 * s14 + s58;
    const q60 xs = d[5] - d[6] - d[7] + d[8], ys = d[5] + d[6] - d[7] - d[8];
    const q60 m4 = -2 * d[1] + 2 * d[3] + xs;
    const q60 m6 = -2 * d[2] + 2 * d[4] + ys;
    const q60 m7 = d[1] - d[2] + d[3] - d[4];
    const q60 m8 = d[5] - d[6] + d[7] - d[8];
    // meq (2DRB.F90:698-706) relative to the rest state: e1 = -2 dr + 3 rho u^2,
    // e2 = dr - 3 rho u^2, e4 = -rho u, e6 = -rho v, e7 = rho (uu - vv), e8 = rho u v
    const q60 ru2 = ruu + rvv;
    const q60 n1 = m1 + 2 * dr - 3 * ru2;
    const q60 n2 = m2 - dr + 3 * ru2;
    const q60 n7 = m7 - (ruu - rvv);
    const q60 n8 = m8 - ruv;
    // c_i = (-s_i n_i + source_i) / D_i (sources 2DRB.F90:729-737 with F_x = 0)
    const q60 sv = mulk<0>(vF, X.e2_s);
    const q60 c1 = -mulk<0>(n1, X.e2_n) + sv;
    const q60 c2 = -mulk<0>(n2, X.e2_n) - sv;
    const q60 c4 = -mulk<0>(m4 + P[0], X.q2_n);
    const q60 c5 = mulk<0>(Fy, X.j2_f);
    const q60 c6 = -mulk<0>(m6 + P[1], X.q2_n) - mulk<0>(Fy, X.q2_s);
    const q60 c7 = -mulk<0>(n7, X.x7_n) - mulk<0>(vF, X.x7_s);
    const q60 c8 = -mulk<0>(n8, X.x7_n) + mulk<0>(uF, X.x8_s);
    // f_post - f = M^T c (columns of M: 2DRB.F90:743-759 times the row norms)
    const q60 ax = -c1 - 2 * c2, dg = 2 * c1 + c2;
    const q60 X4 = 2 * c4, Y6 = c5 - 2 * c6, Y = c5 + c6;
    dp[0] = d[0] - 4 * c1 + 4 * c2;
    dp[1] = d[1] + ax - X4 + c7;
    dp[2] = d[2] + ax + Y6 - c7;
    dp[3] = d[3] + ax + X4 + c7;
    dp[4] = d[4] + ax - Y6 - c7;
    dp[5] = d[5] + dg + c4 + Y + c8;
    dp[6] = d[6] + dg - c4 + Y - c8;
    dp[7] = d[7] + dg - c4 - Y + c8;
    dp[8] = d[8] + dg + c4 - Y - c8;
    return Fy;
}

// ------------------------------------------------------------------------------------
// D3Q19 MRT collision with Guo forcing (3DRB.F90:714-943), F = (0, F_y, 0).
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void collide_3d(const q60* d, q60 rho, const q60* P, const q60* U, q60 tdev, const PhysX& X,
                                           q60* dp) {
    const q60 dr = rho - Qb(kOne);
    const q60 Fy = mul(rho, mulk<0>(tdev, X.gb));
    // equilibrium products rho u_a u_b = P_a u_b
    const q60 ruu = mul(P[0], U[0]), rvv = mul(P[1], U[1]), rww = mul(P[2], U[2]);
    const q60 ruv = mul(P[0], U[1]), rvw = mul(P[1], U[2]), ruw = mul(P[0], U[2]);
    const q60 vF = mul(U[1], Fy), uF = mul(U[0], Fy), wF = mul(U[2], Fy);
    // moments of the deviations (3DRB.F90:714-775)
    const q60 s16 = d[1] + d[2] + d[3] + d[4] + d[5] + d[6];
    const q60 q710 = d[7] + d[8] + d[9] + d[10], q1114 = d[11] + d[12] + d[13] + d[14];
    const q60 e712 = q710 + q1114;
    const q60 e1518 = d[15] + d[16] + d[17] + d[18];
    const q60 s718 = e712 + e1518;
    const q60 m1 = -30 * d[0] - 11 * s16 + 8 * s718;
    const q60 m2 = 12 * d[0] - 4 * s16 + s718;
    const q60 xs = d[7] - d[8] + d[9] - d[10] + d[11] - d[12] + d[13] - d[14];
    const q60 ys = d[7] + d[8] - d[9] - d[10] + d[15] - d[16] + d[17] - d[18];
    const q60 zs = d[11] + d[12] - d[13] - d[14] + d[15] + d[16] - d[17] - d[18];
    const q60 m4 = -4 * (d[1] - d[2]) + xs;
    const q60 m6 = -4 * (d[3] - d[4]) + ys;
    const q60 m8 = -4 * (d[5] - d[6]) + zs;
    const q60 a12 = d[1] + d[2], a36 = d[3] + d[4] + d[5] + d[6];
    const q60 m9 = 2 * a12 - a36 + e712 - 2 * e1518;
    const q60 m10 = -4 * a12 + 2 * a36 + e712 - 2 * e1518;
    const q60 a34m56 = (d[3] + d[4]) - (d[5] + d[6]);
    const q60 m11 = a34m56 + q710 - q1114;
    const q60 m12 = -2 * a34m56 + q710 - q1114;
    const q60 m13 = d[7] - d[8] - d[9] + d[10];
    const q60 m14 = d[15] - d[16] - d[17] + d[18];
    const q60 m15 = d[11] - d[12] - d[13] + d[14];
    const q60 m16 = d[7] - d[8] + d[9] - d[10] - d[11] + d[12] - d[13] + d[14];
    const q60 m17 = -d[7] - d[8] + d[9] + d[10] + d[15] - d[16] + d[17] - d[18];
    const q60 m18 = d[11] + d[12] - d[13] - d[14] - d[15] - d[16] + d[17] + d[18];
    // meq (3DRB.F90:780-798) relative to the rest state: e1 = -11 dr + 19 rho u^2,
    // e2 = 3 dr - 11/2 rho u^2, e4 = -2/3 rho u, e9 = rho (2uu - vv - ww), e10 = -e9/2,
    // e11 = rho (vv - ww), e12 = -e11/2, e13..e15 = rho uv, rho vw, rho uw
    const q60 ru2 = ruu + rvv + rww;
    const q60 n1 = m1 + 11 * dr - 19 * ru2;
    const q60 n2 = m2 - 3 * dr + half(11 * ru2);
    const q60 e9 = 2 * ruu - rvv - rww, e11 = rvv - rww;
    const q60 n9 = m9 - e9, n10 = m10 + half(e9);
    const q60 n11 = m11 - e11, n12 = m12 + half(e11);
    // c_i = (-s_i n_i + source_i) / D_i (rates 3DRB.F90:803-821, sources :831-849)
    const q60 c1 = -mulk<0>(n1, X.e_n) + mulk<0>(vF, X.e_s);
    const q60 c2 = -mulk<0>(n2, X.p_n) - mulk<0>(vF, X.p_s);
    const q60 c4 = -mulk<0>(m4, X.q_n) - mulk<0>(P[0], X.q_p);
    const q60 c5 = mulk<0>(Fy, X.j_f);
    const q60 c6 = -mulk<0>(m6, X.q_n) - mulk<0>(P[1], X.q_p) - mulk<0>(Fy, X.q_s);
    const q60 c8 = -mulk<0>(m8, X.q_n) - mulk<0>(P[2], X.q_p);
    const q60 c9 = -mulk<0>(n9, X.x9_n) - mulk<0>(vF, X.x9_s);
    const q60 c10 = -mulk<0>(n10, X.x10_n) + mulk<0>(vF, X.x10_s);
    const q60 c11 = -mulk<0>(n11, X.x11_n) + mulk<0>(vF, X.x11_s);
    const q60 c12 = -mulk<0>(n12, X.x12_n) - mulk<0>(vF, X.x12_s);
    const q60 c13 = -mulk<0>(m13 - ruv, X.x13_n) + mulk<0>(uF, X.x13_s);
    const q60 c14 = -mulk<0>(m14 - rvw, X.x13_n) + mulk<0>(wF, X.x13_s);
    const q60 c15 = -mulk<0>(m15 - ruw, X.x13_n);
    const q60 c16 = -mulk<0>(m16, X.m_n), c17 = -mulk<0>(m17, X.m_n), c18 = -mulk<0>(m18, X.m_n);
    // f_post - f = M^T c (columns of M: 3DRB.F90:861-943 times the row norms)
    const q60 ba = -11 * c1 - 4 * c2, bd = 8 * c1 + c2;
    const q60 p9 = -c9 + 2 * c10, p11 = c11 - 2 * c12;
    const q60 X4 = 4 * c4, Y6 = c5 - 4 * c6, Z8 = 4 * c8;
    const q60 bx = ba + 2 * c9 - 4 * c10;
    dp[0] = d[0] - 30 * c1 + 12 * c2;
    dp[1] = d[1] + bx - X4;
    dp[2] = d[2] + bx + X4;
    dp[3] = d[3] + ba + Y6 + p9 + p11;
    dp[4] = d[4] + ba - Y6 + p9 + p11;
    dp[5] = d[5] + ba - Z8 + p9 - p11;
    dp[6] = d[6] + ba + Z8 + p9 - p11;
    const q60 Y = c5 + c6;
    const q60 dxy = bd + c9 + c10 + c11 + c12;
    const q60 dxz = bd + c9 + c10 - c11 - c12;
    const q60 dyz = bd - 2 * c9 - 2 * c10;
    dp[7] = d[7] + dxy + c4 + Y + c13 + c16 - c17;
    dp[8] = d[8] + dxy - c4 + Y - c13 - c16 - c17;
    dp[9] = d[9] + dxy + c4 - Y - c13 + c16 + c17;
    dp[10] = d[10] + dxy - c4 - Y + c13 - c16 + c17;
    dp[11] = d[11] + dxz + c4 + c8 + c15 - c16 + c18;
    dp[12] = d[12] + dxz - c4 + c8 - c15 + c16 + c18;
    dp[13] = d[13] + dxz + c4 - c8 - c15 - c16 - c18;
    dp[14] = d[14] + dxz - c4 - c8 + c15 + c16 - c18;
    dp[15] = d[15] + dyz + Y + c8 + c14 + c17 - c18;
    dp[16] = d[16] + dyz - Y + c8 - c14 - c17 - c18;
    dp[17] = d[17] + dyz + Y - c8 - c14 + c17 + c18;
    dp[18] = d[18] + dyz - Y - c8 + c14 - c17 + c18;
}

// ------------------------------------------------------------------------------------
// Thermal MRT collisions with the M1G term: D3Q7 (3DRB.F90:1121-1191) and D2Q5
// (2DRB.F90:921-974).  e: deviations; T = tdev + tref; B: B_prev in, B out (when use_g).
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void collideT_3d(const q60* e, const q60* U, q60 tdev, q60* B, const PhysX& X, q60* ep) {
    const q60 T = tdev + Qb(X.tref);
    const q60 bx = mul(U[0], T), by = mul(U[1], T), bz = mul(U[2], T);
    q60 dbx = Qb(0), dby = Qb(0), dbz = Qb(0);
    if (X.use_g) {
        dbx = bx - B[0];
        dby = by - B[1];
        dbz = bz - B[2];
        B[0] = bx;
        B[1] = by;
        B[2] = bz;
    }
    const q60 n1 = e[1] - e[2], n2 = e[3] - e[4], n3 = e[5] - e[6];
    const q60 s16 = e[1] + e[2] + e[3] + e[4] + e[5] + e[6];
    const q60 n4 = -6 * e[0] + s16;
    const q60 n5 = 2 * (e[1] + e[2]) - (e[3] + e[4] + e[5] + e[6]);
    const q60 n6 = e[3] + e[4] - e[5] - e[6];
    const q60 c1 = -mulk<1>(n1 - bx, X.qk2) + mulk<0>(dbx, X.sg2);
    const q60 c2 = -mulk<1>(n2 - by, X.qk2) + mulk<0>(dby, X.sg2);
    const q60 c3 = -mulk<1>(n3 - bz, X.qk2) + mulk<0>(dbz, X.sg2);
    const q60 ta = mulk<0>(tdev, X.t_a);
    const q60 c4 = -mulk<0>(n4, X.t_n) + (X.t_a_neg ? -ta : ta);
    const q60 c5 = -mulk<0>(n5, X.t5_n), c6 = -mulk<0>(n6, X.t6_n);
    const q60 h = c4 - c5;
    ep[0] = e[0] - 6 * c4;
    ep[1] = e[1] + c1 + c4 + 2 * c5;
    ep[2] = e[2] - c1 + c4 + 2 * c5;
    ep[3] = e[3] + c2 + h + c6;
    ep[4] = e[4] - c2 + h + c6;
    ep[5] = e[5] + c3 + h - c6;
    ep[6] = e[6] - c3 + h - c6;
}

__device__ __forceinline__ void collideT_2d(const q60* e, const q60* U, q60 tdev, q60* B, const PhysX& X, q60* ep) {
    const q60 T = tdev + Qb(X.tref);
    const q60 bx = mul(U[0], T), by = mul(U[1], T);
    q60 dbx = Qb(0), dby = Qb(0);
    if (X.use_g) {
        dbx = bx - B[0];
        dby = by - B[1];
        B[0] = bx;
        B[1] = by;
    }
    const q60 n1 = e[1] - e[3], n2 = e[2] - e[4];
    const q60 n3 = -4 * e[0] + e[1] + e[2] + e[3] + e[4];
    const q60 n4 = e[1] - e[2] + e[3] - e[4];
    const q60 c1 = -mulk<1>(n1 - bx, X.qk2) + mulk<0>(dbx, X.sg2);
    const q60 c2 = -mulk<1>(n2 - by, X.qk2) + mulk<0>(dby, X.sg2);
    const q60 ta = mulk<0>(tdev, X.t_a);
    const q60 c3 = -mulk<0>(n3, X.t_n) + (X.t_a_neg ? -ta : ta);
    const q60 c4 = -mulk<0>(n4, X.t5_n);
    ep[0] = e[0] - 4 * c3;
    ep[1] = e[1] + c1 + c3 + c4;
    ep[2] = e[2] + c2 + c3 - c4;
    ep[3] = e[3] - c1 + c3 + c4;
    ep[4] = e[4] - c2 + c3 - c4;
}

}  // namespace fxa

// ------------------------------------------------------------------------------------
// Arrays of the fixed arithmetic: the fused buffers hold q60 deviations (passed to each
// call); the module arrays are the plain method's FP64 arrays (read by the first step,
// written by the materialisation); the lag state is q60: B_prev, and the 3D T lag
// (T_{n-1} - Tref) or the 2D stored force F_y.
// ------------------------------------------------------------------------------------
struct FixedArrays {
    double *f, *g, *rho, *u, *v, *w, *T, *Bx, *By, *Bz, *Tlag, *Fx, *Fy;
    long long *xb0, *xb1, *xb2, *xlag;
};

namespace fxa {

// Flow collision of step n (lbm_exact.cu k_flow): FIRST reads the module arrays (f, rho,
// u, T); otherwise f_{n-1} = pull(f_post_{n-1}), T_{n-1} = sum pull(g_post_{n-1}), and rho,
// u of the macro step of f_{n-1} with the lag.  2D stores the force F_y,n in the lag.
// g: geometry whose thermal wall terms are deviations (wall term - 2 wT Tref).
// PATH: 0 = any cell (the boundary rule where a pull leaves the lattice), 1 = a cell known to
// touch no face (fixed-offset pulls only), 2 = a face cell (boundary path only), 3 = a cell of
// an interior row (only x can leave the lattice: pull_flow_xrow / pull_thermal_xrow).
// I: index type of the cell's own accesses and of PATH 3's pulls (int when every array
// index fits in 32 bits: half the address arithmetic; the values do not depend on it).
template <int D, bool FIRST, int PATH = 0, class I = long long>
__device__ __forceinline__ void flow_cell(const Geo& g, const PhysX& X, const FixedArrays& A, const long long* fin,
                                          const long long* gin, long long* fout, long long c, int i, int j, int k) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    const I ni = (I)g.ncell, ci = (I)c;
    q60 d[Q], dp[Q], rho, P[3], U[3], tdev;
    if (FIRST) {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = q60(A.f[a * n + c]) - Qb(X.w[a]);
        rho = q60(A.rho[c]);
        U[0] = q60(A.u[c]);
        U[1] = q60(A.v[c]);
        U[2] = D == 3 ? q60(A.w[c]) : Qb(0);
#pragma unroll
        for (int b = 0; b < 3; ++b) P[b] = mul(rho, U[b]);
        tdev = q60(A.T[c]) - Qb(X.tref);
    } else {
        q60 ts = Qb(0);
        if (PATH == 3) {
            auto lf = [&](int a, I cc) { return ldq(fin, a * ni + cc); };
            auto lg = [&](int a, I cc) { return ldq(gin, a * ni + cc); };
#pragma unroll
            for (int a = 0; a < Q; ++a) d[a] = pull_flow_xrow<Q, q60>(g, a, i, ci, lf);
#pragma unroll
            for (int a = 0; a < QT; ++a) ts = ts + pull_thermal_xrow<QT, q60>(g, a, i, ci, lg);
        } else if (PATH == 1 || (PATH == 0 && aa_inner(g, i, j, k))) {  // no pull needs a boundary rule
#pragma unroll
            for (int a = 0; a < Q; ++a) {
                LBM_CHECK_CELL(g, c - lat_off<Q>(g, a));
                d[a] = ldq(fin, a * n + c - lat_off<Q>(g, a));
            }
#pragma unroll
            for (int a = 0; a < QT; ++a) ts = ts + ldq(gin, a * n + c - lat_off<QT>(g, a));
        } else {
            auto lf = [&](int a, long long cc) { return ldq(fin, a * n + cc); };
            auto lg = [&](int a, long long cc) { return ldq(gin, a * n + cc); };
#pragma unroll
            for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, q60>(g, a, i, j, k, c, lf);
#pragma unroll
            for (int a = 0; a < QT; ++a) ts = ts + pull_thermal<QT, q60>(g, a, i, j, k, c, lg);
        }
        tdev = ts;
        macro<D>(d, Qb(A.xlag[ci]), X, rho, P, U);
    }
    if (D == 2) {
        const q60 Fy = collide_2d(d, rho, P, U, tdev, X, dp);
        A.xlag[ci] = Fy.s();
    } else {
        collide_3d(d, rho, P, U, tdev, X, dp);
    }
#pragma unroll
    for (int a = 0; a < Q; ++a) fout[a * ni + ci] = dp[a].s();
}

// Streaming, boundary and macro of the flow, and thermal collision of step n (k_thermal).
template <int D, bool FIRST, int PATH = 0, class I = long long>
__device__ __forceinline__ void thermal_cell(const Geo& g, const PhysX& X, const FixedArrays& A, const long long* fin,
                                             const long long* gin, long long* gout, long long c, int i, int j, int k) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    const I ni = (I)g.ncell, ci = (I)c;
    q60 d[Q], e[QT], ep[QT], rho, P[3], U[3], B[3], tdev;
    const bool inner = PATH == 1 || (PATH == 0 && aa_inner(g, i, j, k));
    auto lf = [&](int a, long long cc) { return ldq(fin, a * n + cc); };
    if (PATH == 3) {
        auto lfi = [&](int a, I cc) { return ldq(fin, a * ni + cc); };
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow_xrow<Q, q60>(g, a, i, ci, lfi);
    } else if (inner) {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = ldq(fin, a * n + c - lat_off<Q>(g, a));
    } else {
#pragma unroll
        for (int a = 0; a < Q; ++a) d[a] = pull_flow<Q, q60>(g, a, i, j, k, c, lf);
    }
    if (FIRST) {
#pragma unroll
        for (int a = 0; a < QT; ++a) e[a] = q60(A.g[a * n + c]) - Qb(X.wt[a]);
        tdev = q60(A.T[c]) - Qb(X.tref);
        B[0] = q60(A.Bx[c]);
        B[1] = q60(A.By[c]);
        B[2] = D == 3 ? q60(A.Bz[c]) : Qb(0);
    } else {
        q60 ts = Qb(0);
        if (PATH == 3) {
            auto lg = [&](int a, I cc) { return ldq(gin, a * ni + cc); };
#pragma unroll
            for (int a = 0; a < QT; ++a) {
                e[a] = pull_thermal_xrow<QT, q60>(g, a, i, ci, lg);
                ts = ts + e[a];
            }
        } else if (inner) {
#pragma unroll
            for (int a = 0; a < QT; ++a) {
                e[a] = ldq(gin, a * n + c - lat_off<QT>(g, a));
                ts = ts + e[a];
            }
        } else {
            auto lg = [&](int a, long long cc) { return ldq(gin, a * n + cc); };
#pragma unroll
            for (int a = 0; a < QT; ++a) {
                e[a] = pull_thermal<QT, q60>(g, a, i, j, k, c, lg);
                ts = ts + e[a];
            }
        }
        tdev = ts;
        B[0] = Qb(A.xb0[ci]);
        B[1] = Qb(A.xb1[ci]);
        B[2] = D == 3 ? Qb(A.xb2[ci]) : Qb(0);
    }
    macro<D>(d, D == 2 ? Qb(A.xlag[ci]) : tdev, X, rho, P, U);
    if (D == 2) {
        collideT_2d(e, U, tdev, B, X, ep);
    } else {
        collideT_3d(e, U, tdev, B, X, ep);
        A.xlag[ci] = tdev.s();
    }
    if (FIRST || X.use_g) {
        A.xb0[ci] = B[0].s();
        A.xb1[ci] = B[1].s();
        if (D == 3) A.xb2[ci] = B[2].s();
    }
#pragma unroll
    for (int a = 0; a < QT; ++a) gout[a * ni + ci] = ep[a].s();
}

// The module arrays of step N (FP64) from the fused buffers f_post_N, g_post_N and the lag:
// f_N, g_N (streamed, with boundaries), rho_N and u_N of the macro step with the lag, T_N,
// B_prev, and the 3D T lag or 2D force.  A cell whose density or velocity left the range of
// a physical state gets a NaN density, which the diagnostics report as diverged.
template <int D>
__device__ __forceinline__ void materialize_cell(const Geo& g, const PhysX& X, const FixedArrays& A,
                                                 const long long* fin, const long long* gin, long long c, int i, int j,
                                                 int k) {
    constexpr int Q = (D == 2) ? 9 : 19, QT = (D == 2) ? 5 : 7;
    const long long n = g.ncell;
    q60 d[Q], rho, P[3], U[3];
    auto lf = [&](int a, long long cc) { return ldq(fin, a * n + cc); };
    auto lg = [&](int a, long long cc) { return ldq(gin, a * n + cc); };
    q60 ts = Qb(0);
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        d[a] = pull_flow<Q, q60>(g, a, i, j, k, c, lf);
        A.f[a * n + c] = to_double(d[a] + Qb(X.w[a]));
    }
#pragma unroll
    for (int a = 0; a < QT; ++a) {
        const q60 e = pull_thermal<QT, q60>(g, a, i, j, k, c, lg);
        ts = ts + e;
        A.g[a * n + c] = to_double(e + Qb(X.wt[a]));
    }
    const q60 lag = Qb(A.xlag[c]);
    macro<D>(d, lag, X, rho, P, U);
    const long long lim = kOne / 2;
    const bool bad = rho.s() <= lim || rho.s() >= 4 * kOne || U[0].s() > lim || U[0].s() < -lim ||
                     U[1].s() > lim || U[1].s() < -lim || U[2].s() > lim || U[2].s() < -lim;
    A.rho[c] = bad ? quiet_nan() : to_double(rho);
    A.u[c] = to_double(U[0]);
    A.v[c] = to_double(U[1]);
    if (D == 3) A.w[c] = to_double(U[2]);
    A.T[c] = to_double(ts + Qb(X.tref));
    A.Bx[c] = to_double(Qb(A.xb0[c]));
    A.By[c] = to_double(Qb(A.xb1[c]));
    if (D == 3) {
        A.Bz[c] = to_double(Qb(A.xb2[c]));
        A.Tlag[c] = to_double(lag + Qb(X.tref));
    } else {
        A.Fx[c] = 0.0;
        A.Fy[c] = to_double(lag);
    }
}

}  // namespace fxa
}  // namespace lbm
