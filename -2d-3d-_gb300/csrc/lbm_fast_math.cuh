// lbm_fast_math.cuh - FP32 per-cell arithmetic of the reduced-storage forms (shared by the
// two-kernel step in lbm_fast.cu and the single fused kernel in lbm_fused.cu).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "lbm_internal.h"

namespace lbm {

// ------------------------------------------------------------------------------------
// storage conversions
// ------------------------------------------------------------------------------------
template <class S> __device__ __forceinline__ float ldS(const S* p, long long i);
template <> __device__ __forceinline__ float ldS<float>(const float* p, long long i) { return __ldg(p + i); }
// FP16 values are fetched through the 16-bit integer __ldg builtin: the compiler schedules
// it like any other load (hoisting it above the pull's boundary selects), which the
// inline-assembly __half overload does not allow, and then reinterpreted.
template <> __device__ __forceinline__ float ldS<__half>(const __half* p, long long i) {
    return __half2float(__ushort_as_half(__ldg(reinterpret_cast<const unsigned short*>(p) + i)));
}
template <class S> __device__ __forceinline__ S toS(float x);
template <> __device__ __forceinline__ float toS<float>(float x) { return x; }
template <> __device__ __forceinline__ __half toS<__half>(float x) { return __float2half_rn(x); }

// ------------------------------------------------------------------------------------
// Stochastic rounding of new FP16 populations.  Near the onset of convection a step
// changes a stored deviation by less than half an FP16 unit in the last place (at 128^3,
// Ra 1e7, the buoyancy of a 1e-3 temperature seed moves populations by ~1e-8 per step
// against units of ~1e-6): round-to-nearest drops every such increment and the lattice
// stays conductive.  Rounding up with probability equal to the dropped fraction keeps the
// increments in expectation.  GB300 does it in one instruction for two values,
// cvt.rs.f16x2.f32 d, a, b, rbits: a goes to the upper half of d and takes rbits[31:16],
// b the lower half and rbits[15:0]; each value rounds up when the low 13 bits of its half
// plus its 13 dropped mantissa bits carry (measured on GB300).  The random bits of the new
// population a of cell c are half a&1 of the 32-bit word a>>1 of a hash of (step counter,
// cell, flow or thermal set), so every kernel form and both access patterns round a value
// alike whatever value it is paired with, and a run is reproducible bit for bit.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned fmix32(unsigned h) {
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    return h ^ (h >> 16);
}
// Seed of one cell's random bits for one set (kind 0 flow, 1 thermal) at step `tick`.
__device__ __forceinline__ unsigned sr_seed(unsigned long long tick, long long c, unsigned kind) {
    return fmix32((unsigned)c ^ fmix32((((unsigned)tick << 1) | kind) + 0x9E3779B9u));
}
// Random bits of directions 2j (low half) and 2j+1 (high half).  The seed is already a full
// avalanche hash of (step, cell, set), uniform over 32 bits, so each word only needs to be a
// distinct bijection of it: an offset, one multiply by an odd constant and an xorshift that
// folds the well-mixed high product bits into the low ones (3 instructions, against 9 for
// another full hash per word; the FP16 kernels are issue-bound at large lattices).
__device__ __forceinline__ unsigned sr_word(unsigned seed, int j) {
    const unsigned h = (seed + 0x9E3779B9u * (unsigned)(j + 1)) * 0x85EBCA6Bu;
    return h ^ (h >> 15);
}
__device__ __forceinline__ unsigned cvt_rs_f16x2(float hi, float lo, unsigned rbits) {
    unsigned d;
    asm("cvt.rs.f16x2.f32 %0, %1, %2, %3;" : "=r"(d) : "f"(hi), "f"(lo), "r"(rbits));
    return d;
}
__device__ __forceinline__ __half lo_half(unsigned d) { return __ushort_as_half((unsigned short)(d & 0xFFFFu)); }
__device__ __forceinline__ __half hi_half(unsigned d) { return __ushort_as_half((unsigned short)(d >> 16)); }

// The Q new populations v of one cell in storage type S (FP16: stochastically when sr,
// otherwise to nearest).
template <int Q>
__device__ __forceinline__ void round_cell(const float* v, float* h, bool, unsigned) {
#pragma unroll
    for (int a = 0; a < Q; ++a) h[a] = v[a];
}
template <int Q>
__device__ __forceinline__ void round_cell(const float* v, __half* h, bool sr, unsigned seed) {
#pragma unroll
    for (int j = 0; 2 * j < Q; ++j) {
        const float lo = v[2 * j], hi = 2 * j + 1 < Q ? v[2 * j + 1] : 0.0f;
        if (sr) {
            const unsigned d = cvt_rs_f16x2(hi, lo, sr_word(seed, j));
            h[2 * j] = lo_half(d);
            if (2 * j + 1 < Q) h[2 * j + 1] = hi_half(d);
        } else {
            h[2 * j] = __float2half_rn(lo);
            if (2 * j + 1 < Q) h[2 * j + 1] = __float2half_rn(hi);
        }
    }
}
// The same for two cells (paired forms): value a of each cell takes the bits it takes in
// round_cell.
template <int Q>
__device__ __forceinline__ void round_pair(const float* v0, const float* v1, float* h0, float* h1, bool, unsigned,
                                           unsigned) {
#pragma unroll
    for (int a = 0; a < Q; ++a) {
        h0[a] = v0[a];
        h1[a] = v1[a];
    }
}
template <int Q>
__device__ __forceinline__ void round_pair(const float* v0, const float* v1, __half* h0, __half* h1, bool sr,
                                           unsigned seed0, unsigned seed1) {
#pragma unroll
    for (int j = 0; 2 * j < Q; ++j) {
        const unsigned w0 = sr ? sr_word(seed0, j) : 0u, w1 = sr ? sr_word(seed1, j) : 0u;
#pragma unroll
        for (int a = 2 * j; a < 2 * j + 2 && a < Q; ++a) {
            if (sr) {
                const unsigned r0 = (a & 1) ? w0 >> 16 : w0 & 0xFFFFu, r1 = (a & 1) ? w1 >> 16 : w1 & 0xFFFFu;
                const unsigned d = cvt_rs_f16x2(v1[a], v0[a], (r1 << 16) | r0);
                h0[a] = lo_half(d);
                h1[a] = hi_half(d);
            } else {
                h0[a] = __float2half_rn(v0[a]);
                h1[a] = __float2half_rn(v1[a]);
            }
        }
    }
}

// Rest weights (D2Q9 2DRB.F90:506-512, D3Q19 3DRB.F90:669-671).
template <int Q>
__host__ __device__ constexpr double wrest(int a) {
    return Q == 9 ? (a == 0 ? 4.0 / 9.0 : (a <= 4 ? 1.0 / 9.0 : 1.0 / 36.0))
                  : (a == 0 ? 1.0 / 3.0 : (a <= 6 ? 1.0 / 18.0 : 1.0 / 36.0));
}

struct PhysF {
    float gBeta, Tref;
    float Snu, Sq, Se, Seps, Spi, Sm;
    float Qk, Qnu, SG, paraA;
    float omegaT0, omegaT1, geqc;
    int use_g, legacy;
    int sr;  // FP16 storage: stochastic rounding of the new populations (round_cell, round_pair)
};

inline PhysF to_physf(const PhysC& P) {
    PhysF F;
    F.gBeta = (float)P.gBeta; F.Tref = (float)P.Tref;
    F.Snu = (float)P.Snu; F.Sq = (float)P.Sq; F.Se = (float)P.Se; F.Seps = (float)P.Seps;
    F.Spi = (float)P.Spi; F.Sm = (float)P.Sm;
    F.Qk = (float)P.Qk; F.Qnu = (float)P.Qnu; F.SG = (float)P.SG; F.paraA = (float)P.paraA;
    F.omegaT0 = (float)P.omegaT0; F.omegaT1 = (float)P.omegaT1; F.geqc = (float)P.geqc;
    F.use_g = P.use_g; F.legacy = P.legacy;
    F.sr = 0;
    return F;
}

// Thermal wall terms for deviations: e_a = -e_opp + 2 wT (Tw - Tref).
inline Geo dev_geo(const Geo& g, const PhysC& P) {
    Geo d = g;
    for (int a = 0; a < 3; ++a) {
        d.bcT_lo[a] = g.bcT_lo[a] - 2.0 * P.omegaT1 * P.Tref;
        d.bcT_hi[a] = g.bcT_hi[a] - 2.0 * P.omegaT1 * P.Tref;
    }
    return d;
}

// ------------------------------------------------------------------------------------
// per-cell arithmetic (FP32, deviations)
// ------------------------------------------------------------------------------------
// D2Q9 MRT collision with Guo forcing (2DRB.F90:688-759) on deviations d.
__device__ __forceinline__ void fcollide_2d(const float* d, float dr, float rho, float u, float v, float Fy,
                                            const PhysF& P, float* dp) {
    const float m1 = -4.0f * d[0] - d[1] - d[2] - d[3] - d[4] + 2.0f * (d[5] + d[6] + d[7] + d[8]);
    const float m2 = 4.0f * d[0] - 2.0f * (d[1] + d[2] + d[3] + d[4]) + d[5] + d[6] + d[7] + d[8];
    const float m3 = d[1] - d[3] + d[5] - d[6] - d[7] + d[8];
    const float m4 = -2.0f * d[1] + 2.0f * d[3] + d[5] - d[6] - d[7] + d[8];
    const float m5 = d[2] - d[4] + d[5] + d[6] - d[7] - d[8];
    const float m6 = -2.0f * d[2] + 2.0f * d[4] + d[5] + d[6] - d[7] - d[8];
    const float m7 = d[1] - d[2] + d[3] - d[4];
    const float m8 = d[5] - d[6] + d[7] - d[8];
    const float uu = u * u, vv = v * v, q2 = uu + vv;
    // equilibrium moments relative to rest: meq_k(rho,u) - meq_k(1,0)
    const float e1 = -2.0f * dr + 3.0f * rho * q2;
    const float e2 = dr - 3.0f * rho * q2;
    const float e4 = -rho * u, e6 = -rho * v;
    const float e7 = rho * (uu - vv), e8 = rho * (u * v);
    // Guo source with Fx = 0
    const float s1 = (6.0f - 3.0f * P.Snu) * (v * Fy);
    const float s2 = -(6.0f - 3.0f * P.Snu) * (v * Fy);
    const float s6 = -(1.0f - 0.5f * P.Sq) * Fy;
    const float s7 = (2.0f - P.Snu) * (-v * Fy);
    const float s8 = (1.0f - 0.5f * P.Snu) * (u * Fy);
    const float mp0 = dr;
    const float mp1 = m1 - P.Snu * (m1 - e1) + s1;
    const float mp2 = m2 - P.Snu * (m2 - e2) + s2;
    const float mp3 = m3;
    const float mp4 = m4 - P.Sq * (m4 - e4);
    const float mp5 = m5 + Fy;
    const float mp6 = m6 - P.Sq * (m6 - e6) + s6;
    const float mp7 = m7 - P.Snu * (m7 - e7) + s7;
    const float mp8 = m8 - P.Snu * (m8 - e8) + s8;
    // M^-1 (2DRB.F90:743-759)
    const float A = mp0 * (1.0f / 9.0f);
    const float B9 = mp1 * (1.0f / 9.0f), B36 = mp1 * (1.0f / 36.0f), B18 = mp1 * (1.0f / 18.0f);
    const float C9 = mp2 * (1.0f / 9.0f), C18 = mp2 * (1.0f / 18.0f), C36 = mp2 * (1.0f / 36.0f);
    const float X6 = mp3 * (1.0f / 6.0f), Xq6 = mp4 * (1.0f / 6.0f), Xq12 = mp4 * (1.0f / 12.0f);
    const float Y6 = mp5 * (1.0f / 6.0f), Yq6 = mp6 * (1.0f / 6.0f), Yq12 = mp6 * (1.0f / 12.0f);
    const float P7 = mp7 * 0.25f, P8 = mp8 * 0.25f;
    const float ax = A - B36 - C18, dg = A + B18 + C36;
    dp[0] = A - B9 + C9;
    dp[1] = ax + X6 - Xq6 + P7;
    dp[2] = ax + Y6 - Yq6 - P7;
    dp[3] = ax - X6 + Xq6 + P7;
    dp[4] = ax - Y6 + Yq6 - P7;
    dp[5] = dg + X6 + Xq12 + Y6 + Yq12 + P8;
    dp[6] = dg - X6 - Xq12 + Y6 + Yq12 - P8;
    dp[7] = dg - X6 - Xq12 - Y6 - Yq12 + P8;
    dp[8] = dg + X6 + Xq12 - Y6 - Yq12 - P8;
}

// D3Q19 MRT collision with Guo forcing (3DRB.F90:714-943) on deviations d.
__device__ __forceinline__ void fcollide_3d(const float* d, float dr, float rho, float u, float v, float w,
                                            float Fy, const PhysF& P, float* dp) {
    const float s16 = d[1] + d[2] + d[3] + d[4] + d[5] + d[6];
    const float e712 = d[7] + d[8] + d[9] + d[10] + d[11] + d[12] + d[13] + d[14];
    const float e1518 = d[15] + d[16] + d[17] + d[18];
    const float s718 = e712 + e1518;
    const float m1 = -30.0f * d[0] - 11.0f * s16 + 8.0f * s718;
    const float m2 = 12.0f * d[0] - 4.0f * s16 + s718;
    const float xs = d[7] - d[8] + d[9] - d[10] + d[11] - d[12] + d[13] - d[14];
    const float m3 = d[1] - d[2] + xs;
    const float m4 = -4.0f * d[1] + 4.0f * d[2] + xs;
    const float ys = d[7] + d[8] - d[9] - d[10] + d[15] - d[16] + d[17] - d[18];
    const float m5 = d[3] - d[4] + ys;
    const float m6 = -4.0f * d[3] + 4.0f * d[4] + ys;
    const float zs = d[11] + d[12] - d[13] - d[14] + d[15] + d[16] - d[17] - d[18];
    const float m7 = d[5] - d[6] + zs;
    const float m8 = -4.0f * d[5] + 4.0f * d[6] + zs;
    const float m9 = 2.0f * (d[1] + d[2]) - (d[3] + d[4] + d[5] + d[6]) + e712 - 2.0f * e1518;
    const float m10 = -4.0f * (d[1] + d[2]) + 2.0f * (d[3] + d[4] + d[5] + d[6]) + e712 - 2.0f * e1518;
    const float q710 = d[7] + d[8] + d[9] + d[10], q1114 = d[11] + d[12] + d[13] + d[14];
    const float m11 = (d[3] + d[4]) - (d[5] + d[6]) + q710 - q1114;
    const float m12 = -2.0f * (d[3] + d[4]) + 2.0f * (d[5] + d[6]) + q710 - q1114;
    const float m13 = d[7] - d[8] - d[9] + d[10];
    const float m14 = d[15] - d[16] - d[17] + d[18];
    const float m15 = d[11] - d[12] - d[13] + d[14];
    const float m16 = d[7] - d[8] + d[9] - d[10] - d[11] + d[12] - d[13] + d[14];
    const float m17 = -d[7] - d[8] + d[9] + d[10] + d[15] - d[16] + d[17] - d[18];
    const float m18 = d[11] + d[12] - d[13] - d[14] - d[15] - d[16] + d[17] + d[18];

    const float uu = u * u, vv = v * v, ww = w * w, u2 = uu + vv + ww;
    const float e1 = -11.0f * dr + 19.0f * rho * u2;
    const float e2 = 3.0f * dr - 5.5f * rho * u2;
    const float e4 = (-2.0f / 3.0f) * rho * u, e6 = (-2.0f / 3.0f) * rho * v, e8 = (-2.0f / 3.0f) * rho * w;
    const float e9 = rho * (2.0f * uu - vv - ww), e10 = -0.5f * e9;
    const float e11 = rho * (vv - ww), e12 = -0.5f * e11;
    const float e13 = rho * u * v, e14 = rho * v * w, e15 = rho * u * w;
    const float vF = v * Fy;  // u.F with F = (0, Fy, 0)
    const float anu = 1.0f - 0.5f * P.Snu, api = 1.0f - 0.5f * P.Spi;
    const float src1 = (1.0f - 0.5f * P.Se) * 38.0f * vF;
    const float src2 = (1.0f - 0.5f * P.Seps) * (-11.0f) * vF;
    const float src6 = (1.0f - 0.5f * P.Sq) * (-2.0f / 3.0f) * Fy;
    const float src9 = anu * (-2.0f * vF), src10 = api * vF, src11 = anu * (2.0f * vF), src12 = api * (-vF);
    const float src13 = anu * (u * Fy), src14 = anu * (w * Fy);

    const float mp0 = dr;
    const float mp1 = m1 - P.Se * (m1 - e1) + src1;
    const float mp2 = m2 - P.Seps * (m2 - e2) + src2;
    const float mp3 = m3;
    const float mp4 = m4 - P.Sq * (m4 - e4);
    const float mp5 = m5 + Fy;
    const float mp6 = m6 - P.Sq * (m6 - e6) + src6;
    const float mp7 = m7;
    const float mp8 = m8 - P.Sq * (m8 - e8);
    const float mp9 = m9 - P.Snu * (m9 - e9) + src9;
    const float mp10 = m10 - P.Spi * (m10 - e10) + src10;
    const float mp11 = m11 - P.Snu * (m11 - e11) + src11;
    const float mp12 = m12 - P.Spi * (m12 - e12) + src12;
    const float mp13 = m13 - P.Snu * (m13 - e13) + src13;
    const float mp14 = m14 - P.Snu * (m14 - e14) + src14;
    const float mp15 = m15 - P.Snu * (m15 - e15);
    const float mp16 = m16 - P.Sm * m16;
    const float mp17 = m17 - P.Sm * m17;
    const float mp18 = m18 - P.Sm * m18;

    // M^-1 (3DRB.F90:861-943) with the divisions folded into constants
    const float A = mp0 * (1.0f / 19.0f);
    const float B1 = mp1 * (5.0f / 399.0f), B2 = mp1 * (11.0f / 2394.0f), B3 = mp1 * (4.0f / 1197.0f);
    const float C1 = mp2 * (1.0f / 21.0f), C2 = mp2 * (1.0f / 63.0f), C3 = mp2 * (1.0f / 252.0f);
    const float X3 = mp3 * 0.1f, X4 = mp4 * 0.1f, X4b = mp4 * 0.025f;
    const float Y5 = mp5 * 0.1f, Y6 = mp6 * 0.1f, Y6b = mp6 * 0.025f;
    const float Z7 = mp7 * 0.1f, Z8 = mp8 * 0.1f, Z8b = mp8 * 0.025f;
    const float P9a = mp9 * (1.0f / 18.0f), P9b = mp9 * (1.0f / 36.0f);
    const float P10a = mp10 * (1.0f / 18.0f), P10b = mp10 * (1.0f / 36.0f), P10c = mp10 * (1.0f / 72.0f);
    const float P11 = mp11 * (1.0f / 12.0f), P12a = mp12 * (1.0f / 12.0f), P12b = mp12 * (1.0f / 24.0f);
    const float Q13 = mp13 * 0.25f, Q14 = mp14 * 0.25f, Q15 = mp15 * 0.25f;
    const float R16 = mp16 * 0.125f, R17 = mp17 * 0.125f, R18 = mp18 * 0.125f;
    const float ax = A - B2 - C2;
    const float axx = ax + P9a - P10a;
    const float ayz = ax - P9b + P10b;
    const float dgc = A + B3 + C3;
    const float dxy = dgc + P9b + P10c + P11 + P12b;
    const float dxz = dgc + P9b + P10c - P11 - P12b;
    const float dyz = dgc - P9a - P10b;
    dp[0] = A - B1 + C1;
    dp[1] = axx + X3 - X4;
    dp[2] = axx - X3 + X4;
    dp[3] = ayz + Y5 - Y6 + P11 - P12a;
    dp[4] = ayz - Y5 + Y6 + P11 - P12a;
    dp[5] = ayz + Z7 - Z8 - P11 + P12a;
    dp[6] = ayz - Z7 + Z8 - P11 + P12a;
    const float xp = X3 + X4b, yp = Y5 + Y6b, zp = Z7 + Z8b;
    dp[7] = dxy + xp + yp + Q13 + R16 - R17;
    dp[8] = dxy - xp + yp - Q13 - R16 - R17;
    dp[9] = dxy + xp - yp - Q13 + R16 + R17;
    dp[10] = dxy - xp - yp + Q13 - R16 + R17;
    dp[11] = dxz + xp + zp + Q15 - R16 + R18;
    dp[12] = dxz - xp + zp - Q15 + R16 + R18;
    dp[13] = dxz + xp - zp - Q15 - R16 - R18;
    dp[14] = dxz - xp - zp + Q15 + R16 - R18;
    dp[15] = dyz + yp + zp + Q14 + R17 - R18;
    dp[16] = dyz - yp + zp - Q14 - R17 - R18;
    dp[17] = dyz + yp - zp - Q14 + R17 + R18;
    dp[18] = dyz - yp - zp + Q14 - R17 + R18;
}

// D2Q5 thermal MRT with the M1G term (2DRB.F90:921-974), full g in FP32.
__device__ __forceinline__ void fcollideT_2d(const float* G, float u, float v, float T, float& Bx, float& By,
                                             const PhysF& P, float* GP) {
    const float bx = u * T, by = v * T;
    const float dBx = P.use_g ? bx - Bx : 0.0f, dBy = P.use_g ? by - By : 0.0f;
    if (P.use_g) {
        Bx = bx;
        By = by;
    }
    const float n0 = G[0] + G[1] + G[2] + G[3] + G[4];
    const float n1 = G[1] - G[3], n2 = G[2] - G[4];
    const float n3 = -4.0f * G[0] + G[1] + G[2] + G[3] + G[4];
    const float n4 = G[1] - G[2] + G[3] - G[4];
    const float neq3 = P.legacy ? T * P.paraA : T * (-2.0f / 3.0f);
    const float p0 = n0;
    const float p1 = n1 - P.Qk * (n1 - T * u) + P.SG * dBx;
    const float p2 = n2 - P.Qk * (n2 - T * v) + P.SG * dBy;
    const float p3 = n3 - P.Qnu * (n3 - neq3);
    const float p4 = n4 - P.Qnu * n4;
    GP[0] = 0.2f * p0 - 0.2f * p3;
    GP[1] = 0.2f * p0 + 0.5f * p1 + 0.05f * p3 + 0.25f * p4;
    GP[2] = 0.2f * p0 + 0.5f * p2 + 0.05f * p3 - 0.25f * p4;
    GP[3] = 0.2f * p0 - 0.5f * p1 + 0.05f * p3 + 0.25f * p4;
    GP[4] = 0.2f * p0 - 0.5f * p2 + 0.05f * p3 - 0.25f * p4;
}

// D3Q7 thermal MRT with the M1G term (3DRB.F90:1121-1191).
__device__ __forceinline__ void fcollideT_3d(const float* g, float u, float v, float w, float T, float& Bx, float& By,
                                             float& Bz, const PhysF& P, float* gp) {
    const float bx = u * T, by = v * T, bz = w * T;
    const float dBx = P.use_g ? bx - Bx : 0.0f, dBy = P.use_g ? by - By : 0.0f, dBz = P.use_g ? bz - Bz : 0.0f;
    if (P.use_g) {
        Bx = bx;
        By = by;
        Bz = bz;
    }
    const float n0 = g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6];
    const float n1 = g[1] - g[2], n2 = g[3] - g[4], n3 = g[5] - g[6];
    const float n4 = -6.0f * g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6];
    const float n5 = 2.0f * g[1] + 2.0f * g[2] - g[3] - g[4] - g[5] - g[6];
    const float n6 = g[3] + g[4] - g[5] - g[6];
    const float neq4 = P.legacy ? P.paraA * T : -0.75f * T;
    const float p0 = n0;
    const float p1 = n1 - P.Qk * (n1 - bx) + P.SG * dBx;
    const float p2 = n2 - P.Qk * (n2 - by) + P.SG * dBy;
    const float p3 = n3 - P.Qk * (n3 - bz) + P.SG * dBz;
    const float p4 = n4 - P.Qnu * (n4 - neq4);
    const float p5 = n5 - P.Qnu * n5;
    const float p6 = n6 - P.Qnu * n6;
    const float a = p0 * (1.0f / 7.0f), b = p4 * (1.0f / 42.0f);
    gp[0] = a - p4 * (1.0f / 7.0f);
    gp[1] = a + 0.5f * p1 + b + p5 * (1.0f / 6.0f);
    gp[2] = a - 0.5f * p1 + b + p5 * (1.0f / 6.0f);
    const float c = a + b - p5 * (1.0f / 12.0f);
    gp[3] = c + 0.5f * p2 + 0.25f * p6;
    gp[4] = c - 0.5f * p2 + 0.25f * p6;
    gp[5] = c + 0.5f * p3 - 0.25f * p6;
    gp[6] = c - 0.5f * p3 - 0.25f * p6;
}

__device__ __forceinline__ bool fcell(const Geo& g, long long& c, int& i, int& j, int& k) {
    c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncell) return false;
    cell_coords(g, c, i, j, k);
    return true;
}
// The same with the cell index and its divisions in the index type I (int where every
// array index fits in 32 bits).
template <class I>
__device__ __forceinline__ bool fcell_i(const Geo& g, I& c, int& i, int& j, int& k) {
    c = (I)blockIdx.x * (I)blockDim.x + (I)threadIdx.x;
    if (c >= (I)g.ncell) return false;
    const I plane = (I)g.nx * (I)g.ny;
    k = (int)(c / plane);
    const I r = c - (I)k * plane;
    j = (int)(r / (I)g.nx);
    i = (int)(r - (I)j * (I)g.nx);
    return true;
}

// Cell of a thread, x-face cells apart: threads [0, rows*(nx-2)) take the cells with
// 0 < i < nx-1 row by row, the last 2*rows threads the x-face cells (i = 0, nx-1 of each
// row).  A warp then holds either x-interior cells, which take the fixed-offset path
// unless their row lies on a y/z face, or face cells only, where with cells in lattice
// order every warp that holds an x-face cell runs both the fixed-offset and the boundary
// path.  The price is warps that no longer start at a row (one more sector per access).
// The launch is ncell threads, as for fcell.
__device__ __forceinline__ bool split_cell(const Geo& g, long long& c, int& i, int& j, int& k) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long rows = (long long)g.ny * g.nz;
    const int nxi = g.nx - 2;
    const long long nin = rows * nxi;
    long long r;
    if (t < nin) {
        r = t / nxi;
        i = 1 + (int)(t - r * nxi);
    } else {
        const long long f = t - nin;
        if (f >= 2 * rows) return false;
        r = f >> 1;
        i = (f & 1) ? g.nx - 1 : 0;
    }
    j = (int)(r % g.ny);
    k = (int)(r / g.ny);
    c = (long long)i + (long long)g.nx * r;
    return true;
}

template <int QT>
__device__ __forceinline__ float wT(const PhysF& P, int a) {
    return a == 0 ? P.omegaT0 : P.omegaT1;
}

// macro on deviations: rho = 1 + sum d; u = (j + F/2)/rho (3D: F_y from the lagged T)
template <int D>
__device__ __forceinline__ void fmacro(const float* d, float lag, const PhysF& P, float& dr, float& rho, float& u,
                                       float& v, float& w, float& Fy) {
    if (D == 2) {
        dr = d[0] + d[1] + d[2] + d[3] + d[4] + d[5] + d[6] + d[7] + d[8];
        rho = 1.0f + dr;
        Fy = lag;  // force stored by the previous collision (2DRB.F90:719, 888)
        const float inv = 1.0f / rho;
        u = (d[1] - d[3] + d[5] - d[6] - d[7] + d[8]) * inv;
        v = (d[2] - d[4] + d[5] + d[6] - d[7] - d[8] + 0.5f * Fy) * inv;
        w = 0.0f;
    } else {
        float s = 0.0f;
#pragma unroll
        for (int a = 0; a < 19; ++a) s += d[a];
        dr = s;
        rho = 1.0f + dr;
        Fy = rho * P.gBeta * (lag - P.Tref);  // 3DRB.F90:1083
        const float inv = 1.0f / rho;
        u = (d[1] - d[2] + d[7] - d[8] + d[9] - d[10] + d[11] - d[12] + d[13] - d[14]) * inv;
        v = (d[3] - d[4] + d[7] + d[8] - d[9] - d[10] + d[15] - d[16] + d[17] - d[18] + 0.5f * Fy) * inv;
        w = (d[5] - d[6] + d[11] + d[12] - d[13] - d[14] + d[15] + d[16] - d[17] - d[18]) * inv;
    }
}

}  // namespace lbm
