// lbm_fp64_int.cuh - binary64 addition and power-of-two scaling on the integer pipes.
//
// GB300's FP64 vector pipe retires 2 thread instructions per clock per SM, while its
// integer and logic pipes retire 64 or more per clock and sit idle in the plain method's
// kernels (FP64-issue bound).  These functions compute IEEE-754 binary64 results, rounded to
// nearest-even, with integer instructions only, so a kernel can move part of its additions
// off the FP64 pipe and still return the same bits.
//
//   iadd(a, b)       a + b   correctly rounded for every finite input (normal, subnormal,
//                            signed zeros, exact cancellation to +0), overflow to +-inf;
//                            inf/NaN inputs give inf/NaN (NaN payloads are not specified).
//   isub(a, b)       a - b = a + (-b) (a sign flip, as IEEE defines subtraction).
//   iscale<K>(x)     x * 2^K, exact whenever the result is normal (an exponent add); a
//                    subnormal or overflowing result takes a rounded slow path.
//
// Method (the textbook alignment / guard-round-sticky addition): order the operands by
// magnitude, place both significands with the hidden bit at bit 62 (10 guard bits below
// the last place), shift the smaller right by the exponent difference with every bit
// shifted out ORed into bit 0, add or subtract, move the leading one to bit 63 (but not
// below the smallest normal exponent: such results are exact subnormals), and round the
// 11 bits below the last place to nearest-even.  A sticky bit kept in bit 0 decides every
// rounding the same way as the exact sum: the jammed value is odd, every rounding boundary
// is even, and the exact value lies strictly between the same two even integers.  The
// round-up carry of the 53-bit significand ripples into the exponent field by plain
// integer addition of the packed word.
//
// The functions are host-callable too; the host build is checked bit for bit against the
// CPU's own binary64 arithmetic.
#pragma once

#include <stdint.h>
#if !defined(__CUDA_ARCH__)
#include <string.h>
#endif

#if defined(__CUDACC__)
#define LBM_I64F_HD __host__ __device__ __forceinline__
#else
#define LBM_I64F_HD inline
#endif

namespace lbm {
namespace i64f {

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kAbs = 0x7FFFFFFFFFFFFFFFull;
constexpr uint64_t kMant = 0x000FFFFFFFFFFFFFull;
constexpr uint64_t kInf = 0x7FF0000000000000ull;
constexpr uint64_t kQuiet = 0x0008000000000000ull;

LBM_I64F_HD uint64_t bits(double x) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
#endif
}

LBM_I64F_HD double dbl(uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, 8);
    return x;
#endif
}

// Number of leading zero bits, 64 for x == 0.
LBM_I64F_HD unsigned clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return (unsigned)__clzll((long long)x);
#else
    return x ? (unsigned)__builtin_clzll(x) : 64u;
#endif
}

// x << n for n in [0, 64] (64 gives 0, as the PTX shift defines it).
LBM_I64F_HD uint64_t shl64(uint64_t x, unsigned n) {
#if defined(__CUDA_ARCH__)
    uint64_t r;
    asm("shl.b64 %0, %1, %2;" : "=l"(r) : "l"(x), "r"(n));
    return r;
#else
    return n >= 64 ? 0 : x << n;
#endif
}

// The sum of two binary64 bit patterns, rounded to nearest-even.
LBM_I64F_HD uint64_t add_bits(uint64_t ua, uint64_t ub) {
    const uint64_t ma = ua & kAbs, mb = ub & kAbs;
    const bool swap = ma < mb;
    const uint64_t x = swap ? ub : ua;  // the operand of larger magnitude carries the sign
    const uint64_t mx = swap ? mb : ma;
    const uint64_t my = swap ? ma : mb;
    const unsigned ex = (unsigned)(mx >> 52), ey = (unsigned)(my >> 52);
    const bool sub = (int64_t)(ua ^ ub) < 0;
    // significands, hidden bit at bit 62; a subnormal has no hidden bit and exponent 1
    const uint64_t fx = ((mx & kMant) | ((uint64_t)(ex != 0) << 52)) << 10;
    const uint64_t fy = ((my & kMant) | ((uint64_t)(ey != 0) << 52)) << 10;
    const unsigned exn = ex + (ex == 0), eyn = ey + (ey == 0);
    unsigned d = exn - eyn;
    d = d < 63 ? d : 63;  // fy < 2^63: a shift by 63 leaves only the sticky bit
    const uint64_t lost = fy & ((1ull << d) - 1);
    const uint64_t ya = (fy >> d) | (uint64_t)(lost != 0);
    const uint64_t r = sub ? fx - ya : fx + ya;
    const unsigned lz = clz64(r);
    const unsigned sh = lz < exn ? lz : exn;  // stop at the subnormal range (exact there)
    const uint64_t n = shl64(r, sh);
    const uint64_t lsb = (n >> 11) & 1;
    const uint64_t up = ((n & 0x7FF) + 0x3FF + lsb) >> 11;
    uint64_t res = (((uint64_t)(exn - sh)) << 52) + (n >> 11) + up;
    res |= x & kSign;
    if (r == 0) res = ua & ub & kSign;  // x - x = +0; (-0) + (-0) = -0
    if (ex >= 2046) {                     // overflow, infinities and NaNs
        if (ex == 2047)
            res = mx > kInf ? (x | kQuiet) : ((sub && my == kInf) ? (kInf | kQuiet) : x);
        else if ((res & kAbs) >= kInf)
            res = (x & kSign) | kInf;
    }
    return res;
}

LBM_I64F_HD double iadd(double a, double b) { return dbl(add_bits(bits(a), bits(b))); }
LBM_I64F_HD double isub(double a, double b) { return dbl(add_bits(bits(a), bits(b) ^ kSign)); }

// x * 2^k when the result is not normal (or x is subnormal): normalise, then round the
// significand shifted into the subnormal range to nearest-even.
LBM_I64F_HD uint64_t scale_slow(uint64_t u, int k) {
    const uint64_t m = u & kAbs;
    const unsigned e = (unsigned)(m >> 52);
    if (m == 0) return u;
    if (e == 2047) return m > kInf ? (u | kQuiet) : u;
    uint64_t f = (m & kMant) | ((uint64_t)(e != 0) << 52);
    const int norm = (int)clz64(f) - 11;  // leading one to bit 52
    f <<= norm;
    const int E = (int)(e + (e == 0)) - norm + k;
    if (E >= 2047) return (u & kSign) | kInf;
    if (E >= 1) return (u & kSign) | ((((uint64_t)(E - 1)) << 52) + f);
    const unsigned s = (unsigned)(1 - E);  // right shift into the subnormal range
    if (s > 54) return u & kSign;
    const uint64_t q = f >> s, rem = f & ((1ull << s) - 1), half = 1ull << (s - 1);
    const uint64_t up = (rem > half || (rem == half && (q & 1))) ? 1 : 0;
    return (u & kSign) | (q + up);
}

template <int K>
LBM_I64F_HD double iscale(double x) {
    static_assert(K >= -64 && K <= 64, "power-of-two scale out of range");
    const uint64_t u = bits(x);
    const unsigned e = (unsigned)(u >> 52) & 0x7FF;
    // normal in, normal out (exponent fields 1..2046 both): add K to the exponent field
    constexpr int lo = K > 0 ? 1 : 1 - K;           // smallest field that stays normal
    constexpr unsigned span = K > 0 ? 2046 - K : 2046 + K;  // fields lo .. lo + span - 1
    if ((unsigned)((int)e - lo) < span) return dbl(u + (uint64_t)((int64_t)K << 52));
    if ((u & kAbs) == 0) return x;
    return dbl(scale_slow(u, K));
}

}  // namespace i64f
}  // namespace lbm
