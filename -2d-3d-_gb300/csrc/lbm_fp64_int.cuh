// lbm_fp64_int.cuh - binary64 products with exact powers of two on the integer pipes.
//
// GB300's FP64 vector pipe retires 2 thread instructions per clock per SM and bounds the
// plain method's kernels, while the integer pipes sit mostly idle beside it.  A product
// with an exact power of two, x * 2^K, is an add to the exponent field whenever input and
// result are normal numbers: the same bits as the FP64 multiply, a handful of integer
// instructions that overlap with the FP64 work.
//
//   iscale<K>(x)     x * 2^K rounded to nearest-even for every input: the exponent add for
//                    normal results, zero unchanged, and a rounded slow path (a real branch,
//                    taken only by subnormal inputs or results, overflow, inf and NaN).
//
// (An IEEE addition in integer arithmetic was measured as well: exact, but on GB300 it
// competes with the FP64 pipe instead of adding to it, so additions stay on the FP64 pipe.)
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
