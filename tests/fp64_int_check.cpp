// Host check of csrc/lbm_fp64_int.cuh: the exponent-add products with exact powers of two,
// compiled as plain C++, against the CPU's own IEEE-754 binary64 multiplication (round to
// nearest-even), bit for bit.  NaN results only have to be NaNs.
// Prints "ok <cases>" and exits 0, or lists the first mismatches and exits 1.
#include "lbm_fp64_int.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using namespace lbm::i64f;

static unsigned long long g_fail = 0, g_cases = 0;

static bool same(double a, double b) { return (std::isnan(a) && std::isnan(b)) || bits(a) == bits(b); }

template <int K>
static void check_scale(double x) {
    volatile double v = x;
    volatile double s = std::ldexp(1.0, K);
    const double h = v * s;
    ++g_cases;
    if (!same(h, iscale<K>(x))) {
        if (g_fail++ < 8) std::printf("scale mismatch %a * 2^%d: cpu %a emu %a\n", x, K, h, iscale<K>(x));
    }
}

template <int K>
static void check_all(double x) {
    check_scale<K>(x);
    check_scale<-K>(x);
}

int main() {
    std::mt19937_64 rng(20261203);
    const double special[] = {0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, 4.9e-324, -4.9e-324,
                              2.2250738585072014e-308, -2.2250738585072014e-308, 2.225073858507201e-308,
                              1.7976931348623157e308, -1.7976931348623157e308, 8.98846567431158e307, 0.5, 3.0,
                              1e-300, 1e300, 0.1, 0.3};
    for (double a : special) {
        check_all<1>(a);
        check_all<2>(a);
        check_all<3>(a);
        check_all<60>(a);
    }
    // random bit patterns: every exponent, subnormals, infinities and NaNs
    for (int i = 0; i < 1000000; ++i) {
        const double x = dbl(rng());
        check_all<1>(x);
        check_all<2>(x);
        check_all<3>(x);
    }
    // the edges of the normal range: exponent fields 0..4 and 2043..2047
    for (int i = 0; i < 200000; ++i) {
        const uint64_t e = (i & 1) ? (rng() % 5) : (2043 + rng() % 5);
        const double x = dbl((rng() & ~(0x7FFull << 52)) | (e << 52));
        check_all<1>(x);
        check_all<2>(x);
        check_all<3>(x);
        check_all<60>(x);
    }
    if (g_fail) {
        std::printf("%llu mismatches in %llu cases\n", g_fail, g_cases);
        return 1;
    }
    std::printf("ok %llu\n", g_cases);
    return 0;
}
