// Host check of csrc/lbm_fp64_int.cuh: the integer-pipe binary64 addition and the
// power-of-two scaling, compiled as plain C++, against the CPU's own IEEE-754 binary64
// arithmetic (round to nearest-even), bit for bit.  NaN results only have to be NaNs.
// Prints "ok <cases>" and exits 0, or lists the first mismatches and exits 1.
#include "lbm_fp64_int.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using namespace lbm::i64f;

static unsigned long long g_fail = 0, g_cases = 0;

static bool same(double a, double b) { return (std::isnan(a) && std::isnan(b)) || bits(a) == bits(b); }

static void check_add(double a, double b) {
    volatile double va = a, vb = b;
    const double h = va + vb, hs = va - vb;
    ++g_cases;
    if (!same(h, iadd(a, b)) || !same(hs, isub(a, b))) {
        if (g_fail++ < 8) std::printf("add mismatch %a %a: cpu %a emu %a\n", a, b, h, iadd(a, b));
    }
}

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

int main() {
    std::mt19937_64 rng(20261203);
    const double special[] = {0.0, -0.0, 1.0, -1.0, INFINITY, -INFINITY, NAN, 4.9e-324, -4.9e-324,
                              2.2250738585072014e-308, -2.2250738585072014e-308, 2.225073858507201e-308,
                              1.7976931348623157e308, -1.7976931348623157e308, 0.5, 3.0, 1e-300, 1e300, 0.1, 0.3};
    for (double a : special)
        for (double b : special) check_add(a, b);
    for (double a : special) {
        check_scale<1>(a);
        check_scale<-1>(a);
        check_scale<3>(a);
        check_scale<-3>(a);
    }
    // random bit patterns
    for (int i = 0; i < 2000000; ++i) check_add(dbl(rng()), dbl(rng()));
    // exponents within 35 binades; every other pair shares leading significand bits
    for (int i = 0; i < 4000000; ++i) {
        const uint64_t a = rng();
        uint64_t b = rng();
        long long eb = (long long)((a >> 52) & 0x7FF) + (long long)(rng() % 70) - 35;
        eb = eb < 0 ? 0 : (eb > 2046 ? 2046 : eb);
        b = (b & ~(0x7FFull << 52)) | ((uint64_t)eb << 52);
        if (i & 1) b = (b & ~kMant) | ((a & kMant) ^ (rng() & ((1ull << (rng() % 53)) - 1)));
        check_add(dbl(a), dbl(b));
    }
    // lattice-Boltzmann magnitudes: moments and populations in [-40, 40], short significands
    // (ties), near-cancelling pairs, pairs far apart in exponent
    std::uniform_real_distribution<double> U(-40.0, 40.0);
    for (int i = 0; i < 2000000; ++i) {
        const double a = U(rng);
        double b = U(rng);
        if (i % 3 == 0) b = std::ldexp(std::floor(std::ldexp(b, 20)), -20);
        if (i % 5 == 0) b = -a + std::ldexp(U(rng), -40);
        if (i % 7 == 0) b = std::ldexp(a, -(int)(rng() % 60));
        check_add(a, b);
        check_add(b, a);
    }
    // subnormal inputs and results; near overflow
    for (int i = 0; i < 1000000; ++i) check_add(dbl(rng() & ~(0x7C0ull << 52)), dbl(rng() & ~(0x7C0ull << 52)));
    for (int i = 0; i < 200000; ++i) {
        const uint64_t a = (rng() & ~(0x7FFull << 52)) | ((uint64_t)(2040 + rng() % 7) << 52);
        const uint64_t b = (rng() & ~(0x7FFull << 52)) | ((uint64_t)(2030 + rng() % 17) << 52);
        check_add(dbl(a), dbl(b));
    }
    for (int i = 0; i < 1000000; ++i) {
        const double x = dbl(rng());
        check_scale<1>(x);
        check_scale<2>(x);
        check_scale<3>(x);
        check_scale<-1>(x);
        check_scale<-2>(x);
        check_scale<-3>(x);
        check_scale<-60>(x);
    }
    if (g_fail) {
        std::printf("%llu mismatches in %llu cases\n", g_fail, g_cases);
        return 1;
    }
    std::printf("ok %llu\n", g_cases);
    return 0;
}
