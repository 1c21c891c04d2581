// Checks the integer-pipe FP64 helpers (shallow-water_gb300/csrc/swe_f64_exact.cuh)
// bitwise against the plain IEEE expressions they replace, on edge values and on
// random operands.  Built and run by tests/test_exact_helpers.py on the CPU; the
// same helpers are compiled into the device code.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <limits>
#include <random>
#include <vector>

#include "../../shallow-water_gb300/csrc/swe_f64_exact.cuh"

using namespace swe::x64;

static long failures = 0;
static bool same(double a, double b) { return bits(a) == bits(b); }
static void report(const char *what, double x, double y, double got, double want) {
    if (++failures <= 20)
        std::printf("MISMATCH %s(%a, %a): got %a want %a\n", what, x, y, got, want);
}

static double ref_positive(double h) { return h > 0.0 ? h : 0.0; }
static double ref_min(double a, double b) { return (b < a) ? b : a; }
static double ref_max(double a, double b) { return (a < b) ? b : a; }

static void check_pair(double a, double b) {
    if (!same(minmod(a, b), minmod_plain(a, b))) report("minmod", a, b, minmod(a, b), minmod_plain(a, b));
    if (!same(dmin(a, b), ref_min(a, b))) report("dmin", a, b, dmin(a, b), ref_min(a, b));
    if (!same(dmax(a, b), ref_max(a, b))) report("dmax", a, b, dmax(a, b), ref_max(a, b));
    if (lt(a, b) != (a < b)) report("lt", a, b, lt(a, b), a < b);
    if (le(a, b) != (a <= b)) report("le", a, b, le(a, b), a <= b);
}

static void check_single(double x) {
    if (!same(positive_part(x), ref_positive(x))) report("positive_part", x, 0, positive_part(x), ref_positive(x));
    if (!same(halve(x), 0.5 * x)) report("halve", x, 0, halve(x), 0.5 * x);
    const double eps = 1e-8;
    if (gt_pos_const(x, bits(eps)) != (x > eps)) report("gt_pos_const", x, eps, gt_pos_const(x, bits(eps)), x > eps);
    for (int k : {-13, -1, 1, 2, 13}) {
        const double p = std::ldexp(1.0, k);
        if (!same(scale2(x, k, p), x * p)) report("scale2", x, p, scale2(x, k, p), x * p);
    }
}

static void check_redivide(double H, double q) {
    if (!(H > 1e-8)) return;  // only called behind safe_velocity's guard
    const double P = H * q;
    const double want = P / H, got = redivide(P, H, q);
    if (!same(got, want)) report("redivide", H, q, got, want);
}

int main(int argc, char **argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
    std::vector<double> edge = {0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 1e-8, -1e-8, 1.0000000000000002,
                                0.9999999999999999, std::numeric_limits<double>::min(),
                                -std::numeric_limits<double>::min(),
                                std::numeric_limits<double>::denorm_min(),
                                -std::numeric_limits<double>::denorm_min(), 1e-300, -1e-300,
                                1e-162, 1e-161, std::ldexp(1.0, -537), std::ldexp(1.0, -538),
                                1e300, -1e300, std::numeric_limits<double>::max(),
                                std::numeric_limits<double>::infinity(),
                                -std::numeric_limits<double>::infinity(),
                                std::numeric_limits<double>::quiet_NaN(),
                                -std::numeric_limits<double>::quiet_NaN(), 3.0, 0.1, -0.3};
    for (double a : edge) {
        check_single(a);
        for (double b : edge) {
            check_pair(a, b);
            check_redivide(std::fabs(a), b);
        }
    }
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    std::uniform_int_distribution<int> ex(-60, 60), bigex(-1074, 1023);
    std::uniform_int_distribution<uint64_t> raw;
    for (long i = 0; i < n; ++i) {
        // physical-scale values, values sharing exponents, raw bit patterns
        const double a = std::ldexp(u(rng), ex(rng));
        const double b = (i & 3) == 0 ? a * (1.0 + 1e-15 * u(rng)) : std::ldexp(u(rng), ex(rng));
        check_single(a);
        check_pair(a, b);
        check_redivide(std::fabs(std::ldexp(u(rng), ex(rng) / 4)) + 1e-8, std::ldexp(u(rng), ex(rng)));
        // powers of two and near-ties for the redivide rounding logic
        check_redivide(1.0 + std::fabs(u(rng)), std::ldexp(1.0, ex(rng)) * ((i & 1) ? 1 : -1));
        const double r1 = from_bits((int64_t)(raw(rng) >> 1) * ((i & 1) ? 1 : -1));
        const double r2 = from_bits((int64_t)raw(rng));
        check_single(r1);
        check_pair(r1, r2);
        check_redivide(std::fabs(r2), r1);
        check_redivide(std::ldexp(1.0 + std::fabs(u(rng)), ex(rng) / 3), std::ldexp(u(rng), bigex(rng)));
    }
    // Near-ties of redivide: small-integer H times short-mantissa q round P = H*q onto
    // exact midpoints of q's neighbours.
    long ties = 0;
    std::uniform_int_distribution<int64_t> kdist(1, (1LL << 53) - 1), sh(0, 52);
    for (long i = 0; i < n; ++i) {
        const double H = std::ldexp((double)(3 + 2 * (i % 40)), (int)(i % 7) - 3);
        const int64_t k = kdist(rng) >> sh(rng) | 1;
        const double q = std::ldexp((double)k, ex(rng) - 52) * ((i & 1) ? -1 : 1);
        const double P = H * q;
        if (std::fabs(std::fma(H, q, -P)) > 0) ++ties;
        check_redivide(H, q);
        check_redivide(H, std::nextafter(q, 0.0));
        check_redivide(H, std::ldexp(1.0, ex(rng)));
    }
    std::printf("checked %ld random rounds (%ld inexact products near ties), %ld mismatches\n",
                n, ties, failures);
    return failures ? 1 : 0;
}
