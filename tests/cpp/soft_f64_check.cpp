// Checks the integer-pipe binary64 division (single and two numerators sharing a
// reciprocal), square root, multiplication and addition
// (shallow-water_gb300/csrc/swe_soft_f64.cuh) bitwise against the host's IEEE
// operations: edge values of every class, random operands over the whole exponent
// range and at physical scales, exact quotients and squares and their neighbours,
// subnormal results including exact rounding ties.  Built with SWE_SOFT_SEED_HOOK the
// FP32 seeds are perturbed by up to 2^-21 relative, well beyond the hardware
// approximations' error, to show the Newton iterations keep their margin.
#include <cinttypes>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <random>
#include <vector>

#include "../../shallow-water_gb300/csrc/swe_soft_f64.cuh"

#if defined(SWE_SOFT_SEED_HOOK)
static std::mt19937_64 g_hook_rng(99);
float swe::sf::swe_soft_seed_hook(float seed) {
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    return (float)((double)seed * (1.0 + std::ldexp(u(g_hook_rng), -21)));
}
#endif

using swe::sf::div_rn;
using swe::sf::add_rn;
using swe::sf::mul_rn;
using swe::sf::sub_rn;
using swe::sf::sqrt_rn;
using swe::x64::bits;
using swe::x64::from_bits;

static long failures = 0, checked = 0;

static bool same(double got, double want) {
    if (std::isnan(want)) return std::isnan(got);
    return bits(got) == bits(want);
}

static void check_div(double x, double y) {
    ++checked;
    const double want = x / y, got = div_rn(x, y);
    if (!same(got, want) && ++failures <= 20)
        std::printf("MISMATCH div(%a, %a): got %a want %a\n", x, y, got, want);
}

static void check_div2(double x1, double x2, double y) {
    checked += 2;
    double q1, q2;
    swe::sf::div2_rn(x1, x2, y, q1, q2);
    if (!same(q1, x1 / y) && ++failures <= 20)
        std::printf("MISMATCH div2(%a, ., %a): got %a want %a\n", x1, y, q1, x1 / y);
    if (!same(q2, x2 / y) && ++failures <= 20)
        std::printf("MISMATCH div2(., %a, %a): got %a want %a\n", x2, y, q2, x2 / y);
}

static void check_mul(double x, double y) {
    ++checked;
    const double want = x * y, got = mul_rn(x, y);
    if (!same(got, want) && ++failures <= 20)
        std::printf("MISMATCH mul(%a, %a): got %a want %a\n", x, y, got, want);
}

static void check_add(double x, double y) {
    checked += 2;
    const double want = x + y, got = add_rn(x, y);
    if (!same(got, want) && ++failures <= 20)
        std::printf("MISMATCH add(%a, %a): got %a want %a\n", x, y, got, want);
    const double wants = x - y, gots = sub_rn(x, y);
    if (!same(gots, wants) && ++failures <= 20)
        std::printf("MISMATCH sub(%a, %a): got %a want %a\n", x, y, gots, wants);
}

static double worst_rsqrt = 0.0;

static void check_sqrt(double x) {
    ++checked;
    const double want = std::sqrt(x), got = sqrt_rn(x);
    if (!same(got, want) && ++failures <= 20)
        std::printf("MISMATCH sqrt(%a): got %a want %a\n", x, got, want);
    if (x > 0.0 && std::isfinite(x)) {
        double s, r;
        swe::sf::sqrt_rsqrt(x, s, r);
        const long double exact = 1.0L / std::sqrt((long double)x);
        const double rel = (double)std::fabs(((long double)r - exact) / exact);
        if (rel > worst_rsqrt) worst_rsqrt = rel;
        if ((!same(s, want) || rel > 0x1p-51) && ++failures <= 20)
            std::printf("MISMATCH sqrt_rsqrt(%a): s %a r %a rel %g\n", x, s, r, rel);
    }
}

int main(int argc, char **argv) {
    const long n = argc > 1 ? std::atol(argv[1]) : 2000000;
    const double dmin = std::numeric_limits<double>::min();
    const double dtrue = std::numeric_limits<double>::denorm_min();
    const double dmax = std::numeric_limits<double>::max();
    const double inf = std::numeric_limits<double>::infinity();
    const double nan = std::numeric_limits<double>::quiet_NaN();
    std::vector<double> edge = {0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 3.0, 0.1, -0.3, 1e-8, 9.80665,
                                1.0000000000000002, 0.9999999999999999, 1.9999999999999998,
                                dmin, -dmin, dtrue, -dtrue, 3 * dtrue, dmin / 3, dmin * 0.75,
                                dmax, -dmax, dmax / 3, 1e300, 1e-300, 1e-320, inf, -inf, nan,
                                -nan, std::ldexp(1.0, -1022), std::ldexp(1.0, 1023),
                                std::ldexp(1.5, -1074 + 52), std::ldexp(1.0, -537)};
    for (double a : edge) {
        check_sqrt(a);
        for (double b : edge) {
            check_div(a, b);
            check_mul(a, b);
            check_add(a, b);
            check_div2(a, b, b);
            check_div2(b, a, a);
        }
    }

    std::mt19937_64 rng(2024);
    std::uniform_real_distribution<double> u(-1.0, 1.0), u1(1.0, 2.0);
    std::uniform_int_distribution<int> ex(-60, 60), bigex(-1080, 1030);
    std::uniform_int_distribution<uint64_t> raw;
    std::uniform_int_distribution<int64_t> m26(1, (1LL << 26) - 1), m27(1, (1LL << 27) - 1);
    for (long i = 0; i < n; ++i) {
        // physical scales and shared exponents
        const double a = std::ldexp(u(rng), ex(rng)), b = std::ldexp(u(rng), ex(rng));
        check_div(a, b);
        check_mul(a, b);
        check_add(a, b);
        check_add(a, a * (1.0 + 1e-12 * u(rng)));
        check_add(a, -a * (1.0 + 1e-15 * u(rng)));
        check_mul(9.80665, std::fabs(b));
        check_div(1.0, b);
        check_div(a, a * (1.0 + 1e-15 * u(rng)));
        check_sqrt(std::fabs(a));
        check_sqrt(9.80665 * std::fabs(b));
        // whole exponent range, raw patterns (subnormal, huge, NaN payloads, signs)
        const double r1 = from_bits((int64_t)raw(rng)), r2 = from_bits((int64_t)raw(rng));
        check_div(r1, r2);
        check_div2(r1, a, r2);
        check_div2(a, b, std::fabs(r1));
        check_mul(r1, r2);
        check_add(r1, r2);
        check_sqrt(r1);
        check_sqrt(std::fabs(r2));
        const double s1 = std::ldexp(u1(rng), bigex(rng)), s2 = std::ldexp(u1(rng), bigex(rng));
        check_div(s1, s2);
        check_div(-s1, s2);
        check_mul(s1, -s2);
        check_add(s1, -s2);
        check_add(s1, std::ldexp(s2, -(int)(i % 70)));
        check_sqrt(s1);
        // exact quotients q = x / y with short significands, and their neighbours
        const double q = std::ldexp((double)m26(rng), ex(rng) - 26);
        const double y = std::ldexp((double)m27(rng), ex(rng) - 27);
        const double x = q * y;  // exact: 26 + 27 bits
        check_div(x, y);
        check_div2(x, std::nextafter(x, -inf), y);
        check_div(std::nextafter(x, inf), y);
        check_div(std::nextafter(x, -inf), y);
        check_div(x, std::nextafter(y, inf));
        // products of 27-bit significands: 53 or 54 bits, exact ties included
        const double p1 = std::ldexp((double)m27(rng), ex(rng) - 27);
        const double p2 = std::ldexp((double)(m27(rng) | 1), ex(rng) - 27);
        check_mul(p1, p2);
        check_mul(std::nextafter(p1, inf), p2);
        check_mul(q, y);
        // sums whose exact value lands on or next to a rounding tie
        check_add(std::ldexp(1.0, ex(rng)), std::ldexp(p1, -60 + (int)(i % 60)));
        check_add(x, std::ldexp(y, -53));
        check_add(-x, std::ldexp(y, -54));
        // exact squares and neighbours
        const double sq = q * q;
        check_sqrt(sq);
        check_sqrt(std::nextafter(sq, inf));
        check_sqrt(std::nextafter(sq, 0.0));
        // subnormal quotients, including exact ties between subnormals
        const int64_t k = (int64_t)(raw(rng) >> 40);
        const double sub = from_bits(k);
        check_div(sub, 2.0);
        check_div(sub, 4.0);
        check_div(sub * 3.0 > 0 ? std::ldexp((double)(2 * (k & 0xFFFF) + 1), -1074) : sub, 2.0);
        check_div(std::ldexp(u1(rng), -1000), std::ldexp(u1(rng), 60));
        check_div(std::ldexp(u1(rng), 1000), std::ldexp(u1(rng), -30));
        // subnormal and overflowing products, ties between subnormals
        check_mul(sub, 0.5);
        check_mul(sub, 3.0);
        check_mul(std::ldexp(u1(rng), -540), std::ldexp(u1(rng), -520));
        check_mul(std::ldexp(u1(rng), -1020), std::ldexp(u1(rng), -30));
        check_mul(std::ldexp(u1(rng), 520), std::ldexp(u1(rng), 505));
        check_mul(std::ldexp((double)(m27(rng) | 1), -1074), std::ldexp(1.0, -27));
        check_add(sub, from_bits((int64_t)(raw(rng) >> 12)));
        check_add(sub, -from_bits((int64_t)(raw(rng) >> 11)));
        check_add(std::ldexp(u1(rng), 1023), std::ldexp(u1(rng), 1023));
    }
    std::printf("worst 1/sqrt relative error %.3g\n", worst_rsqrt);
    std::printf("checked %ld operations, %ld mismatches\n", checked, failures);
    return failures ? 1 : 0;
}
