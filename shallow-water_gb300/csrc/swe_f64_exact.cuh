// Bit-exact FP64 helpers that run on the integer pipe.
//
// GB300 issues FP64 at about 1/64 of its FP32 rate, so every FP64 instruction the
// stencil avoids is time saved.  Each helper below returns exactly the IEEE-754
// result of the expression it replaces (the comments name it), for every input
// including signed zeros, subnormals, infinities and NaN, by working on the bit
// patterns; only rare operands (zeros, subnormals, huge or tiny magnitudes) fall
// back to the plain FP64 expression.  Compiled for host and device so the CPU tests
// can check them against the plain expressions.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define SWE_HD __host__ __device__ __forceinline__
// Rare-operand fallbacks are out of line on the device: inlined, the compiler may
// if-convert them and issue their FP64 instructions for every lane on every call.
#define SWE_COLD static __host__ __device__ __noinline__
#else
#define SWE_HD inline
#define SWE_COLD static inline
#endif

namespace swe {
namespace x64 {

constexpr int64_t SIGN = INT64_MIN;
constexpr int64_t ABS = INT64_MAX;
constexpr int64_t INF_BITS = 0x7FF0000000000000LL;
constexpr int64_t MANT = 0x000FFFFFFFFFFFFFLL;

// On the device the casts are opaque moves: seen through, the compiler folds bit tests
// and sign splices back into FP64 compares, abs, neg and copysign, which run on the
// scarce FP64 pipe.
SWE_HD int64_t bits(double x) {
#if defined(__CUDA_ARCH__)
    int64_t b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return b;
#else
    int64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

SWE_HD double from_bits(int64_t b) {
#if defined(__CUDA_ARCH__)
    double x;
    asm("mov.b64 %0, %1;" : "=d"(x) : "l"(b));
    return x;
#else
    double x;
    std::memcpy(&x, &b, sizeof x);
    return x;
#endif
}

SWE_HD double fma_rn(double a, double b, double c) {
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return __builtin_fma(a, b, c);
#endif
}

SWE_HD bool is_nan(int64_t b) { return (b & ABS) > INF_BITS; }

// Total-order key of a non-NaN double with -0 and +0 mapped together.
SWE_HD int64_t key(int64_t b) { return b >= 0 ? b : (SIGN - b); }

// IEEE a < b (false if either is NaN; -0 == +0).
SWE_HD bool lt(double a, double b) {
    const int64_t ba = bits(a), bb = bits(b);
    if (is_nan(ba) || is_nan(bb)) return false;
    return key(ba) < key(bb);
}

// IEEE a <= b.
SWE_HD bool le(double a, double b) {
    const int64_t ba = bits(a), bb = bits(b);
    if (is_nan(ba) || is_nan(bb)) return false;
    return key(ba) <= key(bb);
}

// std::min(a, b) == (b < a) ? b : a
SWE_HD double dmin(double a, double b) { return lt(b, a) ? b : a; }
// std::max(a, b) == (a < b) ? b : a
SWE_HD double dmax(double a, double b) { return lt(a, b) ? b : a; }

// x > 0.0 ? x : 0.0   (positive_height, HPC_kernels.hpp:33-35)
SWE_HD double positive_part(double x) {
    const int64_t b = bits(x);
    return (b > 0 && b <= INF_BITS) ? x : 0.0;
}

SWE_COLD double mul_cold(double a, double b) { return a * b; }
SWE_COLD double div_cold(double a, double b) { return a / b; }

// 0.5 * x, on the bit pattern for every input: exponent decrement for normal results;
// for |x| below 2^-1021 the magnitude bits are proportional to the value, so halving is
// a right shift rounded half to even; infinities and NaN are returned (NaN quietened).
SWE_HD double halve(double x) {
    const int64_t b = bits(x);
    const int64_t e = (b >> 52) & 0x7FF;
    if (e > 1 && e < 0x7FF) return from_bits(b - (1LL << 52));
    const int64_t mag = b & ABS;
    if (e == 0x7FF) return from_bits(mag > INF_BITS ? (b | (1LL << 51)) : b);
    const int64_t h = (mag >> 1) + (mag & (mag >> 1) & 1);
    return from_bits((b & SIGN) | h);
}

// x * 2^k for |k| small, exact when the result stays normal; else the FP64 product
// with the precomputed power of two p2k (= 2^k).
SWE_HD double scale2(double x, int k, double p2k) {
    const int64_t b = bits(x);
    const int64_t e = (b >> 52) & 0x7FF;
    const int64_t en = e + k;
    if (e > 0 && e < 0x7FF && en > 0 && en < 0x7FF) return from_bits(b + ((int64_t)k << 52));
    if ((b & ABS) == 0) return x;  // +-0 * 2^k
    return mul_cold(x, p2k);
}

SWE_HD double fabs_(double x) { return from_bits(bits(x) & ABS); }
SWE_HD double neg(double x) { return from_bits(bits(x) ^ SIGN); }

// Plain minmod (HPC_kernels.hpp:41-44), the fallback.
SWE_COLD double minmod_plain(double a, double b) {
    if (a * b <= 0.0) return 0.0;
    const double fa = fabs_(a), fb = fabs_(b);
    return (a > 0.0 ? 1.0 : -1.0) * ((fb < fa) ? fb : fa);
}

// minmod(a, b) (HPC_kernels.hpp:41-44): a*b <= 0 ? 0 : sign(a) * min(|a|, |b|).
SWE_HD double minmod(double a, double b) {
    const int64_t ba = bits(a), bb = bits(b);
    const int64_t ma = ba & ABS, mb = bb & ABS;
    // |a|, |b| >= 2^-537 keeps a*b above the underflow-to-zero threshold 2^-1075.
    constexpr int64_t TINY = (int64_t)(1023 - 537) << 52;
    if (ma >= INF_BITS || mb >= INF_BITS) return minmod_plain(a, b);
    if (ma == 0 || mb == 0) return 0.0;
    if ((ba ^ bb) < 0) return 0.0;
    if (ma < TINY || mb < TINY) return minmod_plain(a, b);
    // std::min(|a|, |b|) returns |a| on ties; equal magnitudes give equal bits anyway.
    const int64_t m = mb < ma ? mb : ma;
    return from_bits(m | (ba & SIGN));
}

// (h > eps) where eps is a positive normal constant (safe_velocity's guard).
SWE_HD bool gt_pos_const(double h, int64_t eps_bits) {
    const int64_t b = bits(h);
    return b > eps_bits && b <= INF_BITS;
}

// RN(P / H) where P = RN(H * q) and H > 0: the reference's (h * u) / h
// (huL / hL in hll_x, HPC_kernels.hpp:49-52, after huL = hs * u at :165-169).
// The quotient is within one ulp of q, so it is q or a neighbour of q; the exact
// residual e = H*q - P (one FMA) decides which by comparing |e| with H times half the
// gap to that neighbour, an exact power-of-two scaling.  Ties round to even.
SWE_HD double redivide(double P, double H, double q) {
    const int64_t bq = bits(q), bH = bits(H);
    const int64_t eq = (bq >> 52) & 0x7FF, eH = (bH >> 52) & 0x7FF;
    if ((bq & ABS) == 0) {
        if (eH > 0 && eH < 0x7FF && bH > 0) return q;  // P = +-0, H > 0: P / H = q
        return div_cold(P, H);
    }
    // Range that keeps H*q, the residual and the threshold normal and exact.
    if (eq < 123 || eq > 1923 || eH < 1 || eH > 1923 || bH < 0 || eH + eq > 3046)
        return div_cold(P, H);
    const double e = fma_rn(H, q, -P);
    const int64_t be = bits(e);
    if ((be & ABS) == 0) return q;
    const bool up = (be ^ bq) < 0;  // P/H - q = -e/H has the sign of q: |P/H| > |q|
    // half the gap from q to its neighbour in the rounding direction
    const int64_t shift = (eq - 1076) - ((!up && (bq & MANT) == 0) ? 1 : 0);
    const int64_t thr = bH + (shift << 52);  // H * 2^shift, exact
    const int64_t ae = be & ABS;
    const double qn = from_bits(up ? bq + 1 : bq - 1);
    if (ae < thr) return q;
    if (ae > thr) return qn;
    return (bq & 1) ? qn : q;
}

}  // namespace x64
}  // namespace swe
