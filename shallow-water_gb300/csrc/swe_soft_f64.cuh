// Correctly rounded IEEE-754 binary64 division, square root, multiplication and
// addition on the integer pipes.
//
// GB300 executes FP64 at 2 lane-operations per clock per SM, and a double division or
// square root expands into about twenty FP64-pipe slots there; a few of them per
// interface dominate the FP64 stage kernel.  The integer and FP32 pipes are idle by
// comparison (64-128 lanes per clock), so these routines compute the same
// round-to-nearest-even results from the operands' bit patterns with 64-bit integer
// arithmetic and no FP64 instruction:
//
//   * an FP32 hardware approximation (rcp / rsqrt, relative error near 2^-23) seeds
//     two Newton-Raphson iterations in 64-bit fixed point (y <- y (2 - d y) for 1/d,
//     y <- y (3 - m y^2) / 2 for 1/sqrt(m)), which leaves a relative error near 2^-59
//     (truncation of the fixed-point products), so the quotient or root derived from
//     them is within one unit of the exact truncated result;
//   * the exact remainder (x 2^52 - Q d, or M - S^2) is formed modulo 2^64, which is
//     exact because it is known to be small, corrects that unit, and decides the
//     rounding: round half to even against the divisor for the quotient, and
//     R > S for the root (an exact square-root tie cannot occur);
//   * the product's 106-bit significand comes from four 32x32->64 multiply-adds (the
//     FMA pipe's IMAD.WIDE), then is normalised and rounded half to even;
//   * the sum aligns the smaller operand with ten guard bits and a sticky bit,
//     adds or subtracts, renormalises and rounds half to even; subnormal operands and
//     results take the same path (exponent 1, no hidden bit).
//
// Zeros, subnormals, infinities and NaN operands take a rare branch that follows the
// IEEE-754 rules directly (subnormal operands are normalised, subnormal quotients are
// rounded once at their own precision).  NaN results are the default quiet NaN.
// Compiled for host and device so the CPU tests compare every result bitwise with the
// host's IEEE division, square root and multiplication.
#pragma once

#include <cstdint>
#include <cstring>

#include "swe_f64_exact.cuh"

namespace swe {
namespace sf {

using u64 = unsigned long long;
using i64 = long long;
using u32 = unsigned int;

constexpr u64 SIGN_BIT = 0x8000000000000000ull;
constexpr u64 MANT_BITS = 0x000FFFFFFFFFFFFFull;
constexpr u64 HIDDEN = 0x0010000000000000ull;
constexpr u64 INF = 0x7FF0000000000000ull;
constexpr u64 QNAN = 0x7FF8000000000000ull;

SWE_HD u64 ubits(double x) { return (u64)x64::bits(x); }
SWE_HD double ufrom(u64 b) { return x64::from_bits((int64_t)b); }

SWE_HD u64 umulhi(u64 a, u64 b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (u64)(((unsigned __int128)a * b) >> 64);
#endif
}

SWE_HD int clz64(u64 x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

SWE_HD float f_from(u32 b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float f;
    std::memcpy(&f, &b, sizeof f);
    return f;
#endif
}

SWE_HD u32 f_bits(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    u32 b;
    std::memcpy(&b, &f, sizeof b);
    return b;
#endif
}

#if !defined(__CUDA_ARCH__) && defined(SWE_SOFT_SEED_HOOK)
// CPU tests only: perturbs the FP32 seeds to probe the Newton iterations' margin.
float swe_soft_seed_hook(float seed);
#define SWE_SOFT_SEED(x) swe_soft_seed_hook(x)
#else
#define SWE_SOFT_SEED(x) (x)
#endif

// Approximate 1/f and 1/sqrt(f) for f in [1, 4], relative error well below 2^-20.
SWE_HD float rcp_seed(float f) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
    return r;
#else
    return SWE_SOFT_SEED(1.0f / f);
#endif
}

SWE_HD float rsqrt_seed(float f) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(f));
    return r;
#else
    return SWE_SOFT_SEED(1.0f / __builtin_sqrtf(f));
#endif
}

// A float r in (1/2, 1] as the fixed-point integer r * 2^63.
SWE_HD u64 seed_q63(float r) {
    const u32 b = f_bits(r);
    const int e = (int)(b >> 23) - 127;  // -1 or 0
    return (u64)((b & 0x7FFFFFu) | 0x800000u) << (40 + e);
}

// Rounds sign * m * 2^(e - 1085) to binary64, m having its leading one at bit 62 and a
// sticky bit in bit 0 (e is the biased exponent of a normal result).  Overflow gives
// infinity, tiny values round once to a subnormal or zero.
SWE_HD double round_pack(u64 sign, int e, u64 m) {
    if (e >= 0x7FF) return ufrom(sign | INF);
    if (e < 1) {
        const int sh = 1 - e;
        m = sh < 63 ? ((m >> sh) | (u64)((m << (64 - sh)) != 0)) : (u64)(m != 0);
        const u64 r = m & 0x3FF, q = m >> 10;
        const u64 qr = q + (u64)((r > 0x200) | ((r == 0x200) & (q & 1)));
        return ufrom(sign | qr);  // a carry into bit 52 gives the smallest normal
    }
    const u64 r = m & 0x3FF, q = m >> 10;
    const u64 qr = q + (u64)((r > 0x200) | ((r == 0x200) & (q & 1)));
    return ufrom(sign | (((u64)(e - 1) << 52) + qr));
}

// Significand of a finite nonzero operand as an integer in [2^52, 2^53) and its
// exponent (the biased exponent, <= 0 for subnormals after normalisation).
SWE_HD u64 unpack_normalised(u64 b, int &e) {
    const int be = (int)((b >> 52) & 0x7FF);
    u64 m = b & MANT_BITS;
    if (be != 0) {
        e = be;
        return m | HIDDEN;
    }
    const int lz = clz64(m) - 11;
    e = 1 - lz;
    return m << lz;
}

// Y ~ 2^63 / d for the significand my (d = my / 2^52 in [1, 2)): an FP32 seed and two
// fixed-point Newton steps, relative error about 2^-59.
SWE_HD u64 recip_q63(u64 my) {
    const float f = f_from(0x3F800000u | (u32)((my >> 29) & 0x7FFFFFu));
    u64 Y = seed_q63(rcp_seed(f));
    const u64 D = my << 11;  // d * 2^63
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const i64 E = (i64)((1ull << 62) - umulhi(D, Y));  // 2^62 (1 - d y)
        Y = E >= 0 ? Y + (umulhi(Y, (u64)E) << 2) : Y - (umulhi(Y, (u64)(-E)) << 2);
    }
    return Y;
}

// The correctly rounded quotient of significands mx / my (both in [2^52, 2^53)) with
// exponent e = ex - ey + 1023 and sign, given Y = recip_q63(my).
SWE_HD double quotient(u64 sign, int e, u64 mx, u64 my, u64 Y) {
    if (mx < my) {  // quotient significand in [1, 2)
        mx <<= 1;
        e -= 1;
    }
    // Q = floor(mx 2^52 / my) to within one unit
    u64 Q = umulhi(mx << 10, Y) >> 9;
    i64 R = (i64)((mx << 52) - Q * my);  // exact: -my < R < 2 my
    if (R < 0) {
        Q -= 1;
        R += (i64)my;
    } else if (R >= (i64)my) {
        Q += 1;
        R -= (i64)my;
    }
    if (e >= 1 && e <= 0x7FE) {
        const u64 R2 = (u64)R << 1;
        Q += (u64)((R2 > my) | ((R2 == my) & (Q & 1)));
        return ufrom(sign | (((u64)(e - 1) << 52) + Q));
    }
    return round_pack(sign, e, (Q << 10) | (u64)(R != 0));
}

SWE_COLD double div_special(double x, double y);

// x / y for a normal y and an x that is zero, subnormal, infinite or NaN: zero
// numerators (frequent: fluid at rest) inline, the rest out of line.
SWE_HD double div_by_normal_special(double x, double y) {
    const u64 bx = ubits(x);
    return (bx & ~SIGN_BIT) == 0 ? ufrom((bx ^ ubits(y)) & SIGN_BIT) : div_special(x, y);
}

// x / y, round to nearest even.
SWE_HD double div_rn(double x, double y) {
    const u64 bx = ubits(x), by = ubits(y);
    const u64 ax = bx & ~SIGN_BIT, ay = by & ~SIGN_BIT;
    if (ay - HIDDEN >= INF - HIDDEN) return div_special(x, y);
    if (ax - HIDDEN >= INF - HIDDEN) return div_by_normal_special(x, y);
    const u64 my = (ay & MANT_BITS) | HIDDEN;
    return quotient((bx ^ by) & SIGN_BIT, (int)(ax >> 52) - (int)(ay >> 52) + 1023,
                    (ax & MANT_BITS) | HIDDEN, my, recip_q63(my));
}

// x1 / y and x2 / y, each round to nearest even, sharing the reciprocal of y.
SWE_HD void div2_rn(double x1, double x2, double y, double &q1, double &q2) {
    const u64 b1 = ubits(x1), b2 = ubits(x2), by = ubits(y);
    const u64 a1 = b1 & ~SIGN_BIT, a2 = b2 & ~SIGN_BIT, ay = by & ~SIGN_BIT;
    if (ay - HIDDEN >= INF - HIDDEN) {
        q1 = div_special(x1, y);
        q2 = div_special(x2, y);
        return;
    }
    const u64 my = (ay & MANT_BITS) | HIDDEN;
    const u64 Y = recip_q63(my);
    const int ey = (int)(ay >> 52);
    q1 = a1 - HIDDEN >= INF - HIDDEN
             ? div_by_normal_special(x1, y)
             : quotient((b1 ^ by) & SIGN_BIT, (int)(a1 >> 52) - ey + 1023,
                        (a1 & MANT_BITS) | HIDDEN, my, Y);
    q2 = a2 - HIDDEN >= INF - HIDDEN
             ? div_by_normal_special(x2, y)
             : quotient((b2 ^ by) & SIGN_BIT, (int)(a2 >> 52) - ey + 1023,
                        (a2 & MANT_BITS) | HIDDEN, my, Y);
}

// Some operand zero, subnormal, infinite or NaN.
SWE_COLD double div_special(double x, double y) {
    const u64 bx = ubits(x), by = ubits(y);
    const u64 sign = (bx ^ by) & SIGN_BIT;
    const u64 ax = bx & ~SIGN_BIT, ay = by & ~SIGN_BIT;
    if (ax > INF || ay > INF) return ufrom(QNAN);
    if (ax == INF) return ufrom(ay == INF ? QNAN : (sign | INF));
    if (ay == INF) return ufrom(sign);
    if (ay == 0) return ufrom(ax == 0 ? QNAN : (sign | INF));
    if (ax == 0) return ufrom(sign);
    int ex, ey;
    const u64 mx = unpack_normalised(ax, ex), my = unpack_normalised(ay, ey);
    return quotient(sign, ex - ey + 1023, mx, my, recip_q63(my));
}

// sqrt(x), round to nearest even.
SWE_HD double sqrt_rn(double x) {
    const u64 bx = ubits(x);
    u64 mx;
    int ex;
    if (bx - HIDDEN >= INF - HIDDEN) {
        // zero, subnormal, infinity, NaN or negative
        if ((bx & ~SIGN_BIT) == 0) return x;  // +-0
        if (bx > INF) return ufrom(QNAN);     // NaN or negative
        if (bx == INF) return x;
        mx = unpack_normalised(bx, ex);
    } else {
        ex = (int)(bx >> 52);
        mx = (bx & MANT_BITS) | HIDDEN;
    }
    int E = ex - 1023;  // x = mx 2^(E - 52)
    if (E & 1) {
        mx <<= 1;
        E -= 1;
    }
    // sqrt(x) = sqrt(mx 2^52) 2^(E/2 - 52); m = mx / 2^52 in [1, 4)
    const float f = (float)(u32)(mx >> 22) * 9.31322574615478515625e-10f;  // * 2^-30
    u64 Y = seed_q63(rsqrt_seed(f));
    const u64 M = mx << 10;  // m * 2^62
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const u64 T = umulhi(umulhi(Y, Y), M);  // y^2 m 2^60
        const i64 E1 = (i64)((1ull << 60) - T);
        Y = E1 >= 0 ? Y + (umulhi(Y, (u64)E1) << 3) : Y - (umulhi(Y, (u64)(-E1)) << 3);
    }
    u64 S = umulhi(M, Y) >> 9;            // floor(sqrt(mx 2^52)) to within one unit
    i64 R = (i64)((mx << 52) - S * S);    // exact: -(2 S + 1) <= R < 4 S + 4
    if (R < 0) {
        S -= 1;
        R += (i64)(2 * S + 1);
    } else if (R > (i64)(2 * S)) {
        R -= (i64)(2 * S + 1);
        S += 1;
    }
    S += (u64)(R > (i64)S);
    return ufrom(((u64)((E >> 1) + 1022) << 52) + S);
}

// sqrt(x) rounded to nearest even and 1/sqrt(x) to about 2^-58 relative (the Newton
// iterate of the root, truncated to 53 bits), for a positive normal x; other operands
// give (sqrt_rn(x), 1 / sqrt_rn(x)) through the rare branch.  For callers that need a
// wave speed and its reciprocal together (the adjoint's dc/dh = g / (2 c)).
SWE_HD void sqrt_rsqrt(double x, double &s, double &r) {
    const u64 bx = ubits(x);
    if (bx - HIDDEN >= INF - HIDDEN) {
        s = sqrt_rn(x);
        r = div_rn(1.0, s);
        return;
    }
    u64 mx = (bx & MANT_BITS) | HIDDEN;
    int E = (int)(bx >> 52) - 1023;
    if (E & 1) {
        mx <<= 1;
        E -= 1;
    }
    const float f = (float)(u32)(mx >> 22) * 9.31322574615478515625e-10f;  // * 2^-30
    u64 Y = seed_q63(rsqrt_seed(f));
    const u64 M = mx << 10;
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const u64 T = umulhi(umulhi(Y, Y), M);
        const i64 E1 = (i64)((1ull << 60) - T);
        Y = E1 >= 0 ? Y + (umulhi(Y, (u64)E1) << 3) : Y - (umulhi(Y, (u64)(-E1)) << 3);
    }
    u64 S = umulhi(M, Y) >> 9;
    i64 R = (i64)((mx << 52) - S * S);
    if (R < 0) {
        S -= 1;
        R += (i64)(2 * S + 1);
    } else if (R > (i64)(2 * S)) {
        R -= (i64)(2 * S + 1);
        S += 1;
    }
    S += (u64)(R > (i64)S);
    s = ufrom(((u64)((E >> 1) + 1022) << 52) + S);
    // Y ~ 2^63 / sqrt(m), m = mx / 2^52 in [1, 4): Y in (2^61, 2^63]; 1/sqrt(x) = Y 2^-63
    // 2^(-E/2)
    const int lz = clz64(Y);
    const u64 q = (Y << lz) >> 11;  // 53 bits, leading one at bit 52
    r = ufrom(((u64)(1022 - lz - (E >> 1)) << 52) + q);
}

// Rare operands of mul_rn: zeros, subnormals, infinities, NaN.
SWE_COLD double mul_special(u64 ax, u64 ay, u64 sign);

// Full 106-bit product of two significands below 2^53: hi:lo.
SWE_HD void mul53(u64 a, u64 b, u64 &hi, u64 &lo) {
    const u32 al = (u32)a, ah = (u32)(a >> 32), bl = (u32)b, bh = (u32)(b >> 32);
    const u64 p0 = (u64)al * bl;
    const u64 p1 = (u64)al * bh + (p0 >> 32);
    const u64 p2 = (u64)ah * bl + (u32)p1;
    hi = (u64)ah * bh + (p1 >> 32) + (p2 >> 32);
    lo = (p2 << 32) | (u32)p0;
}

// x * y, round to nearest even.
SWE_HD double mul_rn(double x, double y) {
    const u64 bx = ubits(x), by = ubits(y);
    const u64 sign = (bx ^ by) & SIGN_BIT;
    const u64 ax = bx & ~SIGN_BIT, ay = by & ~SIGN_BIT;
    if (ax - HIDDEN >= INF - HIDDEN || ay - HIDDEN >= INF - HIDDEN) {
        if ((ax == 0 && ay < INF) || (ay == 0 && ax < INF)) return ufrom(sign);
        return mul_special(ax, ay, sign);
    }
    int e = (int)(ax >> 52) + (int)(ay >> 52) - 1023;
    u64 hi, lo;
    mul53((ax & MANT_BITS) | HIDDEN, (ay & MANT_BITS) | HIDDEN, hi, lo);
    // product in [2^104, 2^106): bring its leading one to bit 105 (bit 41 of hi)
    if (hi >> 41) {
        e += 1;
    } else {
        hi = (hi << 1) | (lo >> 63);
        lo <<= 1;
    }
    const u64 q = (hi << 11) | (lo >> 53);  // 53 significant bits
    const u64 half = (lo >> 52) & 1, sticky = (u64)((lo << 12) != 0);
    if (e >= 1 && e <= 0x7FE)
        return ufrom(sign | (((u64)(e - 1) << 52) + q + (half & (sticky | (q & 1)))));
    return round_pack(sign, e, (q << 10) | (half << 9) | sticky);
}

SWE_COLD double mul_special(u64 ax, u64 ay, u64 sign) {
    if (ax > INF || ay > INF) return ufrom(QNAN);
    if (ax == INF || ay == INF) return ufrom((ax == 0 || ay == 0) ? QNAN : (sign | INF));
    if (ax == 0 || ay == 0) return ufrom(sign);
    int ex, ey;
    const u64 mx = unpack_normalised(ax, ex), my = unpack_normalised(ay, ey);
    int e = ex + ey - 1023;
    u64 hi, lo;
    mul53(mx, my, hi, lo);
    if (hi >> 41) {
        e += 1;
    } else {
        hi = (hi << 1) | (lo >> 63);
        lo <<= 1;
    }
    const u64 q = (hi << 11) | (lo >> 53);
    const u64 half = (lo >> 52) & 1, sticky = (u64)((lo << 12) != 0);
    return round_pack(sign, e, (q << 10) | (half << 9) | sticky);
}

// Infinite or NaN a (|a| >= |b|) in add_rn.
SWE_COLD double add_special(u64 a, u64 b) {
    const u64 aa = a & ~SIGN_BIT, ab = b & ~SIGN_BIT;
    if (aa > INF || ab > INF) return ufrom(QNAN);
    if (ab == INF && ((a ^ b) & SIGN_BIT)) return ufrom(QNAN);  // inf - inf
    return ufrom(a);
}

// x + y, round to nearest even.
SWE_HD double add_rn(double x, double y) {
    u64 a = ubits(x), b = ubits(y);
    u64 aa = a & ~SIGN_BIT, ab = b & ~SIGN_BIT;
    if (aa < ab) {  // |a| >= |b|
        const u64 t = a, ta = aa;
        a = b;
        aa = ab;
        b = t;
        ab = ta;
    }
    if (aa >= INF) return add_special(a, b);
    if (ab == 0) return ufrom(aa == 0 ? (a & b) : a);  // x + 0; -0 + -0 = -0
    const int ea0 = (int)(aa >> 52), eb0 = (int)(ab >> 52);
    const int ea = ea0 ? ea0 : 1, eb = eb0 ? eb0 : 1;
    const u64 ma = ((aa & MANT_BITS) | (ea0 ? HIDDEN : 0)) << 10;
    u64 mb = ((ab & MANT_BITS) | (eb0 ? HIDDEN : 0)) << 10;
    const int d = ea - eb;
    if (d) mb = d < 63 ? ((mb >> d) | (u64)((mb << (64 - d)) != 0)) : 1;
    int e = ea;
    u64 m;
    if ((i64)(a ^ b) >= 0) {
        m = ma + mb;
        if (m >> 63) {
            m = (m >> 1) | (m & 1);
            e += 1;
        }
    } else {
        m = ma - mb;
        if (m == 0) return 0.0;  // exact cancellation is +0
        int lz = clz64(m) - 1;
        if (lz > e - 1) lz = e - 1;  // subnormal result: stay at exponent 1
        m <<= lz;
        e -= lz;
    }
    if (e >= 0x7FF) return ufrom((a & SIGN_BIT) | INF);
    const u64 r = m & 0x3FF, q = m >> 10;
    const u64 up = (u64)((r > 0x200) | ((r == 0x200) & (q & 1)));
    return ufrom((a & SIGN_BIT) | (((u64)(e - 1) << 52) + q + up));
}

// x - y == x + (-y) exactly, signed zeros included.
SWE_HD double sub_rn(double x, double y) { return add_rn(x, ufrom(ubits(y) ^ SIGN_BIT)); }

}  // namespace sf
}  // namespace swe
