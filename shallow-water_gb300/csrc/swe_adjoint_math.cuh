// Reverse-mode (vector-Jacobian product) of one interface of the scheme.
//
// Forward: the interface of compute_x_fluxes / compute_y_fluxes
// (HPC_kernels.hpp:136-184, 203-251) in normal/tangential form.  Inputs are the 4-cell
// stencil (m1, c0 | p1, p2) of eta = h + B, the normal momentum qn and the tangential
// momentum qt, and B of the two adjacent cells.  Outputs are the mass flux fh, the
// tangential flux fqt, and the normal-momentum flux seen by the minus cell (with
// corr_minus) and by the plus cell (with corr_plus).
//
// The VJP takes adjoints of the four outputs and returns adjoints of the 14 inputs.
// Branches (minmod, positive parts, dry guards, HLL regimes, min/max of the wave speeds)
// take the derivative of the branch the forward pass took, which is the discrete adjoint
// of the scheme as executed.  Templated on the scalar type so the same code runs on the
// host (finite-difference tests) and on the device in FP64 and FP32.
#pragma once

#include <cmath>
#include <type_traits>

#include "swe_soft_f64.cuh"

#if defined(__CUDACC__)
#define SWE_HD __host__ __device__ __forceinline__
#else
#define SWE_HD inline
#endif

namespace swe {
namespace adj {

template <class T>
struct FaceIn {
    T e[4], n[4], t[4];  // eta, qn, qt at m1, c0, p1, p2
    T bm, bp;            // B at c0 and p1
};

template <class T>
struct FaceOut {
    T fh, fqt, fqn_m, fqn_p;
};

template <class T>
SWE_HD T tmin(T a, T b) { return (b < a) ? b : a; }
template <class T>
SWE_HD T tmax(T a, T b) { return (a < b) ? b : a; }
template <class T>
SWE_HD T tabs(T a) { return a < T(0) ? -a : a; }

// minmod value and which argument it selected (0: none / zero, 1: a, 2: b).
template <class T>
SWE_HD T minmod_sel(T a, T b, int &sel) {
    if (a * b <= T(0)) {
        sel = 0;
        return T(0);
    }
    if (tabs(b) < tabs(a)) {
        sel = 2;
        return b;
    }
    sel = 1;
    return a;
}

template <class T>
SWE_HD void face_forward(const FaceIn<T> &in, T g, T eps, FaceOut<T> &out) {
    const T half = T(0.5);
    int s;
    const T eta_m = in.e[1] + half * minmod_sel(in.e[1] - in.e[0], in.e[2] - in.e[1], s);
    const T eta_p = in.e[2] - half * minmod_sel(in.e[2] - in.e[1], in.e[3] - in.e[2], s);
    const T qn_m = in.n[1] + half * minmod_sel(in.n[1] - in.n[0], in.n[2] - in.n[1], s);
    const T qt_m = in.t[1] + half * minmod_sel(in.t[1] - in.t[0], in.t[2] - in.t[1], s);
    const T qn_p = in.n[2] - half * minmod_sel(in.n[2] - in.n[1], in.n[3] - in.n[2], s);
    const T qt_p = in.t[2] - half * minmod_sel(in.t[2] - in.t[1], in.t[3] - in.t[2], s);
    const T bs = tmax(in.bm, in.bp);
    const T h_m = tmax(eta_m - in.bm, T(0)), h_p = tmax(eta_p - in.bp, T(0));
    const T un_m = h_m > eps ? qn_m / h_m : T(0), ut_m = h_m > eps ? qt_m / h_m : T(0);
    const T un_p = h_p > eps ? qn_p / h_p : T(0), ut_p = h_p > eps ? qt_p / h_p : T(0);
    const T hL = tmax(eta_m - bs, T(0)), hR = tmax(eta_p - bs, T(0));
    const T qnL = hL * un_m, qtL = hL * ut_m, qnR = hR * un_p, qtR = hR * ut_p;
    const T unL = hL > eps ? qnL / hL : T(0), utL = hL > eps ? qtL / hL : T(0);
    const T unR = hR > eps ? qnR / hR : T(0), utR = hR > eps ? qtR / hR : T(0);
    const T cL = sqrt(g * hL), cR = sqrt(g * hR);
    const T sL = tmin(unL - cL, unR - cR), sR = tmax(unL + cL, unR + cR);
    const T FL[3] = {qnL, qnL * unL + half * g * hL * hL, qnL * utL};
    const T FR[3] = {qnR, qnR * unR + half * g * hR * hR, qnR * utR};
    const T UL[3] = {hL, qnL, qtL}, UR[3] = {hR, qnR, qtR};
    T F[3];
    if (sL >= T(0)) {
        for (int c = 0; c < 3; ++c) F[c] = FL[c];
    } else if (sR <= T(0)) {
        for (int c = 0; c < 3; ++c) F[c] = FR[c];
    } else {
        const T inv = T(1) / (sR - sL);
        for (int c = 0; c < 3; ++c) F[c] = (sR * FL[c] - sL * FR[c] + sL * sR * (UR[c] - UL[c])) * inv;
    }
    out.fh = F[0];
    out.fqt = F[2];
    out.fqn_m = F[1] + half * g * (h_m * h_m - hL * hL);
    out.fqn_p = F[1] + half * g * (h_p * h_p - hR * hR);
}

template <class T>
SWE_HD T trsqrt(T x) {
#if defined(__CUDA_ARCH__)
    return rsqrt(x);
#else
    return T(1) / sqrt(x);
#endif
}

// Branch tests and reciprocals of face_vjp.  For double they work on the bit patterns
// (the same decisions as the IEEE comparisons for every non-NaN operand) and the
// reciprocal is the correctly rounded integer-pipe division, so the GPU spends its
// scarce FP64 slots on the arithmetic alone.
template <class T>
SWE_HD bool lt_(T a, T b) {
    if constexpr (std::is_same<T, double>::value) return x64::lt(a, b);
    else return a < b;
}
template <class T>
SWE_HD bool pos_(T a) {  // a > 0
    if constexpr (std::is_same<T, double>::value) {
        const int64_t b = x64::bits(a);
        return b > 0 && b <= x64::INF_BITS;
    } else {
        return a > T(0);
    }
}
template <class T>
SWE_HD T rcp_(T a) {
    if constexpr (std::is_same<T, double>::value) {
        return sf::div_rn(1.0, a);
    } else {
#if defined(__CUDA_ARCH__)
        // FP32: the approximate reciprocal (about 1 ulp) of the FP32 forward's velocities
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
        return r;
#else
        return T(1) / a;
#endif
    }
}
template <class T>
SWE_HD T half_(T a) {  // 0.5 * a, exact
    if constexpr (std::is_same<T, double>::value) return x64::halve(a);
    else return T(0.5) * a;
}
// c = sqrt(x) and rc = 1 / c for x > 0, both 0 otherwise; for double from one
// integer-pipe root (c correctly rounded, rc to about 1 ulp).
template <class T>
SWE_HD void speed_(T x, T &c, T &rc) {
    if (!pos_(x)) {
        c = rc = T(0);
        return;
    }
    if constexpr (std::is_same<T, double>::value) {
        sf::sqrt_rsqrt(x, c, rc);
    } else {
        rc = trsqrt(x);
        c = x * rc;
    }
}

// minmod_sel with the sign and magnitude tests on the bit patterns for double.
template <class T>
SWE_HD T msel_(T a, T b, int &sel) {
    if constexpr (std::is_same<T, double>::value) {
        const int64_t ba = x64::bits(a), bb = x64::bits(b);
        const int64_t ma = ba & x64::ABS, mb = bb & x64::ABS;
        if (ma == 0 || mb == 0 || (ba ^ bb) < 0) {
            sel = 0;
            return T(0);
        }
        if (mb < ma) {
            sel = 2;
            return b;
        }
        sel = 1;
        return a;
    } else {
        return minmod_sel(a, b, sel);
    }
}


// Adjoint of face_forward: given d = dJ/d(out), returns a = dJ/d(in) (overwritten).
//
// The forward part is recomputed for its branch decisions and intermediates with one
// reciprocal per depth (q/h as q * (1/h)), the hydrostatic velocities (hs*u)/hs taken as
// u (equal in exact arithmetic) and the wave speed from one root; these differ from the
// forward's rounding by an ulp, which matters only at exact ties of a branch test.
//
// Reverse sweep.  Each side (L: the minus cell's hydrostatic state, R: the plus cell's)
// has depth h, velocities u, v, and the flux velocities uc, vc (u, v where h > eps,
// else 0): U = (h, h u, h v) and F = (h u, h u uc + g h^2 / 2, h u vc).  The HLL flux
// is F* = aL FL + aR FR + bL UL + bR UR with (aL, aR, bL, bR) = (1, 0, 0, 0) if
// sL >= 0, (0, 1, 0, 0) if sR <= 0, else (sR, -sL, -sL sR, sL sR) / (sR - sL).  With
// the side sums P = dF . (1, u, v) and Pc = dF . (1, uc, vc),
//   dF . F = h u Pc + dF1 g h^2 / 2   and   dF . U = h P,
// so each side's adjoints are
//   dh = a (u Pc + dF1 g h) + b P,   du = h (a (Pc + dF1 uc) + b dF1),
//   dv = h dF2 (a uc + b),
// and the HLL speed derivatives take the sums A = dF . (FR - FL) and
// S = dF . (UR - UL) from the same P: no flux vector is formed.  In double, one
// interface costs three reciprocals and two roots on the integer pipe and about 125
// FP64 operations; in float the reciprocals and roots are the approximate ones.
template <class T>
SWE_HD void face_vjp(const FaceIn<T> &in, T g, T eps, const FaceOut<T> &d, FaceIn<T> &a) {
    // ---- forward recomputation, keeping branch decisions ----
    int s_em, s_ep, s_nm, s_tm, s_np, s_tp;
    const T de0 = in.e[1] - in.e[0], de1 = in.e[2] - in.e[1], de2 = in.e[3] - in.e[2];
    const T dn0 = in.n[1] - in.n[0], dn1 = in.n[2] - in.n[1], dn2 = in.n[3] - in.n[2];
    const T dt0 = in.t[1] - in.t[0], dt1 = in.t[2] - in.t[1], dt2 = in.t[3] - in.t[2];
    // halving is exact: an integer-pipe exponent step for double
    const T eta_m = in.e[1] + half_(msel_(de0, de1, s_em));
    const T eta_p = in.e[2] - half_(msel_(de1, de2, s_ep));
    const T qn_m = in.n[1] + half_(msel_(dn0, dn1, s_nm));
    const T qt_m = in.t[1] + half_(msel_(dt0, dt1, s_tm));
    const T qn_p = in.n[2] - half_(msel_(dn1, dn2, s_np));
    const T qt_p = in.t[2] - half_(msel_(dt1, dt2, s_tp));
    const bool bstar_is_p = lt_(in.bm, in.bp);  // std::max(bm, bp) == (bm < bp) ? bp : bm
    const T bs = bstar_is_p ? in.bp : in.bm;
    const T xm = eta_m - in.bm, xp = eta_p - in.bp;
    const bool pm = pos_(xm), pp = pos_(xp);
    const T h_m = pm ? xm : T(0), h_p = pp ? xp : T(0);
    const bool wm = lt_(eps, h_m), wp = lt_(eps, h_p);
    const T rm = wm ? rcp_(h_m) : T(0), rp = wp ? rcp_(h_p) : T(0);
    const T uL = qn_m * rm, vL = qt_m * rm, uR = qn_p * rp, vR = qt_p * rp;
    const T yL = eta_m - bs, yR = eta_p - bs;
    const bool pL = pos_(yL), pR = pos_(yR);
    const T hL = pL ? yL : T(0), hR = pR ? yR : T(0);
    const bool wL = lt_(eps, hL), wR = lt_(eps, hR);
    const T uLc = wL ? uL : T(0), uRc = wR ? uR : T(0);
    const T ghL = g * hL, ghR = g * hR;
    T cL, rcL, cR, rcR;
    speed_(ghL, cL, rcL);
    speed_(ghR, cR, rcR);
    const T a1 = uLc - cL, a2 = uRc - cR, b1 = uLc + cL, b2 = uRc + cR;
    const bool sL_is2 = lt_(a2, a1), sR_is2 = lt_(b1, b2);
    const T sL = sL_is2 ? a2 : a1, sR = sR_is2 ? b2 : b1;
    const int regime = !lt_(sL, T(0)) ? 0 : (!lt_(T(0), sR) ? 1 : 2);

    // ---- reverse sweep ----
    const T dF0 = d.fh, dF1 = d.fqn_m + d.fqn_p, dF2 = d.fqt;
    const T PL = dF0 + dF1 * uL + dF2 * vL, PR = dF0 + dF1 * uR + dF2 * vR;
    const T PLc = wL ? PL : dF0, PRc = wR ? PR : dF0;
    T aL = regime == 0 ? T(1) : T(0), aR = regime == 1 ? T(1) : T(0);
    T bL = T(0), bR = T(0);
    T duLs = T(0), dcL = T(0), duRs = T(0), dcR = T(0);  // through the wave speeds
    if (regime == 2) {
        const T W = rcp_(sR - sL);
        const T sRW = sR * W, sLW = sL * W;
        aL = sRW;
        aR = -sLW;
        bR = sL * sRW;
        bL = -bR;
        // dF*/dsR = sL (FR - FL - sL (UR - UL)) W^2, dF*/dsL = sR (sR (UR - UL) - FR + FL) W^2
        const T S = hR * PR - hL * PL;
        const T A = ((hR * uR) * PRc - (hL * uL) * PLc) + half_(dF1 * (ghR * hR - ghL * hL));
        const T dsR = (A - sL * S) * (sLW * W);
        const T dsL = (sR * S - A) * (sRW * W);
        // sL = min(uLc - cL, uRc - cR), sR = max(uLc + cL, uRc + cR)
        const T sum = dsL + dsR, diff = dsR - dsL;
        const bool lL = !sL_is2, lR = !sR_is2;  // the speed taken from side L
        duLs = lL ? (lR ? sum : dsL) : (lR ? dsR : T(0));
        dcL = lL ? (lR ? diff : -dsL) : (lR ? dsR : T(0));
        duRs = lL ? (lR ? T(0) : dsR) : (lR ? dsL : sum);
        dcR = lL ? (lR ? T(0) : dsR) : (lR ? -dsL : diff);
    }
    const T hg = half_(g);
    // side L, then its hydrostatic correction g/2 (h_m^2 - hL^2) of the minus flux and
    // the wave speed c = sqrt(g h) (dc/dh = g / (2 c))
    const T aLP = aL * PLc, aLF = aL * dF1;
    const T dhL = ((aLP * uL + (aLF * ghL + bL * PL)) - ghL * d.fqn_m) + dcL * (hg * rcL);
    const T duL = hL * (aLF * uLc + (aLP + bL * dF1)) + (wL ? duLs : T(0));
    const T dvL = (hL * dF2) * (aL * uLc + bL);
    const T aRP = aR * PRc, aRF = aR * dF1;
    const T dhR = ((aRP * uR + (aRF * ghR + bR * PR)) - ghR * d.fqn_p) + dcR * (hg * rcR);
    const T duR = hR * (aRF * uRc + (aRP + bR * dF1)) + (wR ? duRs : T(0));
    const T dvR = (hR * dF2) * (aR * uRc + bR);
    // velocities u = q / h_m: dq = du / h_m, dh_m = -(du u + dv v) / h_m
    const T dqn_m = duL * rm, dqt_m = dvL * rm, dqn_p = duR * rp, dqt_p = dvR * rp;
    const T dh_m = (g * h_m) * d.fqn_m - (duL * uL + dvL * vL) * rm;
    const T dh_p = (g * h_p) * d.fqn_p - (duR * uR + dvR * vR) * rp;
    // hL = max(eta_m - bs, 0), h_m = max(eta_m - bm, 0), bs = max(bm, bp)
    const T eL = pL ? dhL : T(0), eR = pR ? dhR : T(0);
    const T em = pm ? dh_m : T(0), ep = pp ? dh_p : T(0);
    const T deta_m = eL + em, deta_p = eR + ep;
    const T dbs = -(eL + eR);
    const T dstar = dbs - (bstar_is_p ? ep : em);  // the bed bs was taken from
    a.bm = bstar_is_p ? -em : dstar;
    a.bp = bstar_is_p ? dstar : -ep;
    // reconstructions x_m = x1 + m(x1-x0, x2-x1)/2 and x_p = x2 - m(x2-x1, x3-x2)/2, with
    // minmod selecting its first argument (sel 1), its second (sel 2) or zero (sel 0)
    auto recon = [&](T *ax, T dxm, int sm, T dxp, int sp) {
        const T hm = half_(dxm), hp = half_(dxp);
        ax[0] = sm == 1 ? -hm : T(0);
        ax[1] = (sm == 0 ? dxm : (sm == 1 ? dxm + hm : hm)) + (sp == 1 ? hp : T(0));
        ax[2] = (sm == 2 ? hm : T(0)) + (sp == 0 ? dxp : (sp == 1 ? hp : dxp + hp));
        ax[3] = sp == 2 ? -hp : T(0);
    };
    recon(a.e, deta_m, s_em, deta_p, s_ep);
    recon(a.n, dqn_m, s_nm, dqn_p, s_np);
    recon(a.t, dqt_m, s_tm, dqt_p, s_tp);
}

}  // namespace adj
}  // namespace swe
