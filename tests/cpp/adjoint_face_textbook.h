// The interface VJP written the textbook way: flux vectors FL, FR and state vectors UL, UR
// of both sides, their adjoints dFL, dFR, dUL, dUR from the HLL weights, then the chain
// through the physical fluxes.  tests/cpp/adjoint_face_check.cpp checks the production
// VJP (shallow-water_gb300/csrc/swe_adjoint_math.cuh), which works on per-side sums and
// forms none of these vectors, against it: the two derivations must agree to rounding.
// Same forward recomputation and branch decisions as the production VJP.
#pragma once

#include "../../shallow-water_gb300/csrc/swe_adjoint_math.cuh"

namespace swe {
namespace adj_textbook {

using adj::FaceIn;
using adj::FaceOut;
using adj::half_;
using adj::lt_;
using adj::msel_;
using adj::pos_;
using adj::rcp_;
using adj::speed_;

template <class T>
SWE_HD void face_vjp_textbook(const FaceIn<T> &in, T g, T eps, const FaceOut<T> &d, FaceIn<T> &a) {
    const T half = T(0.5);
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
    const T un_m = qn_m * rm, ut_m = qt_m * rm;
    const T un_p = qn_p * rp, ut_p = qt_p * rp;
    const T yL = eta_m - bs, yR = eta_p - bs;
    const bool pL = pos_(yL), pR = pos_(yR);
    const T hL = pL ? yL : T(0), hR = pR ? yR : T(0);
    const T qnL = hL * un_m, qtL = hL * ut_m, qnR = hR * un_p, qtR = hR * ut_p;
    const bool wL = lt_(eps, hL), wR = lt_(eps, hR);
    const T unL = wL ? un_m : T(0), utL = wL ? ut_m : T(0);
    const T unR = wR ? un_p : T(0), utR = wR ? ut_p : T(0);
    const T ghL = g * hL, ghR = g * hR;
    T cL, rcL, cR, rcR;
    speed_(ghL, cL, rcL);
    speed_(ghR, cR, rcR);
    const T a1 = unL - cL, a2 = unR - cR, b1 = unL + cL, b2 = unR + cR;
    const bool sL_is2 = lt_(a2, a1), sR_is2 = lt_(b1, b2);
    const T sL = sL_is2 ? a2 : a1, sR = sR_is2 ? b2 : b1;
    const T hg = half * g;
    // g/2 h^2 as (g h) h / 2: the halving is exact, so these are (g/2 h) h bit for bit
    const T FL[3] = {qnL, qnL * unL + half_(ghL * hL), qnL * utL};
    const T FR[3] = {qnR, qnR * unR + half_(ghR * hR), qnR * utR};
    const T UL[3] = {hL, qnL, qtL}, UR[3] = {hR, qnR, qtR};
    const int regime = !lt_(sL, T(0)) ? 0 : (!lt_(T(0), sR) ? 1 : 2);

    // ---- reverse sweep ----
    const T dF[3] = {d.fh, d.fqn_m + d.fqn_p, d.fqt};
    T dh_m = g * h_m * d.fqn_m, dh_p = g * h_p * d.fqn_p;
    T dhL = -ghL * d.fqn_m, dhR = -ghR * d.fqn_p;
    T dFL[3] = {0, 0, 0}, dFR[3] = {0, 0, 0}, dUL[3] = {0, 0, 0}, dUR[3] = {0, 0, 0};
    T dsL = 0, dsR = 0;
    if (regime == 0) {
        for (int c = 0; c < 3; ++c) dFL[c] = dF[c];
    } else if (regime == 1) {
        for (int c = 0; c < 3; ++c) dFR[c] = dF[c];
    } else {
        // F = (sR FL - sL FR + sL sR dU) / (sR - sL) with dU = UR - UL, G = FR - FL:
        // dF/dsR = sL (G - sL dU) / (sR - sL)^2, dF/dsL = sR (sR dU - G) / (sR - sL)^2
        // with A = sum dF G and S = sum dF dU: sum dF (G - sL dU) = A - sL S and
        // sum dF (sR dU - G) = sR S - A
        const T inv = rcp_(sR - sL);
        const T sLi = sL * inv, sRi = sR * inv, sLsRi = sL * sRi;
        T A = 0, S = 0;
        for (int c = 0; c < 3; ++c) {
            const T dU = UR[c] - UL[c], G = FR[c] - FL[c];
            dFL[c] = dF[c] * sRi;
            dFR[c] = -dF[c] * sLi;
            dUR[c] = dF[c] * sLsRi;
            dUL[c] = -dUR[c];
            A += dF[c] * G;
            S += dF[c] * dU;
        }
        dsR = (A - sL * S) * (sLi * inv);
        dsL = (sR * S - A) * (sRi * inv);
    }
    T dunL = 0, dunR = 0, dcL = 0, dcR = 0;
    if (sL_is2) {
        dunR += dsL;
        dcR -= dsL;
    } else {
        dunL += dsL;
        dcL -= dsL;
    }
    if (sR_is2) {
        dunR += dsR;
        dcR += dsR;
    } else {
        dunL += dsR;
        dcL += dsR;
    }
    dhL += dcL * hg * rcL;  // dc/dh = g / (2 c)
    dhR += dcR * hg * rcR;
    // physical fluxes FL = (qnL, qnL unL + g/2 hL^2, qnL utL); U = (h, qn, qt)
    const T dqnL = dFL[0] + dFL[1] * unL + dFL[2] * utL + dUL[1];
    const T dqtL = dUL[2];
    dunL += dFL[1] * qnL;
    T dutL = dFL[2] * qnL;
    dhL += dFL[1] * ghL + dUL[0];
    const T dqnR = dFR[0] + dFR[1] * unR + dFR[2] * utR + dUR[1];
    const T dqtR = dUR[2];
    dunR += dFR[1] * qnR;
    T dutR = dFR[2] * qnR;
    dhR += dFR[1] * ghR + dUR[0];
    // unL = un_m (wet L), qnL = hL un_m, ...
    T dun_m = dqnL * hL + (wL ? dunL : T(0)), dut_m = dqtL * hL + (wL ? dutL : T(0));
    T dun_p = dqnR * hR + (wR ? dunR : T(0)), dut_p = dqtR * hR + (wR ? dutR : T(0));
    dhL += dqnL * un_m + dqtL * ut_m;
    dhR += dqnR * un_p + dqtR * ut_p;
    // hL = max(eta_m - bs, 0)
    T deta_m = 0, deta_p = 0, dbs = 0;
    if (pL) {
        deta_m += dhL;
        dbs -= dhL;
    }
    if (pR) {
        deta_p += dhR;
        dbs -= dhR;
    }
    // un_m = qn_m / h_m (wet)
    const T dqn_m = dun_m * rm, dqt_m = dut_m * rm;
    const T dqn_p = dun_p * rp, dqt_p = dut_p * rp;
    dh_m -= (dun_m * un_m + dut_m * ut_m) * rm;
    dh_p -= (dun_p * un_p + dut_p * ut_p) * rp;
    // h_m = max(eta_m - bm, 0)
    T dbm = 0, dbp = 0;
    if (pm) {
        deta_m += dh_m;
        dbm -= dh_m;
    }
    if (pp) {
        deta_p += dh_p;
        dbp -= dh_p;
    }
    if (bstar_is_p)
        dbp += dbs;
    else
        dbm += dbs;
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
    a.bm = dbm;
    a.bp = dbp;
}

}  // namespace adj_textbook
}  // namespace swe
