// Checks the interface VJP (shallow-water_gb300/csrc/swe_adjoint_math.cuh) against central
// finite differences of the interface forward function, in FP64, on random states that
// exercise every HLL regime, minmod branch and dry guard.  Points where a branch flips
// inside the difference stencil (one-sided differences disagree) are skipped.  Then
// against the textbook derivation of the same VJP (adjoint_face_textbook.h), which must
// agree to rounding everywhere, nearly dry sides included.  Built and run by
// tests/test_adjoint_cpu.py.
#include <cmath>
#include <cstdio>
#include <random>

#include "../../shallow-water_gb300/csrc/swe_adjoint_math.cuh"
#include "adjoint_face_textbook.h"

using namespace swe::adj;

static double objective(const FaceIn<double> &in, const FaceOut<double> &w, double g) {
    FaceOut<double> o;
    face_forward(in, g, 1e-8, o);
    return w.fh * o.fh + w.fqt * o.fqt + w.fqn_m * o.fqn_m + w.fqn_p * o.fqn_p;
}

static double *slot(FaceIn<double> &in, int k) {
    if (k < 4) return &in.e[k];
    if (k < 8) return &in.n[k - 4];
    if (k < 12) return &in.t[k - 8];
    return k == 12 ? &in.bm : &in.bp;
}

int main(int argc, char **argv) {
    const int cases = argc > 1 ? std::atoi(argv[1]) : 20000;
    std::mt19937_64 rng(7);
    std::uniform_real_distribution<double> u(-1.0, 1.0);
    const double g = 9.80665;
    long checked = 0, skipped = 0, bad = 0;
    double worst = 0.0;
    int regimes[3] = {0, 0, 0};
    for (int c = 0; c < cases; ++c) {
        FaceIn<double> in;
        const double flow = (c % 3 == 0) ? 6.0 : 0.4;  // every third case supersonic-ish
        for (int k = 0; k < 4; ++k) {
            in.e[k] = 1.0 + 0.2 * u(rng);
            in.n[k] = flow * u(rng) + (c % 3 == 0 ? 4.0 * ((c / 3) % 2 ? 1 : -1) : 0.0);
            in.t[k] = 0.3 * u(rng);
        }
        in.bm = 0.3 * u(rng);
        in.bp = 0.3 * u(rng);
        if (c % 7 == 0) in.bp = in.e[2] + 0.05 * std::fabs(u(rng));  // dry plus side
        FaceOut<double> w{u(rng), u(rng), u(rng), u(rng)};
        FaceIn<double> grad;
        face_vjp(in, g, 1e-8, w, grad);
        {
            // classify regime for coverage
            FaceOut<double> o;
            face_forward(in, g, 1e-8, o);
        }
        for (int k = 0; k < 14; ++k) {
            const double h = 1e-6;
            FaceIn<double> p = in, m = in;
            *slot(p, k) += h;
            *slot(m, k) -= h;
            const double f0 = objective(in, w, g), fp = objective(p, w, g), fm = objective(m, w, g);
            const double fwd = (fp - f0) / h, bwd = (f0 - fm) / h, cen = (fp - fm) / (2 * h);
            const double scale = std::fmax(1.0, std::fabs(cen));
            if (std::fabs(fwd - bwd) > 1e-4 * scale) {  // a branch flips within +-h
                ++skipped;
                continue;
            }
            const double a = *slot(grad, k);
            const double err = std::fabs(a - cen) / scale;
            worst = std::fmax(worst, err);
            ++checked;
            if (err > 2e-6) {
                if (++bad <= 10)
                    std::printf("case %d input %d: vjp %.12g fd %.12g err %.3g\n", c, k, a, cen, err);
            }
        }
    }
    (void)regimes;
    std::printf("checked %ld partials, skipped %ld at kinks, worst rel err %.3g, %ld bad\n",
                checked, skipped, worst, bad);

    // The two derivations, relative to the largest partial of each case.  Case kinds:
    // subsonic and supersonic flow, a dry plus side, hydrostatic depths of 0 to 5e-9 on
    // either side (below the 1e-8 wet threshold while the cell itself is wet), a dry
    // minus cell.
    long differ = 0;
    double worst_tb = 0.0;
    for (int c = 0; c < 12 * cases; ++c) {
        FaceIn<double> in;
        const int kind = c % 6;
        const double flow = kind == 0 ? 6.0 : 0.4;
        for (int k = 0; k < 4; ++k) {
            in.e[k] = 1.0 + 0.2 * u(rng);
            in.n[k] = flow * u(rng) + (kind == 0 ? 4.0 * ((c / 6) % 2 ? 1 : -1) : 0.0);
            in.t[k] = 0.3 * u(rng);
        }
        in.bm = 0.3 * u(rng);
        in.bp = 0.3 * u(rng);
        if (kind == 1) in.bp = in.e[2] + 0.05 * std::fabs(u(rng));
        if (kind == 2) {
            for (int k = 0; k < 4; ++k) in.e[k] = in.e[1];
            in.bp = in.e[1] - 0.5e-8 * std::fabs(u(rng));
            in.bm = in.bp - 0.1;
        }
        if (kind == 3) {
            for (int k = 0; k < 4; ++k) in.e[k] = in.e[2];
            in.bm = in.e[2] - 0.5e-8 * std::fabs(u(rng));
            in.bp = in.bm - 0.1;
        }
        if (kind == 4) in.bm = in.e[1] + 0.1;
        FaceOut<double> w{u(rng), u(rng), u(rng), u(rng)};
        FaceIn<double> a, b;
        face_vjp(in, g, 1e-8, w, a);
        swe::adj_textbook::face_vjp_textbook(in, g, 1e-8, w, b);
        double scale = 1e-300, diff = 0.0;
        for (int k = 0; k < 14; ++k) scale = std::fmax(scale, std::fabs(*slot(b, k)));
        for (int k = 0; k < 14; ++k) diff = std::fmax(diff, std::fabs(*slot(a, k) - *slot(b, k)));
        worst_tb = std::fmax(worst_tb, diff / scale);
        if (diff > 1e-9 * scale && ++differ <= 10)
            std::printf("case %d kind %d: the derivations differ by %.3g\n", c, kind, diff / scale);
    }
    std::printf("textbook derivation: %d cases, worst rel diff %.3g, %ld differ\n", 12 * cases,
                worst_tb, differ);
    return (bad || differ) ? 1 : 0;
}
