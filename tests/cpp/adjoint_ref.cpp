// CPU reference of the discrete adjoint of the SSP-RK3 scheme (test infrastructure).
//
// Straightforward scatter form: every interface VJP (swe_adjoint_math.cuh) adds into the
// cells of its stencil, ghost contributions are folded onto the interior cells they
// mirror (reflecting, normal momentum negated) or copy (transmissive), and the RK3
// stages and positivity clamps are reversed in order.  Used (a) by
// tests/test_adjoint_cpu.py to check the assembly against finite differences of the
// same forward and (b) by the GPU adjoint tests as an independent gather-free
// implementation.  Forward steps use face_forward, the reference's arithmetic.
#include <cmath>
#include <cstring>
#include <vector>

#include "../../shallow-water_gb300/csrc/swe_adjoint_math.cuh"

using namespace swe::adj;

namespace {

struct Grid {
    int Nx, Ny, bc;
    double dx, dy, g;
    int S() const { return Ny + 4; }
    int idx(int i, int j) const { return (i + 2) * S() + (j + 2); }  // interior coords
    size_t n() const { return (size_t)(Nx + 4) * S(); }
};

// map an interior coordinate to (source, flip)
int mapc(int a, int N, int bc, bool &flip) {
    flip = false;
    if (a < 0) {
        if (bc == 0) {
            a = -1 - a;
            flip = true;
        } else {
            a = 0;
        }
    } else if (a >= N) {
        if (bc == 0) {
            a = 2 * N - 1 - a;
            flip = true;
        } else {
            a = N - 1;
        }
    }
    return a;
}

struct State {
    std::vector<double> h, hu, hv;
};

// value of field f at (i, j) possibly ghost, with the wall rule (B read where it lies).
double sval(const Grid &G, const State &U, int f, int i, int j) {
    bool fx, fy;
    const int mi = mapc(i, G.Nx, G.bc, fx), mj = mapc(j, G.Ny, G.bc, fy);
    const int k = G.idx(mi, mj);
    if (f == 0) return U.h[k];
    if (f == 1) return fx ? -U.hu[k] : U.hu[k];
    return fy ? -U.hv[k] : U.hv[k];
}

FaceIn<double> face_in(const Grid &G, const State &U, const double *B, int i, int j, int dir) {
    FaceIn<double> in;
    for (int k = 0; k < 4; ++k) {
        const int ii = dir == 0 ? i - 1 + k : i, jj = dir == 0 ? j : j - 1 + k;
        const double h = sval(G, U, 0, ii, jj);
        in.e[k] = h + B[(ii + 2) * G.S() + (jj + 2)];
        const double hu = sval(G, U, 1, ii, jj), hv = sval(G, U, 2, ii, jj);
        in.n[k] = dir == 0 ? hu : hv;
        in.t[k] = dir == 0 ? hv : hu;
    }
    const int i1 = dir == 0 ? i + 1 : i, j1 = dir == 0 ? j : j + 1;
    in.bm = B[(i + 2) * G.S() + (j + 2)];
    in.bp = B[(i1 + 2) * G.S() + (j1 + 2)];
    return in;
}

// rhs = L(U) on the interior
void rhs(const Grid &G, const State &U, const double *B, State &R) {
    R.h.assign(G.n(), 0.0);
    R.hu.assign(G.n(), 0.0);
    R.hv.assign(G.n(), 0.0);
    const double idx = 1.0 / G.dx, idy = 1.0 / G.dy;
    for (int i = -1; i < G.Nx; ++i)
        for (int j = 0; j < G.Ny; ++j) {
            FaceOut<double> o;
            face_forward(face_in(G, U, B, i, j, 0), G.g, 1e-8, o);
            if (i >= 0) {
                const int k = G.idx(i, j);
                R.h[k] -= idx * o.fh;
                R.hu[k] -= idx * o.fqn_m;
                R.hv[k] -= idx * o.fqt;
            }
            if (i + 1 < G.Nx) {
                const int k = G.idx(i + 1, j);
                R.h[k] += idx * o.fh;
                R.hu[k] += idx * o.fqn_p;
                R.hv[k] += idx * o.fqt;
            }
        }
    for (int i = 0; i < G.Nx; ++i)
        for (int j = -1; j < G.Ny; ++j) {
            FaceOut<double> o;
            face_forward(face_in(G, U, B, i, j, 1), G.g, 1e-8, o);
            if (j >= 0) {
                const int k = G.idx(i, j);
                R.h[k] -= idy * o.fh;
                R.hv[k] -= idy * o.fqn_m;
                R.hu[k] -= idy * o.fqt;
            }
            if (j + 1 < G.Ny) {
                const int k = G.idx(i, j + 1);
                R.h[k] += idy * o.fh;
                R.hv[k] += idy * o.fqn_p;
                R.hu[k] += idy * o.fqt;
            }
        }
}

// adds (dL/dU)^T w into gU and (dL/dB)^T w into gB (interior cells; ghost folds applied)
void rhs_vjp(const Grid &G, const State &U, const double *B, const State &w, State &gU,
             std::vector<double> &gB) {
    const double idx = 1.0 / G.dx, idy = 1.0 / G.dy;
    auto wv = [&](const std::vector<double> &a, int i, int j) {
        if (i < 0 || i >= G.Nx || j < 0 || j >= G.Ny) return 0.0;
        return a[G.idx(i, j)];
    };
    auto add_cell = [&](int i, int j, int dir, double e, double qn, double qt, double b) {
        bool fx, fy;
        const int mi = mapc(i, G.Nx, G.bc, fx), mj = mapc(j, G.Ny, G.bc, fy);
        const int k = G.idx(mi, mj);
        double hu = dir == 0 ? qn : qt, hv = dir == 0 ? qt : qn;
        if (fx) hu = -hu;
        if (fy) hv = -hv;
        gU.h[k] += e;
        gU.hu[k] += hu;
        gU.hv[k] += hv;
        gB[k] += e + b;  // eta = h + B; B ghosts follow the wall rule
    };
    for (int dir = 0; dir < 2; ++dir) {
        const int ni = dir == 0 ? G.Nx : G.Nx, nj = dir == 0 ? G.Ny : G.Ny;
        for (int i = dir == 0 ? -1 : 0; i < ni; ++i)
            for (int j = dir == 0 ? 0 : -1; j < nj; ++j) {
                const int i1 = dir == 0 ? i + 1 : i, j1 = dir == 0 ? j : j + 1;
                const double c = dir == 0 ? idx : idy;
                FaceOut<double> d;
                const std::vector<double> &wn = dir == 0 ? w.hu : w.hv;
                const std::vector<double> &wt = dir == 0 ? w.hv : w.hu;
                d.fh = c * (wv(w.h, i1, j1) - wv(w.h, i, j));
                d.fqt = c * (wv(wt, i1, j1) - wv(wt, i, j));
                d.fqn_m = -c * wv(wn, i, j);
                d.fqn_p = c * wv(wn, i1, j1);
                FaceIn<double> a;
                face_vjp(face_in(G, U, B, i, j, dir), G.g, 1e-8, d, a);
                for (int k = 0; k < 4; ++k) {
                    const int ii = dir == 0 ? i - 1 + k : i, jj = dir == 0 ? j : j - 1 + k;
                    add_cell(ii, jj, dir, a.e[k], a.n[k], a.t[k], 0.0);
                }
                add_cell(i, j, dir, 0, 0, 0, a.bm);
                add_cell(i1, j1, dir, 0, 0, 0, a.bp);
            }
    }
}

void combine(const Grid &G, int stage, double dt, const State &Un, const State &Us,
             const State &R, State &out, std::vector<unsigned char> &mask) {
    out = Us;
    mask.assign(G.n(), 0);
    for (int i = 0; i < G.Nx; ++i)
        for (int j = 0; j < G.Ny; ++j) {
            const int k = G.idx(i, j);
            double o[3];
            const double s[3] = {Us.h[k], Us.hu[k], Us.hv[k]};
            const double n[3] = {Un.h[k], Un.hu[k], Un.hv[k]};
            const double r[3] = {R.h[k], R.hu[k], R.hv[k]};
            for (int f = 0; f < 3; ++f) {
                if (stage == 1) o[f] = s[f] + dt * r[f];
                else if (stage == 2) o[f] = 0.75 * n[f] + 0.25 * (s[f] + dt * r[f]);
                else o[f] = (1.0 / 3.0) * n[f] + (2.0 / 3.0) * (s[f] + dt * r[f]);
            }
            if (o[0] < 1e-8) {
                o[0] = 1e-8;
                o[1] = o[2] = 0.0;
                mask[k] = 1;
            }
            out.h[k] = o[0];
            out.hu[k] = o[1];
            out.hv[k] = o[2];
        }
}

}  // namespace

extern "C" {

// Runs `steps` fixed-dt steps from (h, hu, hv) over B (ghosted, (Nx+4)x(Ny+4)) and
// returns J = sum over steps 1..steps and gauges of (h - obs)^2; with grads non-NULL,
// also dJ/dh0, dJ/dhu0, dJ/dhv0 and dJ/dB (h0, hu0, hv0 held fixed) on the interior.
double adjref_run(int Nx, int Ny, double Lx, double Ly, double g, int bc, int steps, double dt,
                  const double *h, const double *hu, const double *hv, const double *B,
                  int ng, const int *gi, const int *gj, const double *obs, double *gh,
                  double *ghu, double *ghv, double *gBout) {
    Grid G{Nx, Ny, bc, Lx / Nx, Ly / Ny, g};
    const size_t n = G.n();
    std::vector<State> traj(steps + 1), S1(steps), S2(steps);
    std::vector<std::vector<unsigned char>> M1(steps), M2(steps), M3(steps);
    traj[0].h.assign(h, h + n);
    traj[0].hu.assign(hu, hu + n);
    traj[0].hv.assign(hv, hv + n);
    double J = 0.0;
    for (int s = 0; s < steps; ++s) {
        State R;
        rhs(G, traj[s], B, R);
        combine(G, 1, dt, traj[s], traj[s], R, S1[s], M1[s]);
        rhs(G, S1[s], B, R);
        combine(G, 2, dt, traj[s], S1[s], R, S2[s], M2[s]);
        rhs(G, S2[s], B, R);
        combine(G, 3, dt, traj[s], S2[s], R, traj[s + 1], M3[s]);
        for (int q = 0; q < ng; ++q) {
            const double r = traj[s + 1].h[G.idx(gi[q], gj[q])] - obs[(size_t)s * ng + q];
            J += r * r;
        }
    }
    if (!gh) return J;
    State lam{std::vector<double>(n, 0.0), std::vector<double>(n, 0.0), std::vector<double>(n, 0.0)};
    std::vector<double> gB(n, 0.0);
    const double coef[4] = {0, 1.0, 0.25, 2.0 / 3.0};
    for (int s = steps - 1; s >= 0; --s) {
        for (int q = 0; q < ng; ++q) {
            const int k = G.idx(gi[q], gj[q]);
            lam.h[k] += 2.0 * (traj[s + 1].h[k] - obs[(size_t)s * ng + q]);
        }
        State ln{std::vector<double>(n, 0.0), std::vector<double>(n, 0.0), std::vector<double>(n, 0.0)};
        const State *src[4] = {nullptr, &traj[s], &S1[s], &S2[s]};
        const std::vector<unsigned char> *mk[4] = {nullptr, &M1[s], &M2[s], &M3[s]};
        for (int stage = 3; stage >= 1; --stage) {
            State pre = lam, w = lam, out{std::vector<double>(n, 0.0), std::vector<double>(n, 0.0),
                                          std::vector<double>(n, 0.0)};
            for (size_t k = 0; k < n; ++k) {
                const bool clamped = (*mk[stage])[k];
                pre.h[k] = clamped ? 0.0 : lam.h[k];
                pre.hu[k] = clamped ? 0.0 : lam.hu[k];
                pre.hv[k] = clamped ? 0.0 : lam.hv[k];
                w.h[k] = coef[stage] * dt * pre.h[k];
                w.hu[k] = coef[stage] * dt * pre.hu[k];
                w.hv[k] = coef[stage] * dt * pre.hv[k];
            }
            rhs_vjp(G, *src[stage], B, w, out, gB);
            for (size_t k = 0; k < n; ++k) {
                out.h[k] += coef[stage] * pre.h[k];
                out.hu[k] += coef[stage] * pre.hu[k];
                out.hv[k] += coef[stage] * pre.hv[k];
                if (stage == 3) {
                    ln.h[k] = pre.h[k] / 3.0;
                    ln.hu[k] = pre.hu[k] / 3.0;
                    ln.hv[k] = pre.hv[k] / 3.0;
                } else if (stage == 2) {
                    ln.h[k] += 0.75 * pre.h[k];
                    ln.hu[k] += 0.75 * pre.hu[k];
                    ln.hv[k] += 0.75 * pre.hv[k];
                } else {
                    out.h[k] += ln.h[k];
                    out.hu[k] += ln.hu[k];
                    out.hv[k] += ln.hv[k];
                }
            }
            lam = out;
        }
    }
    std::memcpy(gh, lam.h.data(), n * sizeof(double));
    std::memcpy(ghu, lam.hu.data(), n * sizeof(double));
    std::memcpy(ghv, lam.hv.data(), n * sizeof(double));
    std::memcpy(gBout, gB.data(), n * sizeof(double));
    return J;
}

}  // extern "C"

extern "C" {
// L(U) on the interior (ghosted arrays), and the VJP of w . L(U) w.r.t. U and B.
void adjref_rhs(int Nx, int Ny, double Lx, double Ly, double g, int bc, const double *h,
                const double *hu, const double *hv, const double *B, double *rh, double *rhu,
                double *rhv) {
    Grid G{Nx, Ny, bc, Lx / Nx, Ly / Ny, g};
    const size_t n = G.n();
    State U{std::vector<double>(h, h + n), std::vector<double>(hu, hu + n),
            std::vector<double>(hv, hv + n)};
    State R;
    rhs(G, U, B, R);
    std::memcpy(rh, R.h.data(), n * 8);
    std::memcpy(rhu, R.hu.data(), n * 8);
    std::memcpy(rhv, R.hv.data(), n * 8);
}
void adjref_rhs_vjp(int Nx, int Ny, double Lx, double Ly, double g, int bc, const double *h,
                    const double *hu, const double *hv, const double *B, const double *wh,
                    const double *whu, const double *whv, double *gh, double *ghu, double *ghv,
                    double *gBo) {
    Grid G{Nx, Ny, bc, Lx / Nx, Ly / Ny, g};
    const size_t n = G.n();
    State U{std::vector<double>(h, h + n), std::vector<double>(hu, hu + n),
            std::vector<double>(hv, hv + n)};
    State w{std::vector<double>(wh, wh + n), std::vector<double>(whu, whu + n),
            std::vector<double>(whv, whv + n)};
    State gU{std::vector<double>(n, 0.0), std::vector<double>(n, 0.0), std::vector<double>(n, 0.0)};
    std::vector<double> gB(n, 0.0);
    rhs_vjp(G, U, B, w, gU, gB);
    std::memcpy(gh, gU.h.data(), n * 8);
    std::memcpy(ghu, gU.hu.data(), n * 8);
    std::memcpy(ghv, gU.hv.data(), n * 8);
    std::memcpy(gBo, gB.data(), n * 8);
}
}
