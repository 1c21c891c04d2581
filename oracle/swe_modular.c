/* CPU oracle for the reference's modular solver: plain-C restatement of
 * SerialSolver<ReflectingWalls, Recon, Riemann, SSPRK3, Bathymetry>
 * (include/backend/serial/serial_solver.hpp:140-291) with every reconstruction
 * (PiecewiseConst, MUSCL) and Riemann solver (HLL, Rusanov, ROE) it composes, with and
 * without bathymetry.  TEST INFRASTRUCTURE ONLY (see swe_oracle.h): the GPU parity
 * tests use it as the checker, never the shipped library.
 *
 * Each function keeps the reference's operation order, including the association of
 * its CellState and std::array expressions, so that results are bitwise equal when
 * compiled without floating-point contraction (oracle/Makefile).  Single-threaded:
 * it is only run on small grids.
 */
#include "swe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define EPS 1.0e-8     /* constants::eps, include/constants.hpp:5 */
#define H_FLOOR 1.0e-8 /* serial_solver.hpp:454 */

typedef struct {
    double h, hu, hv;
} cs_t; /* CellState, include/core/cell_state.hpp:6-35 */

typedef struct {
    int Nx, Ny, NxT, NyT;
    double dx, dy, g;
} mview_t;

static inline cs_t cs(double h, double hu, double hv) {
    cs_t s = {h, hu, hv};
    return s;
}

static inline double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min */
static inline double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max */

/* CellState::u / v (cell_state.hpp:18-25) */
static inline double cs_u(cs_t s) { return (s.h > EPS) ? (s.hu / s.h) : 0.0; }
static inline double cs_v(cs_t s) { return (s.h > EPS) ? (s.hv / s.h) : 0.0; }

/* RiemannSolver::F and G (riemann/riemann.hpp:10-19) */
static inline cs_t flux_F(double g, cs_t U) {
    return cs(U.hu, cs_u(U) * cs_u(U) * U.h + 0.5 * g * U.h * U.h, U.hu * cs_v(U));
}
static inline cs_t flux_G(double g, cs_t U) {
    return cs(U.hv, U.hu * cs_v(U), U.h * cs_v(U) * cs_v(U) + 0.5 * g * U.h * U.h);
}

/* HLL (riemann/HLL.hpp:10-45).  dir 0: x_flux with u and F; 1: y_flux with v and G.
 * Returns 2 where the reference throws "HLL could not provide dissipation speed." */
static int hll(double g, int dir, cs_t A, cs_t Bs, cs_t *out) {
    const double uA = dir == 0 ? cs_u(A) : cs_v(A), uB = dir == 0 ? cs_u(Bs) : cs_v(Bs);
    const double sR = dmax(uA + sqrt(g * A.h), uB + sqrt(g * Bs.h));
    const double sL = dmin(uA - sqrt(g * A.h), uB - sqrt(g * Bs.h));
    const cs_t FA = dir == 0 ? flux_F(g, A) : flux_G(g, A);
    const cs_t FB = dir == 0 ? flux_F(g, Bs) : flux_G(g, Bs);
    if (sL >= 0.0) {
        *out = FA;
    } else if (sL < 0.0 && sR > 0.0) {
        /* (sR F(A) - sL F(B) + (sL sR)(B - A)) / (sR - sL), component-wise */
        const double ss = sL * sR, d = sR - sL;
        *out = cs((sR * FA.h - sL * FB.h + ss * (Bs.h - A.h)) / d,
                  (sR * FA.hu - sL * FB.hu + ss * (Bs.hu - A.hu)) / d,
                  (sR * FA.hv - sL * FB.hv + ss * (Bs.hv - A.hv)) / d);
    } else if (sR <= 0.0) {
        *out = FB;
    } else {
        return 2;
    }
    return 0;
}

/* Rusanov (riemann/rusanov.hpp:12-30) */
static void rusanov(double g, int dir, cs_t A, cs_t Bs, cs_t *out) {
    const double uA = dir == 0 ? cs_u(A) : cs_v(A), uB = dir == 0 ? cs_u(Bs) : cs_v(Bs);
    const double hB = dmax(Bs.h, 0.0), hA = dmax(A.h, 0.0);
    const double a = dmax(fabs(uA) + sqrt(g * hA), fabs(uB) + sqrt(g * hB));
    const cs_t FA = dir == 0 ? flux_F(g, A) : flux_G(g, A);
    const cs_t FB = dir == 0 ? flux_F(g, Bs) : flux_G(g, Bs);
    const double ha = 0.5 * a;
    *out = cs(0.5 * (FA.h + FB.h) - ha * (Bs.h - A.h), 0.5 * (FA.hu + FB.hu) - ha * (Bs.hu - A.hu),
              0.5 * (FA.hv + FB.hv) - ha * (Bs.hv - A.hv));
}

/* ROE::compute_roe_avg (riemann/ROE.hpp:66-69) */
static inline double roe_avg(double u1, double h1, double u2, double h2) {
    return ((sqrt(h1) * u1) + (sqrt(h2) * u2)) / (sqrt(h1) + sqrt(h2));
}

/* ROE (riemann/ROE.hpp:10-63).  The std::array sums add right operand to left, which
 * is the same IEEE result; 0 and 1 entries of the eigenvectors are multiplied as
 * written (0 * x keeps its sign and NaN). */
static void roe(double g, int dir, cs_t A, cs_t Bs, cs_t *out) {
    const double h = (A.h + Bs.h) / 2.0;
    const double c = sqrt(g * h);
    const double u_roe = roe_avg(cs_u(A), A.h, cs_u(Bs), Bs.h);
    const double v_roe = roe_avg(cs_v(A), A.h, cs_v(Bs), Bs.h);
    const double vn = dir == 0 ? u_roe : v_roe;
    const double l1 = vn - c, l2 = vn, l3 = vn + c;
    double r1[3], r2[3], r3[3];
    if (dir == 0) {
        r1[0] = 1; r1[1] = l1; r1[2] = v_roe;
        r2[0] = 0; r2[1] = 0; r2[2] = 1;
        r3[0] = 1; r3[1] = l3; r3[2] = v_roe;
    } else {
        r1[0] = 1; r1[1] = u_roe; r1[2] = l1;
        r2[0] = 0; r2[1] = 1; r2[2] = 0;
        r3[0] = 1; r3[1] = u_roe; r3[2] = l3;
    }
    const double dh = Bs.h - A.h, dhu = Bs.hu - A.hu, dhv = Bs.hv - A.hv;
    const double dqn = dir == 0 ? dhu : dhv, dqt = dir == 0 ? dhv : dhu;
    const double vt = dir == 0 ? v_roe : u_roe;
    const double alpha1 = 0.5 * (dh - ((dqn - vn * dh) / c));
    const double alpha3 = 0.5 * (dh + ((dqn - vn * dh) / c));
    const double alpha2 = dqt - vt * dh;
    const double w1 = fabs(l1) * alpha1, w2 = fabs(l2) * alpha2, w3 = fabs(l3) * alpha3;
    double s[3];
    for (int k = 0; k < 3; ++k) s[k] = ((r1[k] * w1 + r2[k] * w2) + r3[k] * w3) * 0.5;
    const cs_t FA = dir == 0 ? flux_F(g, A) : flux_G(g, A);
    const cs_t FB = dir == 0 ? flux_F(g, Bs) : flux_G(g, Bs);
    *out = cs(0.5 * (FA.h + FB.h) - s[0], 0.5 * (FA.hu + FB.hu) - s[1],
              0.5 * (FA.hv + FB.hv) - s[2]);
}

static int riemann(double g, int kind, int dir, cs_t A, cs_t Bs, cs_t *out) {
    if (kind == SWE_ORACLE_RIEMANN_HLL) return hll(g, dir, A, Bs, out);
    if (kind == SWE_ORACLE_RIEMANN_RUSANOV)
        rusanov(g, dir, A, Bs, out);
    else
        roe(g, dir, A, Bs, out);
    return 0;
}

/* minmod_scalar (reconstruction/muscl.hpp:7-10) */
static inline double minmod_scalar(double a, double b) {
    if (a * b <= 0.0) return 0.0;
    return (a > 0.0 ? 1.0 : -1.0) * dmin(fabs(a), fabs(b));
}

static inline cs_t at(const mview_t *v, const double *W[3], int i, int j) {
    const size_t k = (size_t)i * v->NyT + j;
    return cs(W[0][k], W[1][k], W[2][k]);
}

/* MUSCL::minmod_x / minmod_y (muscl.hpp:40-66): di, dj pick the direction. */
static cs_t slope(const mview_t *v, const double *W[3], int i, int j, int di, int dj) {
    const cs_t c0 = at(v, W, i, j), cm = at(v, W, i - di, j - dj), cp = at(v, W, i + di, j + dj);
    return cs(minmod_scalar(c0.h - cm.h, cp.h - c0.h), minmod_scalar(c0.hu - cm.hu, cp.hu - c0.hu),
              minmod_scalar(c0.hv - cm.hv, cp.hv - c0.hv));
}

/* U_L / U_B and U_R / U_T of the interface after (i, j) in direction (di, dj):
 * PiecewiseConst (reconstruction/piecewise_const.hpp:11-30) or MUSCL (muscl.hpp:14-37). */
static void reconstruct(const mview_t *v, int recon, const double *W[3], int i, int j, int di,
                        int dj, cs_t *A, cs_t *Bs) {
    const cs_t c0 = at(v, W, i, j), c1 = at(v, W, i + di, j + dj);
    if (recon == SWE_ORACLE_RECON_PIECEWISE_CONST) {
        *A = c0;
        *Bs = c1;
        return;
    }
    const cs_t s0 = slope(v, W, i, j, di, dj), s1 = slope(v, W, i + di, j + dj, di, dj);
    *A = cs(c0.h + 0.5 * s0.h, c0.hu + 0.5 * s0.hu, c0.hv + 0.5 * s0.hv);
    *Bs = cs(c1.h - 0.5 * s1.h, c1.hu - 0.5 * s1.hu, c1.hv - 0.5 * s1.hv);
}

/* ReflectingWalls::apply_BC(State&) (include/boundary/reflecting_walls.hpp:9-50):
 * bottom/top rows over all i first, then left/right columns over all j. */
static void apply_bc(const mview_t *v, double *h, double *hu, double *hv) {
    const int nG = 2, NxT = v->NxT, NyT = v->NyT;
    for (int g = 0; g < nG; ++g) {
        const int jb = nG - 1 - g, jbi = nG + g, jt = NyT - nG + g, jti = NyT - nG - 1 - g;
        for (int i = 0; i < NxT; ++i) {
            const size_t r = (size_t)i * NyT;
            h[r + jb] = h[r + jbi];
            hu[r + jb] = hu[r + jbi];
            hv[r + jb] = -hv[r + jbi];
            h[r + jt] = h[r + jti];
            hu[r + jt] = hu[r + jti];
            hv[r + jt] = -hv[r + jti];
        }
    }
    for (int g = 0; g < nG; ++g) {
        const int il = nG - 1 - g, ili = nG + g, ir = NxT - nG + g, iri = NxT - nG - 1 - g;
        for (int j = 0; j < NyT; ++j) {
            h[(size_t)il * NyT + j] = h[(size_t)ili * NyT + j];
            hu[(size_t)il * NyT + j] = -hu[(size_t)ili * NyT + j];
            hv[(size_t)il * NyT + j] = hv[(size_t)ili * NyT + j];
            h[(size_t)ir * NyT + j] = h[(size_t)iri * NyT + j];
            hu[(size_t)ir * NyT + j] = -hu[(size_t)iri * NyT + j];
            hv[(size_t)ir * NyT + j] = hv[(size_t)iri * NyT + j];
        }
    }
}

typedef struct {
    double *W[3];         /* (eta or h, hu, hv) the reconstruction reads */
    double *fxm[3], *fxp[3], *fym[3], *fyp[3];
    double *rhs[3];       /* ghost entries stay 0, as the reference's rhs_ */
    double *U1[3], *U2[3], *Un1[3];
} mwork_t;

/* FluxAssemblyBathy::compute_x/y_fluxes (flux_assembly/flux_assembly_bathy.hpp:18-192)
 * or, without bathymetry, FluxAssembly (flux_assembly/flux_assembly.hpp:11-45), then
 * FiniteVolumeBathy / FiniteVolume::apply_spatial_operator (finite_volume_bathy.hpp:
 * 14-30, finite_volume.hpp:14-28).  Returns 2 on the HLL failure. */
static int compute_rhs(const mview_t *v, int recon, int kind, int bathy, const double *U[3],
                       const double *B, mwork_t *w) {
    const size_t n = (size_t)v->NxT * v->NyT;
    const double g = v->g;
    for (size_t k = 0; k < n; ++k) {
        w->W[0][k] = bathy ? U[0][k] + B[k] : U[0][k];  /* W.h() += B */
        w->W[1][k] = U[1][k];
        w->W[2][k] = U[2][k];
    }
    const double *W[3] = {w->W[0], w->W[1], w->W[2]};
    for (int dir = 0; dir < 2; ++dir) {
        const int di = dir == 0 ? 1 : 0, dj = 1 - di;
        const int i0 = dir == 0 ? 1 : 2, i1 = 2 + v->Nx, j0 = dir == 0 ? 2 : 1, j1 = 2 + v->Ny;
        double **fm = dir == 0 ? w->fxm : w->fym, **fp = dir == 0 ? w->fxp : w->fyp;
        for (int i = i0; i < i1; ++i)
            for (int j = j0; j < j1; ++j) {
                const size_t k = (size_t)i * v->NyT + j;
                cs_t A, Bs, F;
                reconstruct(v, recon, W, i, j, di, dj, &A, &Bs);
                if (!bathy) {
                    if (riemann(g, kind, dir, A, Bs, &F)) return 2;
                    fm[0][k] = F.h;
                    fm[1][k] = F.hu;
                    fm[2][k] = F.hv;
                    continue;
                }
                const double eta_m = A.h, eta_p = Bs.h;
                const double b_m = B[k], b_p = B[k + (size_t)di * v->NyT + dj];
                const double b_star = dmax(b_m, b_p);
                const double h_m = dmax(0.0, eta_m - b_m), h_p = dmax(0.0, eta_p - b_p);
                /* safe_velocity (flux_assembly_bathy.hpp:180-185) */
                const double u_m = (h_m < EPS) ? 0.0 : A.hu / h_m;
                const double v_m = (h_m < EPS) ? 0.0 : A.hv / h_m;
                const double u_p = (h_p < EPS) ? 0.0 : Bs.hu / h_p;
                const double v_p = (h_p < EPS) ? 0.0 : Bs.hv / h_p;
                const double hs_m = dmax(0.0, eta_m - b_star), hs_p = dmax(0.0, eta_p - b_star);
                const cs_t Um = cs(hs_m, hs_m * u_m, hs_m * v_m);
                const cs_t Up = cs(hs_p, hs_p * u_p, hs_p * v_p);
                if (riemann(g, kind, dir, Um, Up, &F)) return 2;
                const double corr_m = 0.5 * g * (h_m * h_m - hs_m * hs_m);
                const double corr_p = 0.5 * g * (h_p * h_p - hs_p * hs_p);
                fm[0][k] = F.h;
                fp[0][k] = F.h;
                if (dir == 0) {
                    fm[1][k] = F.hu + corr_m;
                    fp[1][k] = F.hu + corr_p;
                    fm[2][k] = F.hv;
                    fp[2][k] = F.hv;
                } else {
                    fm[1][k] = F.hu;
                    fp[1][k] = F.hu;
                    fm[2][k] = F.hv + corr_m;
                    fp[2][k] = F.hv + corr_p;
                }
            }
    }
    double **xp = bathy ? w->fxp : w->fxm, **yp = bathy ? w->fyp : w->fym;
    for (int i = 2; i < 2 + v->Nx; ++i)
        for (int j = 2; j < 2 + v->Ny; ++j) {
            const size_t k = (size_t)i * v->NyT + j;
            for (int f = 0; f < 3; ++f)
                w->rhs[f][k] = (-1.0 / v->dx) * (w->fxm[f][k] - xp[f][k - v->NyT]) -
                               (1.0 / v->dy) * (w->fym[f][k] - yp[f][k - 1]);
        }
    return 0;
}

/* serial_solver.hpp:453-478: interior floor, then the finiteness test. */
static int enforce_positivity(const mview_t *v, double *h, double *hu, double *hv) {
    for (int i = 2; i < 2 + v->Nx; ++i)
        for (int j = 2; j < 2 + v->Ny; ++j) {
            const size_t k = (size_t)i * v->NyT + j;
            if (h[k] < H_FLOOR) {
                h[k] = H_FLOOR;
                hu[k] = 0.0;
                hv[k] = 0.0;
            }
            if (!isfinite(h[k]) || !isfinite(hu[k]) || !isfinite(hv[k])) return 1;
        }
    return 0;
}

int swe_oracle_modular_run(const swe_oracle_grid *p, int recon, int kind, int bathy, int steps,
                           double dt, double *h, double *hu, double *hv, const double *B,
                           double *t_inout) {
    mview_t v;
    v.Nx = p->Nx;
    v.Ny = p->Ny;
    v.NxT = p->Nx + 4;
    v.NyT = p->Ny + 4;
    v.dx = p->dx > 0.0 ? p->dx : p->Lx / p->Nx;
    v.dy = p->dy > 0.0 ? p->dy : p->Ly / p->Ny;
    v.g = p->g;
    const size_t n = (size_t)v.NxT * v.NyT;
    double *mem = (double *)calloc(27 * n, sizeof(double));
    if (!mem) return -1;
    mwork_t w;
    for (int f = 0; f < 3; ++f) {
        w.W[f] = mem + (0 + f) * n;
        w.fxm[f] = mem + (3 + f) * n;
        w.fxp[f] = mem + (6 + f) * n;
        w.fym[f] = mem + (9 + f) * n;
        w.fyp[f] = mem + (12 + f) * n;
        w.rhs[f] = mem + (15 + f) * n;
        w.U1[f] = mem + (18 + f) * n;
        w.U2[f] = mem + (21 + f) * n;
        w.Un1[f] = mem + (24 + f) * n;
    }
    /* SSPRK3 coefficients (ssp_rk3.hpp:12-37) */
    const double c2 = dt / 4.0, c3 = 2.0 * dt / 3.0;
    double *Un[3] = {h, hu, hv};
    double t = t_inout ? *t_inout : 0.0;
    int st = 0;
    for (int step = 0; step < steps && st == 0; ++step) {
        /* serial_solver.hpp:183-244 (bathymetry) and 247-306 (without) */
        apply_bc(&v, Un[0], Un[1], Un[2]);
        const double *S0[3] = {Un[0], Un[1], Un[2]};
        if ((st = compute_rhs(&v, recon, kind, bathy, S0, B, &w))) break;
        for (int f = 0; f < 3; ++f)
            for (size_t k = 0; k < n; ++k) w.U1[f][k] = 1.0 * Un[f][k] + dt * w.rhs[f][k];
        if (bathy && (st = enforce_positivity(&v, w.U1[0], w.U1[1], w.U1[2]))) break;

        apply_bc(&v, w.U1[0], w.U1[1], w.U1[2]);
        const double *S1[3] = {w.U1[0], w.U1[1], w.U1[2]};
        if ((st = compute_rhs(&v, recon, kind, bathy, S1, B, &w))) break;
        for (int f = 0; f < 3; ++f)
            for (size_t k = 0; k < n; ++k)
                w.U2[f][k] = 3.0 / 4.0 * Un[f][k] + 1.0 / 4.0 * w.U1[f][k] + c2 * w.rhs[f][k];
        if (bathy && (st = enforce_positivity(&v, w.U2[0], w.U2[1], w.U2[2]))) break;

        apply_bc(&v, w.U2[0], w.U2[1], w.U2[2]);
        const double *S2[3] = {w.U2[0], w.U2[1], w.U2[2]};
        if ((st = compute_rhs(&v, recon, kind, bathy, S2, B, &w))) break;
        for (int f = 0; f < 3; ++f)
            for (size_t k = 0; k < n; ++k)
                w.Un1[f][k] = 1.0 / 3.0 * Un[f][k] + 2.0 / 3.0 * w.U2[f][k] + c3 * w.rhs[f][k];
        if (bathy && (st = enforce_positivity(&v, w.Un1[0], w.Un1[1], w.Un1[2]))) break;
        for (int f = 0; f < 3; ++f) memcpy(Un[f], w.Un1[f], n * sizeof(double));
        t += dt;
        apply_bc(&v, Un[0], Un[1], Un[2]);
    }
    if (t_inout) *t_inout = t;
    free(mem);
    return st;
}

/* compute_stable_dt of include/solver_assembly/time_utils.hpp:14-38, the CFL guard of
 * SerialSolver::run (serial_solver.hpp:148-157).  Returns 0, or 1 where the reference
 * throws on h < 0. */
int swe_oracle_modular_stable_dt(const swe_oracle_grid *p, const double *h, const double *hu,
                                 const double *hv, double *out) {
    const double dx = p->dx > 0.0 ? p->dx : p->Lx / p->Nx;
    const double dy = p->dy > 0.0 ? p->dy : p->Ly / p->Ny;
    const int NyT = p->Ny + 4;
    double lim = 1.7976931348623157e308; /* std::numeric_limits<double>::max() */
    for (int i = 2; i < 2 + p->Nx; ++i)
        for (int j = 2; j < 2 + p->Ny; ++j) {
            const size_t k = (size_t)i * NyT + j;
            if (h[k] < 0.0) return 1;
            const double u = hu[k] / h[k], v = hv[k] / h[k];
            const double dt_cell = p->cfl / ((fabs(u) + sqrt(p->g * h[k])) / dx +
                                             (fabs(v) + sqrt(p->g * h[k])) / dy);
            lim = dmin(lim, dt_cell);
        }
    *out = lim;
    return 0;
}
