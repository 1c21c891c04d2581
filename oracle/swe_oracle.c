/* CPU oracle: plain-C restatement of the reference's optimised MUSCL + HLL +
 * hydrostatic-bathymetry SSP-RK3 solver.  TEST INFRASTRUCTURE ONLY (see
 * swe_oracle.h): used by tests/, the smoke check and bench.py's CPU-baseline leg.
 *
 * Every function keeps the reference's operation order so results are bitwise
 * equal to it when compiled without floating-point contraction (oracle/Makefile).
 * The loops are OpenMP-parallel like omp_kernels.hpp:135-330; each cell is
 * written by exactly one iteration and the max-reduction is exact, so the result
 * does not depend on the thread count.
 */
#include "swe_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define EPS 1.0e-8     /* constants::eps, include/constants.hpp:5 */
#define H_FLOOR 1.0e-8 /* enforce_positivity default h_floor, HPC_kernels.hpp:301 */

typedef struct {
    int Nx, Ny, nG, Nx_total, Ny_total, stride;
    double dx, dy, g;
} view_t; /* GridView, HPC_kernels.hpp:18-27 (plus g) */

static view_t make_view(const swe_oracle_grid *p) {
    view_t v;
    v.Nx = p->Nx;
    v.Ny = p->Ny;
    v.nG = 2;
    v.Nx_total = p->Nx + 4;
    v.Ny_total = p->Ny + 4;
    v.stride = v.Ny_total;
    v.dx = p->dx > 0.0 ? p->dx : p->Lx / p->Nx; /* include/core/grid.hpp:19-20 */
    v.dy = p->dy > 0.0 ? p->dy : p->Ly / p->Ny;
    v.g = p->g;
    return v;
}

/* HPC_kernels.hpp:33-35 */
static inline double positive_height(double h) { return h > 0.0 ? h : 0.0; }

/* HPC_kernels.hpp:37-39 */
static inline double safe_velocity(double q, double h) { return (h > EPS) ? (q / h) : 0.0; }

static inline double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min */
static inline double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max */

/* HPC_kernels.hpp:41-44 */
static inline double minmod(double a, double b) {
    if (a * b <= 0.0) return 0.0;
    return (a > 0.0 ? 1.0 : -1.0) * dmin(fabs(a), fabs(b));
}

/* hll_x (HPC_kernels.hpp:46-82); with the roles of hu and hv exchanged it is
 * hll_y (:84-120), which is how the y sweep calls it below. */
static inline void hll_normal(double g, double hL, double qnL, double qtL, double hR,
                              double qnR, double qtR, double *fh, double *fqn, double *fqt) {
    const double unL = safe_velocity(qnL, hL);
    const double utL = safe_velocity(qtL, hL);
    const double unR = safe_velocity(qnR, hR);
    const double utR = safe_velocity(qtR, hR);

    const double cL = sqrt(g * hL);
    const double cR = sqrt(g * hR);

    const double sL = dmin(unL - cL, unR - cR);
    const double sR = dmax(unL + cL, unR + cR);

    const double FL_h = qnL;
    const double FL_n = qnL * unL + 0.5 * g * hL * hL;
    const double FL_t = qnL * utL;

    const double FR_h = qnR;
    const double FR_n = qnR * unR + 0.5 * g * hR * hR;
    const double FR_t = qnR * utR;

    if (sL >= 0.0) {
        *fh = FL_h;
        *fqn = FL_n;
        *fqt = FL_t;
    } else if (sR <= 0.0) {
        *fh = FR_h;
        *fqn = FR_n;
        *fqt = FR_t;
    } else {
        const double inv = 1.0 / (sR - sL);
        *fh = (sR * FL_h - sL * FR_h + sL * sR * (hR - hL)) * inv;
        *fqn = (sR * FL_n - sL * FR_n + sL * sR * (qnR - qnL)) * inv;
        *fqt = (sR * FL_t - sL * FR_t + sL * sR * (qtR - qtL)) * inv;
    }
}

/* One interface of compute_x_fluxes (HPC_kernels.hpp:136-184) / compute_y_fluxes
 * (:203-251) between cell a (minus side) and cell b = a + d (plus side); d is the
 * stride for x-faces and 1 for y-faces.  qn is the normal momentum (hu for x,
 * hv for y), qt the tangential one.  Outputs the common fluxes fh, fqt, and the
 * normal-momentum flux with the minus / plus hydrostatic corrections. */
static inline void face_flux(const view_t *v, const double *h, const double *qn,
                             const double *qt, const double *B, int k, int d, double *fh,
                             double *fqt, double *fqn_m, double *fqn_p) {
    const int kr = k + d;
    const double g = v->g;

    const double eta_im1 = h[k - d] + B[k - d];
    const double eta_i = h[k] + B[k];
    const double eta_ip1 = h[kr] + B[kr];
    const double eta_ip2 = h[kr + d] + B[kr + d];

    const double eta_minus = eta_i + 0.5 * minmod(eta_i - eta_im1, eta_ip1 - eta_i);
    const double eta_plus = eta_ip1 - 0.5 * minmod(eta_ip1 - eta_i, eta_ip2 - eta_ip1);

    /* The reference names these hu_* / hv_*; for the y sweep hu is tangential. */
    const double qn_minus = qn[k] + 0.5 * minmod(qn[k] - qn[k - d], qn[kr] - qn[k]);
    const double qt_minus = qt[k] + 0.5 * minmod(qt[k] - qt[k - d], qt[kr] - qt[k]);
    const double qn_plus = qn[kr] - 0.5 * minmod(qn[kr] - qn[k], qn[kr + d] - qn[kr]);
    const double qt_plus = qt[kr] - 0.5 * minmod(qt[kr] - qt[k], qt[kr + d] - qt[kr]);

    const double b_minus = B[k];
    const double b_plus = B[kr];
    const double b_star = dmax(b_minus, b_plus);

    const double h_minus = positive_height(eta_minus - b_minus);
    const double h_plus = positive_height(eta_plus - b_plus);

    const double un_minus = safe_velocity(qn_minus, h_minus);
    const double ut_minus = safe_velocity(qt_minus, h_minus);
    const double un_plus = safe_velocity(qn_plus, h_plus);
    const double ut_plus = safe_velocity(qt_plus, h_plus);

    const double hs_minus = positive_height(eta_minus - b_star);
    const double hs_plus = positive_height(eta_plus - b_star);

    double f_h, f_n, f_t;
    hll_normal(g, hs_minus, hs_minus * un_minus, hs_minus * ut_minus, hs_plus,
               hs_plus * un_plus, hs_plus * ut_plus, &f_h, &f_n, &f_t);

    const double corr_minus = 0.5 * g * (h_minus * h_minus - hs_minus * hs_minus);
    const double corr_plus = 0.5 * g * (h_plus * h_plus - hs_plus * hs_plus);

    *fh = f_h;
    *fqt = f_t;
    *fqn_m = f_n + corr_minus;
    *fqn_p = f_n + corr_plus;
}

typedef struct {
    double *xm[3], *xp[3], *ym[3], *yp[3]; /* [h, hu, hv] flux arrays, HPC_solver.hpp:470-473 */
    double *rhs[3];
} work_t;

/* compute_x_fluxes (HPC_kernels.hpp:122-187): faces i+1/2, i in [nG-1, nG+Nx). */
static void compute_x_fluxes(const view_t *v, const double *h, const double *hu,
                             const double *hv, const double *B, work_t *w) {
    const int s = v->stride, nG = v->nG;
#pragma omp parallel for schedule(static)
    for (int i = nG - 1; i < nG + v->Nx; ++i) {
        for (int j = nG; j < nG + v->Ny; ++j) {
            const int k = i * s + j;
            double fh, fhv, fhu_m, fhu_p;
            face_flux(v, h, hu, hv, B, k, s, &fh, &fhv, &fhu_m, &fhu_p);
            w->xm[0][k] = fh;
            w->xm[1][k] = fhu_m;
            w->xm[2][k] = fhv;
            w->xp[0][k] = fh;
            w->xp[1][k] = fhu_p;
            w->xp[2][k] = fhv;
        }
    }
}

/* compute_y_fluxes (HPC_kernels.hpp:189-254): faces j+1/2, j in [nG-1, nG+Ny). */
static void compute_y_fluxes(const view_t *v, const double *h, const double *hu,
                             const double *hv, const double *B, work_t *w) {
    const int s = v->stride, nG = v->nG;
#pragma omp parallel for schedule(static)
    for (int i = nG; i < nG + v->Nx; ++i) {
        for (int j = nG - 1; j < nG + v->Ny; ++j) {
            const int k = i * s + j;
            double gh, ghu, ghv_m, ghv_p;
            face_flux(v, h, hv, hu, B, k, 1, &gh, &ghu, &ghv_m, &ghv_p);
            w->ym[0][k] = gh;
            w->ym[1][k] = ghu;
            w->ym[2][k] = ghv_m;
            w->yp[0][k] = gh;
            w->yp[1][k] = ghu;
            w->yp[2][k] = ghv_p;
        }
    }
}

/* apply_divergence (HPC_kernels.hpp:256-279). */
static void apply_divergence(const view_t *v, work_t *w) {
    const int s = v->stride;
    const double inv_dx = 1.0 / v->dx;
    const double inv_dy = 1.0 / v->dy;
#pragma omp parallel for schedule(static)
    for (int i = v->nG; i < v->nG + v->Nx; ++i) {
        for (int j = v->nG; j < v->nG + v->Ny; ++j) {
            const int k = i * s + j;
            for (int c = 0; c < 3; ++c) {
                w->rhs[c][k] = -inv_dx * (w->xm[c][k] - w->xp[c][k - s]) -
                               inv_dy * (w->ym[c][k] - w->yp[c][k - 1]);
            }
        }
    }
}

/* enforce_positivity (HPC_kernels.hpp:300-315); returns 1 on a non-finite state. */
static int enforce_positivity(const view_t *v, double *h, double *hu, double *hv) {
    int nonfinite = 0;
#pragma omp parallel for schedule(static) reduction(max : nonfinite)
    for (int i = v->nG; i < v->nG + v->Nx; ++i) {
        for (int j = v->nG; j < v->nG + v->Ny; ++j) {
            const int k = i * v->stride + j;
            if (h[k] < H_FLOOR) {
                h[k] = H_FLOOR;
                hu[k] = 0.0;
                hv[k] = 0.0;
            }
            if (!isfinite(h[k]) || !isfinite(hu[k]) || !isfinite(hv[k])) nonfinite = 1;
        }
    }
    return nonfinite;
}

/* Ghost refresh.  Reflecting: apply_reflecting_bc (HPC_solver.hpp:320-371), x-ghost
 * rows for interior j (hu negated), then y-ghost columns over all rows (hv negated).
 * Transmissive (no reference counterpart): the same two sweeps, copying the
 * nearest interior row / column unchanged. */
static void fill_ghosts(const view_t *v, int bc, double *h, double *hu, double *hv) {
    const int nG = v->nG, Nx = v->Nx, Ny = v->Ny, s = v->stride;
    const int refl = (bc == SWE_ORACLE_BC_REFLECTING);
    for (int gi = 0; gi < nG; ++gi) {
        const int iL = nG - 1 - gi, iR = nG + Nx + gi;
        const int iSL = refl ? nG + gi : nG;
        const int iSR = refl ? nG + Nx - 1 - gi : nG + Nx - 1;
        for (int j = nG; j < nG + Ny; ++j) {
            const int kL = iL * s + j, kSL = iSL * s + j;
            const int kR = iR * s + j, kSR = iSR * s + j;
            h[kL] = h[kSL];
            hu[kL] = refl ? -hu[kSL] : hu[kSL];
            hv[kL] = hv[kSL];
            h[kR] = h[kSR];
            hu[kR] = refl ? -hu[kSR] : hu[kSR];
            hv[kR] = hv[kSR];
        }
    }
    for (int gj = 0; gj < nG; ++gj) {
        const int jB = nG - 1 - gj, jT = nG + Ny + gj;
        const int jSB = refl ? nG + gj : nG;
        const int jST = refl ? nG + Ny - 1 - gj : nG + Ny - 1;
        for (int i = 0; i < v->Nx_total; ++i) {
            const int kB = i * s + jB, kSB = i * s + jSB;
            const int kT = i * s + jT, kST = i * s + jST;
            h[kB] = h[kSB];
            hu[kB] = hu[kSB];
            hv[kB] = refl ? -hv[kSB] : hv[kSB];
            h[kT] = h[kST];
            hu[kT] = hu[kST];
            hv[kT] = refl ? -hv[kST] : hv[kST];
        }
    }
}

void swe_oracle_fill_ghosts(const swe_oracle_grid *p, double *h, double *hu, double *hv) {
    const view_t v = make_view(p);
    fill_ghosts(&v, p->bc, h, hu, hv);
}

/* apply_scalar_reflecting_bc (HPC_solver.hpp:373-404) or its zero-gradient twin. */
void swe_oracle_fill_scalar_ghosts(const swe_oracle_grid *p, double *a) {
    const view_t v = make_view(p);
    const int nG = v.nG, Nx = v.Nx, Ny = v.Ny, s = v.stride;
    const int refl = (p->bc == SWE_ORACLE_BC_REFLECTING);
    for (int gi = 0; gi < nG; ++gi) {
        const int iL = nG - 1 - gi, iR = nG + Nx + gi;
        const int iSL = refl ? nG + gi : nG;
        const int iSR = refl ? nG + Nx - 1 - gi : nG + Nx - 1;
        for (int j = nG; j < nG + Ny; ++j) {
            a[iL * s + j] = a[iSL * s + j];
            a[iR * s + j] = a[iSR * s + j];
        }
    }
    for (int gj = 0; gj < nG; ++gj) {
        const int jB = nG - 1 - gj, jT = nG + Ny + gj;
        const int jSB = refl ? nG + gj : nG;
        const int jST = refl ? nG + Ny - 1 - gj : nG + Ny - 1;
        for (int i = 0; i < v.Nx_total; ++i) {
            a[i * s + jB] = a[i * s + jSB];
            a[i * s + jT] = a[i * s + jST];
        }
    }
}

double swe_oracle_max_wave_speed(const swe_oracle_grid *p, const double *h, const double *hu,
                                 const double *hv) {
    const view_t v = make_view(p);
    double max_speed = 0.0;
#pragma omp parallel for schedule(static) reduction(max : max_speed)
    for (int i = v.nG; i < v.nG + v.Nx; ++i) {
        for (int j = v.nG; j < v.nG + v.Ny; ++j) {
            const int k = i * v.stride + j;
            const double hk = h[k];
            const double u = safe_velocity(hu[k], hk);
            const double vv = safe_velocity(hv[k], hk);
            const double c = sqrt(v.g * dmax(0.0, hk));
            max_speed = dmax(max_speed, fabs(u) + c);
            max_speed = dmax(max_speed, fabs(vv) + c);
        }
    }
    return max_speed;
}

/* compute_stable_dt (HPC_kernels.hpp:281-298). */
double swe_oracle_stable_dt(const swe_oracle_grid *p, const double *h, const double *hu,
                            const double *hv) {
    const view_t v = make_view(p);
    const double max_speed = swe_oracle_max_wave_speed(p, h, hu, hv);
    if (max_speed <= EPS) return 1.0e100;
    return p->cfl * dmin(v.dx, v.dy) / max_speed;
}

static int alloc_work(work_t *w, size_t n) {
    double *all = (double *)calloc(15 * n, sizeof(double));
    if (!all) return -1;
    for (int c = 0; c < 3; ++c) {
        w->xm[c] = all + (0 + c) * n;
        w->xp[c] = all + (3 + c) * n;
        w->ym[c] = all + (6 + c) * n;
        w->yp[c] = all + (9 + c) * n;
        w->rhs[c] = all + (12 + c) * n;
    }
    return 0;
}

static void free_work(work_t *w) { free(w->xm[0]); }

/* compute_rhs (HPC_solver.hpp:203-231). */
static void compute_rhs(const view_t *v, const double *h, const double *hu, const double *hv,
                        const double *B, work_t *w) {
    compute_x_fluxes(v, h, hu, hv, B, w);
    compute_y_fluxes(v, h, hu, hv, B, w);
    apply_divergence(v, w);
}

/* The three SSP-RK3 combines of rk3_step (HPC_solver.hpp:244-250, 269-275, 294-301),
 * over all n_total cells (ghost rhs are zero). */
static void rk_combine(int stage, size_t n, double dt, const double *hn, const double *hun,
                       const double *hvn, const double *hs, const double *hus, const double *hvs,
                       double *const *rhs, double *ho, double *huo, double *hvo) {
    const double *rh = rhs[0], *rhu = rhs[1], *rhv = rhs[2];
    if (stage == 1) {
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n; ++k) {
            ho[k] = hs[k] + dt * rh[k];
            huo[k] = hus[k] + dt * rhu[k];
            hvo[k] = hvs[k] + dt * rhv[k];
        }
    } else if (stage == 2) {
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n; ++k) {
            ho[k] = 0.75 * hn[k] + 0.25 * (hs[k] + dt * rh[k]);
            huo[k] = 0.75 * hun[k] + 0.25 * (hus[k] + dt * rhu[k]);
            hvo[k] = 0.75 * hvn[k] + 0.25 * (hvs[k] + dt * rhv[k]);
        }
    } else {
#pragma omp parallel for schedule(static)
        for (size_t k = 0; k < n; ++k) {
            ho[k] = (1.0 / 3.0) * hn[k] + (2.0 / 3.0) * (hs[k] + dt * rh[k]);
            huo[k] = (1.0 / 3.0) * hun[k] + (2.0 / 3.0) * (hus[k] + dt * rhu[k]);
            hvo[k] = (1.0 / 3.0) * hvn[k] + (2.0 / 3.0) * (hvs[k] + dt * rhv[k]);
        }
    }
}

#ifdef _OPENMP
#include <omp.h>
#define SET_THREADS(p)                                                                    \
    int prev_threads_ = omp_get_max_threads();                                            \
    if ((p)->threads > 0) omp_set_num_threads((p)->threads)
#define RESTORE_THREADS() omp_set_num_threads(prev_threads_)
#else
#define SET_THREADS(p)
#define RESTORE_THREADS()
#endif

int swe_oracle_stage(const swe_oracle_grid *p, int stage, double dt, const double *hn,
                     const double *hun, const double *hvn, const double *hs, const double *hus,
                     const double *hvs, const double *B, double *ho, double *huo, double *hvo) {
    const view_t v = make_view(p);
    const size_t n = (size_t)v.Nx_total * (size_t)v.Ny_total;
    work_t w;
    if (alloc_work(&w, n)) return 2;
    SET_THREADS(p);
    compute_rhs(&v, hs, hus, hvs, B, &w);
    rk_combine(stage, n, dt, hn, hun, hvn, hs, hus, hvs, w.rhs, ho, huo, hvo);
    int st = enforce_positivity(&v, ho, huo, hvo);
    fill_ghosts(&v, p->bc, ho, huo, hvo);
    RESTORE_THREADS();
    free_work(&w);
    return st;
}

struct swe_oracle_ws {
    size_t n;
    work_t w;
    double *st; /* U1, U2: 6 arrays */
};

swe_oracle_ws *swe_oracle_ws_create(const swe_oracle_grid *p) {
    const size_t n = (size_t)(p->Nx + 4) * (size_t)(p->Ny + 4);
    swe_oracle_ws *ws = (swe_oracle_ws *)calloc(1, sizeof *ws);
    if (!ws) return NULL;
    ws->n = n;
    ws->st = (double *)calloc(6 * n, sizeof(double));
    if (!ws->st || alloc_work(&ws->w, n)) {
        free(ws->st);
        free(ws);
        return NULL;
    }
    return ws;
}

void swe_oracle_ws_destroy(swe_oracle_ws *ws) {
    if (!ws) return;
    free_work(&ws->w);
    free(ws->st);
    free(ws);
}

/* rk3_step (HPC_solver.hpp:233-318) repeated `steps` times (run loop :168-197). */
int swe_oracle_run_ws(const swe_oracle_grid *p, swe_oracle_ws *ws, int steps, double dt_fixed,
                      double *h, double *hu, double *hv, const double *B, double *dt_log,
                      double *t_inout) {
    const view_t v = make_view(p);
    const size_t n = (size_t)v.Nx_total * (size_t)v.Ny_total;
    if (!ws || ws->n != n) return 2;
    work_t w = ws->w;
    double *st = ws->st;
    double *h1 = st, *hu1 = st + n, *hv1 = st + 2 * n;
    double *h2 = st + 3 * n, *hu2 = st + 4 * n, *hv2 = st + 5 * n;
    int status = 0;
    SET_THREADS(p);
    fill_ghosts(&v, p->bc, h, hu, hv);
    for (int step = 0; step < steps && status == 0; ++step) {
        const double dt = dt_fixed > 0.0 ? dt_fixed : swe_oracle_stable_dt(p, h, hu, hv);
        if (dt_log) dt_log[step] = dt;

        fill_ghosts(&v, p->bc, h, hu, hv);
        compute_rhs(&v, h, hu, hv, B, &w);
        rk_combine(1, n, dt, NULL, NULL, NULL, h, hu, hv, w.rhs, h1, hu1, hv1);
        status = enforce_positivity(&v, h1, hu1, hv1);
        if (status) break;
        fill_ghosts(&v, p->bc, h1, hu1, hv1);

        compute_rhs(&v, h1, hu1, hv1, B, &w);
        rk_combine(2, n, dt, h, hu, hv, h1, hu1, hv1, w.rhs, h2, hu2, hv2);
        status = enforce_positivity(&v, h2, hu2, hv2);
        if (status) break;
        fill_ghosts(&v, p->bc, h2, hu2, hv2);

        compute_rhs(&v, h2, hu2, hv2, B, &w);
        rk_combine(3, n, dt, h, hu, hv, h2, hu2, hv2, w.rhs, h, hu, hv);
        status = enforce_positivity(&v, h, hu, hv);
        fill_ghosts(&v, p->bc, h, hu, hv);
        if (t_inout) *t_inout += dt;
    }
    RESTORE_THREADS();
    return status;
}

int swe_oracle_run(const swe_oracle_grid *p, int steps, double dt_fixed, double *h, double *hu,
                   double *hv, const double *B, double *dt_log, double *t_inout) {
    swe_oracle_ws *ws = swe_oracle_ws_create(p);
    if (!ws) return 2;
    const int st = swe_oracle_run_ws(p, ws, steps, dt_fixed, h, hu, hv, B, dt_log, t_inout);
    swe_oracle_ws_destroy(ws);
    return st;
}
