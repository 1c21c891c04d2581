/* CPU oracle for the MUSCL + hydrostatic-reconstruction + HLL + SSP-RK3 hot path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C restatement of the reference's optimised
 * serial/OpenMP solver (include/backend/serial/HPC/HPC_kernels.hpp,
 * include/backend/serial/HPC/HPC_solver.hpp, include/backend/openmp/omp_kernels.hpp).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as
 * the checker or the timed CPU baseline; the shipped library never links it.
 *
 * Layout: full ghosted row-major arrays, nG = 2, Nx_total = Nx + 4,
 * Ny_total = Ny + 4, index k = i * Ny_total + j (i = x, slow; j = y, contiguous),
 * as HPC_kernels.hpp:18-31 and include/core/array2D.hpp:33.
 *
 * Parity is pinned against the reference compiled from its own sources
 * (oracle/_ref, tests/test_oracle_ref.py) and against tests/golden/.
 */
#ifndef SWE_ORACLE_H
#define SWE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

enum { SWE_ORACLE_BC_REFLECTING = 0, SWE_ORACLE_BC_TRANSMISSIVE = 1 };

typedef struct swe_oracle_grid {
    int Nx, Ny;   /* interior cells */
    double Lx, Ly;/* domain lengths: dx = Lx / Nx, dy = Ly / Ny (include/core/grid.hpp:19-20) */
    double g;     /* gravity; the reference hard-codes 9.80665 (include/constants.hpp:4) */
    double cfl;   /* CFL number for compute_stable_dt */
    int bc;       /* SWE_ORACLE_BC_* */
    int threads;  /* OpenMP threads; <= 0 uses the OpenMP default */
    double dx, dy;/* > 0: cell sizes used instead of Lx / Nx, Ly / Ny (a slab of a grid) */
} swe_oracle_grid;

/* Runs `steps` SSP-RK3 steps in place on h, hu, hv (ghosts refreshed on return).
 * dt_fixed > 0: every step uses it (HPC_solver.hpp:94).  Otherwise dt is
 * compute_stable_dt(U^n) before each step.  dt_log (optional) receives each dt,
 * *t_inout (optional) accumulates time += dt (HPC_solver.hpp:170).
 * Returns 0, or 1 when enforce_positivity meets a non-finite state
 * (HPC_kernels.hpp:310-312); the state is then left as of that stage. */
int swe_oracle_run(const swe_oracle_grid *p, int steps, double dt_fixed, double *h, double *hu,
                   double *hv, const double *B, double *dt_log, double *t_inout);

/* Reusable work buffers (flux, rhs and stage arrays) for repeated runs on one grid
 * size, so timed runs exclude allocation like the reference, which allocates in its
 * constructor (HPC_solver.hpp:97-103). */
typedef struct swe_oracle_ws swe_oracle_ws;
swe_oracle_ws *swe_oracle_ws_create(const swe_oracle_grid *p);
void swe_oracle_ws_destroy(swe_oracle_ws *ws);

/* swe_oracle_run on a workspace from swe_oracle_ws_create for the same grid. */
int swe_oracle_run_ws(const swe_oracle_grid *p, swe_oracle_ws *ws, int steps, double dt_fixed,
                      double *h, double *hu, double *hv, const double *B, double *dt_log,
                      double *t_inout);

/* One RK stage: out = combine(stage, U^n, U^src, dt * L(U^src)), positivity applied and
 * ghosts refreshed.  stage 1: U1 = Us + dt L; 2: 0.75 Un + 0.25 (Us + dt L);
 * 3: 1/3 Un + 2/3 (Us + dt L) (HPC_solver.hpp:244-301).  Un is unused for stage 1.
 * The ghosts of the source must already be valid.  Returns as swe_oracle_run. */
int swe_oracle_stage(const swe_oracle_grid *p, int stage, double dt, const double *hn,
                     const double *hun, const double *hvn, const double *hs, const double *hus,
                     const double *hvs, const double *B, double *ho, double *huo, double *hvo);

/* compute_stable_dt (HPC_kernels.hpp:281-298); 1e100 when the max speed <= 1e-8. */
double swe_oracle_stable_dt(const swe_oracle_grid *p, const double *h, const double *hu,
                            const double *hv);

/* Max over interior cells of max(|u| + c, |v| + c), c = sqrt(g max(0, h)). */
double swe_oracle_max_wave_speed(const swe_oracle_grid *p, const double *h, const double *hu,
                                 const double *hv);

/* Ghost refresh: reflecting walls as apply_reflecting_bc (HPC_solver.hpp:320-371),
 * or zero-gradient copies for transmissive walls (no reference counterpart). */
void swe_oracle_fill_ghosts(const swe_oracle_grid *p, double *h, double *hu, double *hv);

/* Scalar ghost mirror for the bathymetry (apply_scalar_reflecting_bc,
 * HPC_solver.hpp:373-404), or zero-gradient copies for transmissive walls. */
void swe_oracle_fill_scalar_ghosts(const swe_oracle_grid *p, double *a);

/* ---- The modular solver (oracle/swe_modular.c) -------------------------------------
 * SerialSolver<ReflectingWalls, Recon, Riemann, SSPRK3, Bathymetry>
 * (include/backend/serial/serial_solver.hpp:140-291), restated for every
 * reconstruction and Riemann solver it composes. */
enum { SWE_ORACLE_RECON_PIECEWISE_CONST = 0, SWE_ORACLE_RECON_MUSCL = 1 };
enum { SWE_ORACLE_RIEMANN_HLL = 0, SWE_ORACLE_RIEMANN_RUSANOV = 1, SWE_ORACLE_RIEMANN_ROE = 2 };

/* `steps` fixed-dt steps in place on h, hu, hv (reflecting walls; ghosts refreshed on
 * return).  bathy != 0: FluxAssemblyBathy, FiniteVolumeBathy and enforce_positivity (the
 * Flat / GaussHill instantiations); 0: FluxAssembly and FiniteVolume (None).  B is read
 * only when bathy != 0.  *t_inout accumulates time += dt.  Returns 0; 1 where the
 * reference throws "non-finite state detected in positivity correction"; 2 where HLL
 * throws "HLL could not provide dissipation speed."; -1 on allocation failure. */
int swe_oracle_modular_run(const swe_oracle_grid *p, int recon, int riemann, int bathy,
                           int steps, double dt, double *h, double *hu, double *hv,
                           const double *B, double *t_inout);

/* The modular solver's CFL guard, compute_stable_dt of time_utils.hpp:14-38.  Returns 0,
 * or 1 where the reference throws on h < 0. */
int swe_oracle_modular_stable_dt(const swe_oracle_grid *p, const double *h, const double *hu,
                                 const double *hv, double *out);

#ifdef __cplusplus
}
#endif
#endif
