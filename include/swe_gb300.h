/* swe_gb300.h - C ABI of the GB300 (sm_103a) backend for the shallow-water hot path:
 * MUSCL reconstruction with hydrostatic well-balanced bathymetry, HLL fluxes in x
 * and y, the SSP-RK3 stage update, wall boundary conditions and the CFL
 * max-wave-speed reduction.
 *
 * The reference has no C ABI: its backends are C++ classes that own host and device
 * arrays and call kernels directly (include/backend/cuda/cuda_solver.hpp:107-597).
 * This header is the thin layer a backend class calls instead; each entry point
 * names the reference member it replaces.  Plain pointers and sizes only, no
 * exceptions: every call returns an swe_status and the context keeps a message.
 *
 * Layout contract (include/backend/serial/HPC/HPC_kernels.hpp:18-31,
 * include/core/array2D.hpp:33): host arrays are full ghosted double grids with
 * nG = 2, Nx_total = Nx + 4, Ny_total = Ny + 4, row-major, index
 * k = i * Ny_total + j, i = x (slow), j = y (contiguous).  The library owns all device
 * memory; callers own host buffers, which are copied in and out.
 *
 * Threading: one context per host thread.  Each context owns one CUDA stream;
 * calls are synchronous on return.
 */
#ifndef SWE_GB300_H
#define SWE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWE_GB300_ABI_VERSION 2

typedef enum swe_status {
    SWE_OK = 0,
    SWE_ERR_BAD_ARG = 1,     /* invalid argument or context */
    SWE_ERR_CUDA = 2,        /* a CUDA runtime call failed (CUDA_SOLVER_CHECK, cuda_solver.hpp:36-44) */
    SWE_ERR_NONFINITE = 3,   /* non-finite state after a stage (HPC_kernels.hpp:310-312) */
    SWE_ERR_CFL = 4,         /* fixed dt above the CFL limit (HPC_solver.hpp:142-145) */
    SWE_ERR_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    SWE_ERR_NO_DEVICE = 6,   /* no usable CUDA device */
    SWE_ERR_UNSUPPORTED = 7, /* option not available in this build */
    SWE_ERR_IO = 8           /* an output file could not be created or written (the
                                reference's netCDF::exceptions, netCDF_writer.cpp:20) */
} swe_status;

/* Both wall rules take a ghost row's values from rows next to the same wall, which
 * swe_step_host's band schedule relies on when it fills and copies out the first and
 * last bands while other bands still compute; a rule that wraps across the domain would
 * have to take swe_step_host's three-call path (it does for any other value). */
typedef enum swe_bc {
    SWE_BC_REFLECTING = 0,   /* apply_reflecting_bc, HPC_solver.hpp:320-371 */
    SWE_BC_TRANSMISSIVE = 1  /* zero-gradient ghost copies; no reference counterpart */
} swe_bc;

typedef enum swe_precision {
    SWE_PRECISION_FP64 = 0,       /* the drop-in: bitwise equal to HPC_solver */
    SWE_PRECISION_FP32_MIXED = 1  /* FP32 bulk, FP64 where balance/conservation need it */
} swe_precision;

typedef enum swe_scheme {
    SWE_SCHEME_FUSED = 0,    /* FastHLLMUSCLBathySolver's arithmetic (HPC_solver.hpp, the
                                OptimizedSerial / OpenMP / CUDA backends): the drop-in */
    SWE_SCHEME_MODULAR = 1   /* SerialSolver<ReflectingWalls, reconstruction, riemann,
                                SSPRK3, bathymetry>'s arithmetic (serial_solver.hpp, the
                                Serial backend); FP64, reflecting walls, fixed dt */
} swe_scheme;

typedef enum swe_reconstruction {
    SWE_RECON_PIECEWISE_CONST = 0, /* reconstruction/piecewise_const.hpp */
    SWE_RECON_MUSCL = 1            /* reconstruction/muscl.hpp */
} swe_reconstruction;

typedef enum swe_riemann {
    SWE_RIEMANN_HLL = 0,     /* riemann/HLL.hpp */
    SWE_RIEMANN_RUSANOV = 1, /* riemann/rusanov.hpp */
    SWE_RIEMANN_ROE = 2      /* riemann/ROE.hpp */
} swe_riemann;

typedef struct swe_params {
    int Nx, Ny;       /* interior cells, each >= 2 (mesh.Nx/Ny, configs/config.hpp:21-30) */
    int nG;           /* ghost layers; must be 2 (MUSCL, solver_assembly.hpp validate_config) */
    double Lx, Ly;    /* domain size; dx = Lx / Nx, dy = Ly / Ny (include/core/grid.hpp:19-20) */
    double g;         /* gravity; <= 0 selects the reference's 9.80665 (include/constants.hpp:4) */
    double cfl;       /* CFL number (time.cfl) used by the max-wave-speed reduction */
    int bc;           /* swe_bc */
    int precision;    /* swe_precision */
    int device;       /* CUDA device ordinal */
    int x_halo_lo;    /* nonzero: this grid is an x-slab whose 2 ghost rows below row 0
                         hold the neighbour slab's rows (swe_halo), not the wall rule */
    int x_halo_hi;    /* the same for the 2 ghost rows above row Nx - 1 */
    int reserved;     /* must be zero */
    double dx, dy;    /* > 0: cell sizes used instead of Lx / Nx and Ly / Ny, so that an
                         x-slab keeps its grid's dx exactly; 0: derived */
    int scheme;       /* swe_scheme; the three fields below apply to SWE_SCHEME_MODULAR */
    int reconstruction; /* swe_reconstruction */
    int riemann;      /* swe_riemann */
    int bathymetry;   /* nonzero: FluxAssemblyBathy + FiniteVolumeBathy + positivity (the
                         Flat / GaussHill instantiations); 0: FluxAssembly + FiniteVolume
                         (None), B unused */
} swe_params;

typedef struct swe_ctx swe_ctx; /* opaque */

/* sizeof(swe_params) and sizeof(swe_snapshot_params) as this library was built, so that
 * bindings written in other languages can check their copy of the layout. */
size_t swe_params_size(void);
size_t swe_snapshot_params_size(void);

/* Fills *p with defaults: nG = 2, L = 1, g = 9.80665, cfl = 0.45, reflecting, FP64,
 * the fused scheme (modular fields: MUSCL, HLL, bathymetry on),
 * device 0.  Nx and Ny must still be set. */
void swe_params_default(swe_params *p);

/* Allocates the device state for one grid.  Replaces the backend constructors'
 * allocation (cuda_solver.hpp:109-152, allocate_device :233-252). */
int swe_create(const swe_params *p, swe_ctx **out);

/* Releases device memory and the stream (cuda_solver.hpp:149). NULL is ignored. */
void swe_destroy(swe_ctx *ctx);

/* Copies a full ghosted state and bathymetry from host memory to the device
 * (upload_initial_state_to_device, cuda_solver.hpp:277-286).  Ghost values of
 * h, hu, hv are ignored (the boundary condition defines them); ghost values of B are
 * used as given, as the reference does after apply_scalar_reflecting_bc
 * (HPC_solver.hpp:112-117).  B may be NULL to keep the previous bathymetry. */
int swe_upload(swe_ctx *ctx, const double *h, const double *hu, const double *hv,
               const double *B);

/* Copies the state back with ghosts refreshed by the boundary condition, i.e.
 * exactly the arrays h_, hu_, hv_ of the reference after a step
 * (download_state_from_device, cuda_solver.hpp:288-296). */
int swe_download(swe_ctx *ctx, double *h, double *hu, double *hv);

/* Advances n_steps SSP-RK3 steps (rk3_step, HPC_solver.hpp:233-318, inside the run
 * loop :168-197).  dt > 0: every step uses dt (the reference's fixed
 * end_time / time_steps, HPC_solver.hpp:94).  dt <= 0: adaptive, every step uses
 * cfl * min(dx, dy) / max_wave_speed(U^n) (compute_stable_dt, HPC_kernels.hpp:281-298),
 * reduced on the device inside the last stage of the previous step.  If t_inout is
 * not NULL, *t_inout += dt for every step, in step order (HPC_solver.hpp:170).
 * Returns SWE_ERR_NONFINITE if any stage produced a non-finite interior value (the
 * state is then undefined), checked once per call.  Returns SWE_ERR_TIMEOUT if a tile's
 * TMA copy did not land within its deadline (50 ms): every later tile of the call then
 * returns without work, so the call ends within about two deadlines of the failure; the
 * state is undefined and the context stays usable (upload a state again).
 * SWE_SCHEME_MODULAR: the step loop of SerialSolver::run (serial_solver.hpp:183-244 with
 * bathymetry, 247-306 without); dt must be > 0 (the Serial backend has no adaptive dt),
 * else SWE_ERR_UNSUPPORTED.  SWE_ERR_NONFINITE then also reports where the reference
 * throws: a non-finite state after positivity (with bathymetry) or an HLL interface
 * without a dissipation speed (swe_last_error names which). */
int swe_step(swe_ctx *ctx, int n_steps, double dt, double *t_inout);

/* swe_upload(h, hu, hv, B) + swe_step(n_steps, dt, t_inout) + swe_download(h_out,
 * hu_out, hv_out) in one call, with the same results, for a host that holds the state
 * between steps (the reference's SolverAssembly loop, whose solvers keep h_, hu_, hv_ in
 * host memory).  The FP64 fused scheme on one grid overlaps the transfers with the
 * stage kernels: the state is uploaded in bands of rows while the first stage computes
 * the flux divergence of the bands already resident and reduces their wave speeds (the
 * step's dt is applied once every band is in), and the last stage runs by bands whose
 * rows are copied back while the next band computes.  Host arrays in page-locked memory
 * overlap; pageable ones give the same results without overlap.  The outputs may be the
 * input arrays.  Other forms and slab contexts run the three calls in sequence.  No
 * reference counterpart: the reference's GPU backends upload once and download per
 * output (cuda_solver.hpp:277-296). */
int swe_step_host(swe_ctx *ctx, const double *h, const double *hu, const double *hv,
                  const double *B, double *h_out, double *hu_out, double *hv_out, int n_steps,
                  double dt, double *t_inout);

/* ---- Slabs (x-decomposition over several GPUs) ---------------------------------------
 * The reference's 4-GPU backend splits x into slabs (build_subdomains,
 * cuda_solver_4gpu.hpp:281-304) and exchanges two ghost rows per neighbour after every
 * stage.  A slab is a context created with x_halo_lo / x_halo_hi set on its interface
 * sides (FP64 only): its stage kernels read those ghost rows as stored, swe_download
 * leaves them as they are, and swe_upload keeps the uploaded ones.  A driver then runs
 * each step as swe_stage(1..3) with one global dt (the max of every slab's
 * swe_max_wave_speed), exchanging the just-written buffer's interface rows with swe_halo
 * after every stage; the result is bitwise that of one grid.  No reference counterpart
 * for the entry points themselves. */

/* One RK stage with fixed dt > 0: stage 1: U1 = Un + dt L(Un); 2: U2 = 3/4 Un +
 * 1/4 (U1 + dt L(U1)); 3: Un = 1/3 Un + 2/3 (U2 + dt L(U2)), after which
 * swe_max_wave_speed reports the new state (HPC_solver.hpp:244-301).  Buffers: stage s
 * writes buffer s % 3 (0: U^n, 1: U^(1), 2: U^(2)).  SWE_ERR_NONFINITE as swe_step. */
int swe_stage(swe_ctx *ctx, int stage, double dt);

/* Interface rows of buffer (0: U^n, 1: U^(1), 2: U^(2)) on side (0: low x, 1: high x).
 * op 0 copies the 2 interior rows next to that side (rows 0, 1 or Nx - 2, Nx - 1) to
 * rows; op 1 copies rows into that side's 2 ghost rows.  rows holds h, hu, hv, each
 * 2 x (Ny + 4) doubles in row order, in host or device memory; synchronous. */
int swe_halo(swe_ctx *ctx, int buffer, int side, int op, double *rows);

/* Max over interior cells of max(|u| + c, |v| + c), c = sqrt(g max(0, h)), of the
 * current state (the reduction inside compute_stable_dt). */
int swe_max_wave_speed(swe_ctx *ctx, double *out);

/* compute_stable_dt of the current state (HPC_kernels.hpp:281-298): 1e100 when the
 * max wave speed is <= 1e-8.  The reference's CFL guard (HPC_solver.hpp:134-145) is
 * this value compared with the fixed dt.  SWE_SCHEME_MODULAR: the Serial backend's
 * guard instead, min over cells of cfl / ((|u| + c) / dx + (|v| + c) / dy)
 * (solver_assembly/time_utils.hpp:14-38); SWE_ERR_BAD_ARG where it throws (h < 0). */
int swe_stable_dt(swe_ctx *ctx, double *out);

/* Totals of the current state over the interior, times dx * dy: mass = sum h,
 * momentum_x = sum hu, momentum_y = sum hv.  Compensated FP64 summation of 8-cell chunk
 * sums (error about 9 eps times the sum of magnitudes), deterministic.
 * The reference sums h * dx * dy naively on the host for its MassConservation check
 * (tests/sanity_checks/mass_conservation.hpp:45-56); this is the device-side twin. */
int swe_totals(swe_ctx *ctx, double *mass, double *momentum_x, double *momentum_y);

/* Sanity reductions of the current state on the device, the quantities the reference's
 * sanity checks compute from a downloaded state (tests/sanity_checks/): mass =
 * sum h dx dy (MassConservation, mass_conservation.hpp:45-56; compensated here), h_min
 * = min h over the interior (Debug, debug.hpp:40-57), first_negative = i * Ny + j of the
 * first interior cell in row-major order with h < 0, or -1 (the cell Positivity reports,
 * positivity.hpp:28-40), and energy = sum [ (hu^2 + hv^2) / (2h) (0 where h <= 1e-8)
 * + g h^2 / 2 + g h B ] dx dy (no reference counterpart).  FP32 form: h = eta - B. */
int swe_sanity(swe_ctx *ctx, double *mass, double *h_min, long long *first_negative,
               double *energy);

/* Capacity, in partial-sum blocks, of the fixed scratch used by swe_totals_noalloc. */
#define SWE_TOTALS_NOALLOC_MAX_BLOCKS 1024

/* swe_totals without any allocation, for callers that cannot call cudaMalloc: a host
 * whose device memory all belongs to its own allocator (a framework's caching
 * allocator, a pool sized at start-up), or a time-critical loop that must not stall on
 * cudaMalloc, which can synchronise the device.  No counterpart in the reference.
 *
 * It takes the caller's device arrays instead of a context: h (eta for the FP32-mixed
 * form), hu, hv and, for that form, B, in this library's device layout (ghosted
 * (Nx + 4) x pitch rows, elements of the precision's type), and writes
 * (sum h, sum hu, sum hv) * dxdy to out, three doubles in device memory.  It runs on
 * `stream` (a cudaStream_t; NULL is the default stream) with the device that holds the
 * arrays current, and returns without waiting.  The result equals swe_totals for the
 * same state and block count, bitwise; swe_totals uses four blocks per SM, which
 * blocks = 0 also picks whenever that fits the capacity (up to 256 SMs).
 *
 * Scratch: the per-block partial sums go to one fixed device array of
 * SWE_TOTALS_NOALLOC_MAX_BLOCKS * 6 doubles (48 KiB) inside the library, which every GPU
 * that loads the library holds until the process exits.  `blocks` partial blocks are
 * used (0: four per SM, capped at the capacity); more than SWE_TOTALS_NOALLOC_MAX_BLOCKS
 * returns SWE_ERR_BAD_ARG.  Each block's entries are written before they are read, so
 * the array needs no clearing between calls.  All calls on a device share the one array:
 * calls that overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  The first call on each device looks up the array's
 * address (cudaGetSymbolAddress) in the context current on that device, and looks it up
 * again whenever a later call finds a different current context (a non-primary context,
 * or the primary context after a cudaDeviceReset); make those calls before any stream
 * capture. */
int swe_totals_noalloc(const void *h, const void *hu, const void *hv, const void *B,
                       int precision, int Nx, int Ny, long long pitch, double dxdy, int blocks,
                       double *out, void *stream);

/* Copies the dt of each step of the last swe_step call (up to n values) to out and
 * returns how many were written in *written. */
int swe_dt_log(swe_ctx *ctx, double *out, int n, int *written);

/* Message of the last failed call on ctx ("" when none). */
const char *swe_last_error(const swe_ctx *ctx);

/* Static name of a status code. */
const char *swe_status_string(int status);

/* Number of kernels this library launched on ctx since creation (for accounting). */
long long swe_kernel_launches(const swe_ctx *ctx);

/* Device time in milliseconds of the stage kernels of the last swe_step call,
 * measured with CUDA events on the context's stream (the reference's per-phase
 * timers, HPC_solver.hpp:27-86, time the same loop on the host). */
int swe_last_step_ms(const swe_ctx *ctx, double *ms);

/* ---- Discrete adjoint ------------------------------------------------------------------
 * Gradient of the gauge misfit J = sum over steps n = 1..n_steps and gauges q of
 * (h^n(gauge_i[q], gauge_j[q]) - h_obs[(n - 1) * n_gauges + q])^2 for a run of n_steps
 * fixed-dt steps from the context's current state (left unchanged), through a
 * hand-written discrete adjoint of each RK stage (the derivative of the branches the
 * forward pass takes: minmod, HLL regime, dry guards, positivity clamps).  States are
 * recomputed from n_snapshots stored states on a binomial (optimal offline) checkpoint
 * schedule.  n_snapshots = SWE_ADJ_TAPE_ALL instead keeps every state and every step's
 * stage states and clamp masks from one forward sweep (device memory about
 * (75 n_steps + 400) bytes per cell), so the reverse sweep recomputes nothing.
 * n_snapshots = SWE_ADJ_SEGMENTS cuts the steps into segments of L = round(sqrt(n_steps))
 * steps (counted from the end), stores each segment's start in one forward sweep, then
 * recomputes each segment once, last first, keeping its stage states, and reverses it:
 * every step but the last segment's is advanced twice, in memory for
 * ceil(n_steps / L) + 1 snapshots and a tape of L steps, about
 * (24 n_steps / L + 75 L + 450) bytes per cell.  All schedules give the same J and
 * gradients, bitwise.
 * Outputs, in the ghosted host layout with zero ghosts: J, dJ/dh^0,
 * dJ/dhu^0, dJ/dhv^0 and dJ/dB with the initial state held fixed, where the ghosts of B
 * are taken to follow the wall rule (mirror or copy of the interior).  ms (optional)
 * receives the device time.  On an FP32-mixed context the forward is the FP32 stage
 * kernel and the adjoint runs in FP32 with eta = h + B as the state variable (half the
 * memory; (38 n_steps + 200) bytes per cell in tape mode); the outputs are the same
 * derivatives, widened to double.  With all four gradient pointers NULL only J is
 * computed, by one forward sweep through the same kernels (bitwise the J of a gradient
 * call; n_snapshots is ignored): the objective that finite differences of J need.  Fused
 * scheme only.  No reference counterpart. */
#define SWE_ADJ_TAPE_ALL (-1)
#define SWE_ADJ_SEGMENTS (-2)
int swe_adjoint_gauge(swe_ctx *ctx, int n_steps, double dt, int n_gauges, const int *gauge_i,
                      const int *gauge_j, const double *h_obs, int n_snapshots, double *J,
                      double *grad_h, double *grad_hu, double *grad_hv, double *grad_B,
                      double *ms);

/* ---- One grid over several GPUs of this process ---------------------------------------
 * The grid's rows split into `parts` x-slabs as evenly as possible (build_subdomains,
 * cuda_solver_4gpu.hpp:281-304), slab k on devices[k] (NULL: all on p->device; several
 * slabs may share a device).  A step keeps everything on the devices: every stage runs
 * first on each slab's inner tile rows, then on its two edge tile rows once the
 * neighbours' interface rows have arrived; each slab sends the two rows next to each
 * interface of the buffer it wrote to its neighbours with cudaMemcpyPeerAsync on its own
 * stream (the reference synchronises every device and calls cudaMemcpyPeer,
 * exchange_one_array, cuda_solver_4gpu.hpp:480-505); after stage 3 the slabs' max wave
 * speeds are gathered by 8-byte peer copies and maxed on every device, so all slabs take
 * the same dt.  Results are bitwise those of one context over the whole grid.  FP64
 * fused scheme only (SWE_ERR_UNSUPPORTED otherwise).  Arrays are the whole grid's,
 * ghosted, host layout. */
typedef struct swe_slabs swe_slabs; /* opaque */
int swe_slabs_create(const swe_params *p, int parts, const int *devices, swe_slabs **out);
void swe_slabs_destroy(swe_slabs *g);
int swe_slabs_upload(swe_slabs *g, const double *h, const double *hu, const double *hv,
                     const double *B);
int swe_slabs_download(swe_slabs *g, double *h, double *hu, double *hv);
/* As swe_step: dt > 0 fixed, else the grid's adaptive CFL dt; t_inout advanced. */
int swe_slabs_step(swe_slabs *g, int n_steps, double dt, double *t_inout);
/* Device time of the last swe_slabs_step (events on slab 0's stream, joined by all). */
int swe_slabs_last_step_ms(const swe_slabs *g, double *ms);
long long swe_slabs_kernel_launches(const swe_slabs *g);
const char *swe_slabs_last_error(const swe_slabs *g);

/* ---- Batched ensembles ---------------------------------------------------------------
 * Many independent grids of uneven sizes advanced together: one launch per RK stage
 * covers every instance (a flat work list of (instance, tile) pairs), each instance
 * keeps its own CFL dt, max-speed reduction and time, and whole RK3 steps are replayed
 * from CUDA graphs.  No reference counterpart (the reference runs one grid per process);
 * each instance follows the single-grid semantics above. */

typedef struct swe_ens swe_ens; /* opaque */

/* Tile shapes (rows x columns) the ensemble kernels are compiled for.  FP64: 8x32, 8x16,
 * 4x64, and SWE_SHAPE_STRIP: work items of six 8x32 tiles along x walked by one CTA (the
 * single-grid FP64 kernel's strips).  FP32-mixed: 8x32, 16x32, 8x64, and SWE_SHAPE_COLS:
 * work items of 64 rows by 112 columns swept by column warps (the single-grid FP32
 * kernel's scheme). */
enum { SWE_SHAPE_8x32 = 0, SWE_SHAPE_8x16 = 1, SWE_SHAPE_4x64 = 2, SWE_SHAPE_16x32 = 3,
       SWE_SHAPE_8x64 = 4, SWE_SHAPE_COLS = 5, SWE_SHAPE_STRIP = 6 };

/* n instances with interior sizes Nx[q] x Ny[q] and domain sizes Lx[q] x Ly[q] (NULL:
 * 1.0); g, cfl, bc, precision and device come from *base (its Nx, Ny, Lx, Ly are
 * ignored). */
int swe_ens_create(const swe_params *base, int n, const int *Nx, const int *Ny,
                   const double *Lx, const double *Ly, swe_ens **out);
void swe_ens_destroy(swe_ens *ens);

/* Per-instance upload (state, bathymetry; resets the instance's time to 0) and download,
 * with the single-grid layout of that instance. */
int swe_ens_upload(swe_ens *ens, int instance, const double *h, const double *hu,
                   const double *hv, const double *B);
int swe_ens_download(swe_ens *ens, int instance, double *h, double *hu, double *hv);

/* n_steps RK3 steps of every instance; dt > 0 fixed for all, dt <= 0 per-instance CFL. */
int swe_ens_step(swe_ens *ens, int n_steps, double dt);

/* Per-instance simulation times / dt of the last step (arrays of n doubles). */
int swe_ens_times(swe_ens *ens, double *t);
int swe_ens_last_dt(swe_ens *ens, double *dt);

/* Device time of the last swe_ens_step call (CUDA events on the ensemble's stream). */
int swe_ens_last_step_ms(const swe_ens *ens, double *ms);
long long swe_ens_kernel_launches(const swe_ens *ens);

/* Schedule: tile shape (SWE_SHAPE_*) and CTAs per launch (0: one CTA per tile; a larger
 * grid is capped at the CTAs that fit on the GPU at once, each taking an equal contiguous
 * share of the tiles in FP32). */
int swe_ens_set_schedule(swe_ens *ens, int shape, int grid);
int swe_ens_get_schedule(const swe_ens *ens, int *shape, int *grid, int *total_tiles);

/* Autotuner: times every compiled tile shape with one CTA per tile and with a persistent
 * grid of all / half of the CTAs that fit on the GPU at once, `steps` RK3 steps each, on
 * the uploaded ensemble (the state is restored after every candidate), keeps the fastest
 * and returns its ms per step. */
int swe_ens_tune(swe_ens *ens, int steps, double *best_ms);

const char *swe_ens_last_error(const swe_ens *ens);

/* ---- Snapshot output (NetCDF) ---------------------------------------------------------
 * Replaces NetCDFWriter (include/io/netCDF_writer.hpp:12-55, netCDF_writer.cpp:10-149):
 * the same data model - dimensions time (unlimited), x = Nx, y = Ny; double variables
 * time(time), x(x), y(y), h, hu, hv (time, x, y) and B (x, y); "units" attributes on x,
 * y, h, B and time when their unit is non-empty; the global int save_every; and, set by
 * the first swe_snapshot_metadata call, the global dt, backend, riemann_solver,
 * reconstruction, time_integrator, boundary_condition and bathymetry.  Cell centres are
 * x = (i + 0.5) dx, y = (j + 0.5) dy (include/core/grid.hpp:22-23); fields hold the
 * interior only, x slow and y contiguous (pack_interior_into, netCDF_writer.cpp:73-83).
 *
 * The file is written in the netCDF classic encoding (CDF-2, or CDF-5 when a variable
 * reaches 4 GiB), which netCDF readers open like the reference's netCDF-4 files; no
 * netCDF or HDF5 library is used.
 *
 * swe_snapshot_write takes the state from a context's device memory without stopping
 * it: a kernel on the context's stream packs U^n's interior (byte-swapped to the file's
 * big-endian order) into one of two device staging buffers, and a writer thread copies
 * it to pinned host memory on its own stream, in chunks, and writes the record while
 * the context keeps stepping.  A write blocks only while both staging buffers are
 * still being written out. */
typedef struct swe_snapshot swe_snapshot; /* opaque */

typedef struct swe_snapshot_params {
    int Nx, Ny;           /* interior cells */
    double dx, dy;        /* cell sizes (Lx / Nx, Ly / Ny) */
    const char *unit_x;   /* mesh.spatial_unit_x; NULL or "": no attribute */
    const char *unit_y;   /* mesh.spatial_unit_y */
    const char *unit_h;   /* mesh.spatial_unit_h (h and B) */
    const char *unit_time;/* time.time_unit */
    int save_every;       /* time.save_every, stored as a global attribute */
    int format;           /* 0: CDF-2 when every variable fits it, else CDF-5; 2 or 5 */
} swe_snapshot_params;

/* Creates (replaces) the file, making missing directories, and writes the coordinates
 * (the NetCDFWriter constructor, netCDF_writer.cpp:10-27). */
int swe_snapshot_open(const char *path, const swe_snapshot_params *p, swe_snapshot **out);

/* Writes B's interior from a ghosted host array, once (write_bathymetry, :85-98). */
int swe_snapshot_bathymetry(swe_snapshot *s, const double *B);

/* The run metadata write_snapshot attaches once (:100-133): dt unless NaN, and each
 * string unless NULL or empty.  Applied only by the first call that carries dt or one of
 * the strings after backend, as in the reference; later calls are ignored. */
int swe_snapshot_metadata(swe_snapshot *s, double dt, const char *backend,
                          const char *riemann_solver, const char *reconstruction,
                          const char *time_integrator, const char *boundary_condition,
                          const char *bathymetry);

/* Appends one record from ghosted host arrays, synchronously (write_snapshot, :135-149),
 * after every pending device record. */
int swe_snapshot_write_host(swe_snapshot *s, double time, const double *h, const double *hu,
                            const double *hv);

/* Appends one record of ctx's current state (FP64 as stored; FP32-mixed as
 * swe_download converts it) asynchronously; ctx must match the file's Nx and Ny. */
int swe_snapshot_write(swe_snapshot *s, swe_ctx *ctx, double time);

/* Waits until every record is on disk (in the file); returns the first write error. */
int swe_snapshot_flush(swe_snapshot *s);

/* Records appended so far (written or pending). */
long long swe_snapshot_records(const swe_snapshot *s);

/* Seconds the writer thread spent in device-to-host copies and file writes, and the
 * bytes it wrote, over all device records so far. */
int swe_snapshot_stats(const swe_snapshot *s, double *copy_s, double *write_s,
                       long long *bytes);

/* Flushes and closes the file; the object stays valid for swe_snapshot_last_error. */
int swe_snapshot_close(swe_snapshot *s);
void swe_snapshot_destroy(swe_snapshot *s); /* closes if open, frees; NULL is ignored */
const char *swe_snapshot_last_error(const swe_snapshot *s);

/* ---- Sanity-check records (NetCDF) ----------------------------------------------------
 * Replaces SanityCheckNetCDFWriter (include/io/sanity_checks_netdcdf_writer.hpp,
 * sanity_checks_netcdf_writer.cpp:6-71): dimension record (unlimited); variables
 * step (uint64), time, mass_rel_err, h_min (double) with the reference's long_name and
 * units attributes; globals save_every, dt, backend, riemann_solver, reconstruction,
 * time_integrator, boundary_condition, bathymetry, mass_conservation_enabled = 1 and
 * positivity_enabled = 1.  CDF-5 (the encoding that has uint64).  Pairs with
 * swe_sanity, which computes the mass and h_min on the device. */
typedef struct swe_sanity_log swe_sanity_log; /* opaque */

int swe_sanity_log_open(const char *path, const char *time_unit, const char *h_unit,
                        int save_every, double dt, const char *backend,
                        const char *riemann_solver, const char *reconstruction,
                        const char *time_integrator, const char *boundary_condition,
                        const char *bathymetry, swe_sanity_log **out);
/* One record (SanityCheckNetCDFWriter::write, :61-71). */
int swe_sanity_log_write(swe_sanity_log *l, unsigned long long step, double time,
                         double rel_err, double h_min);
int swe_sanity_log_close(swe_sanity_log *l);
void swe_sanity_log_destroy(swe_sanity_log *l);
const char *swe_sanity_log_last_error(const swe_sanity_log *l);

/* ---- Self-test (no counterpart in the reference) ------------------------------------
 * The FP64 kernels compute double division, square root and part of the multiplications
 * and additions correctly rounded with integer arithmetic instead of FP64 instructions.
 * This runs n operand pairs (hashed from seed: every operand class, physical scales,
 * near-equal pairs, exact quotients and their neighbours) through both those routines
 * and the device's own IEEE operations on the current device, and writes how many
 * results differed (NaN results compare equal to any NaN).  Expected: 0. */
int swe_selftest_soft_f64(long long n, unsigned long long seed, long long *mismatches);

/* The failure path of the stage kernels' bounded TMA waits, run without a fault: `ctas`
 * blocks each arm a transaction barrier for bytes that no copy delivers and wait on it
 * through the stage kernels' own helpers, with a deadline of deadline_ms (0 < d <= 1000).
 * As in a stage launch, every block first reads the flag word and returns at once when
 * an earlier wait gave up.  Returns SWE_ERR_TIMEOUT when the waits gave up as designed
 * (SWE_OK would mean a wait completed), with the number of blocks that waited and the
 * launch's device time.  No copy is issued, so nothing is left in flight. */
int swe_selftest_wait_timeout(int ctas, double deadline_ms, long long *waited_ctas,
                              double *elapsed_ms);

/* Test hooks (no counterpart in the reference): the next swe_step, swe_step_host or
 * swe_stage call (swe_ens_step for an ensemble) starts with its error-flag word holding
 * the timeout bit, as if a TMA wait of an earlier launch had given up.  Every stage tile
 * then returns before staging anything and the call returns SWE_ERR_TIMEOUT; the state is
 * undefined afterwards and the context stays usable. */
int swe_test_preset_timeout(swe_ctx *ctx);
int swe_ens_test_preset_timeout(swe_ens *ens);

#ifdef __cplusplus
}
#endif
#endif /* SWE_GB300_H */
