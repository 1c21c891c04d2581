// Shared definitions of the GB300 shallow-water kernels (device side).
//
// Device layout: each field (h, hu, hv, B) is a ghosted (Nx + 4) x pitch array of
// one element type, row-major, i = x (slow), j = y (contiguous); column j of the
// host layout k = i * (Ny + 4) + j sits at i * pitch + j on the device.  The pitch
// is Ny + 4 rounded up to 32 elements so every row starts 256-byte aligned.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace swe {

constexpr int NG = 2;               // ghost layers (MUSCL needs 2)
constexpr double EPS = 1.0e-8;      // constants::eps, include/constants.hpp:5
constexpr double H_FLOOR = 1.0e-8;  // enforce_positivity h_floor, HPC_kernels.hpp:301

enum : int { BC_REFLECTING = 0, BC_TRANSMISSIVE = 1 };
enum : int { FLAG_NONFINITE = 1, FLAG_TIMEOUT = 2 };

// Per-launch parameters of one RK stage.
struct StageParams {
    const void *hs, *hus, *hvs;  // stage source U^(s) (stencil reads)
    const void *hn, *hun, *hvn;  // U^n (pointwise reads; stages 2 and 3)
    const void *B;               // bathymetry with ghosts
    void *ho, *huo, *hvo;        // stage output (interior cells written)
    int Nx, Ny;                  // interior size
    long long pitch;             // device row pitch in elements
    int bc;                      // BC_*
    double inv_dx, inv_dy;       // 1.0 / dx, 1.0 / dy (host-computed, as apply_divergence)
    int kx, ky;                  // log2 of inv_dx / inv_dy when a power of two, else 127
    double g;                    // gravity
    double half_g;               // 0.5 * g (exact)
    double cfl_min_dxdy;         // cfl * min(dx, dy) (compute_stable_dt numerator)
    double dt_fixed;             // > 0: fixed dt; otherwise adaptive from speed slot
    unsigned long long *speed;   // two max-wave-speed slots (double bit patterns)
    int slot_read;               // slot holding max speed of U^n (adaptive dt)
    int slot_write;              // slot receiving max speed of U^(n+1) (stage 3)
    double *t_accum;             // simulation time, += dt once per step (stage 3)
    double *dt_log;              // optional per-step dt record
    int log_index;               // index into dt_log for this step
    int *flags;                  // FLAG_* bits
};

// Maps a possibly out-of-domain interior coordinate a (0-based, may be -2..N+1 or
// beyond for partial tiles) to the interior cell whose value the ghost holds.
// Reflecting walls mirror (apply_reflecting_bc, HPC_solver.hpp:326-370) and report
// a flip of the normal momentum; transmissive walls clamp.  Coordinates further out
// (only in tiles overhanging the domain, never used) are clamped into range.
__device__ __forceinline__ int map_coord(int a, int N, int bc, bool &flip) {
    flip = false;
    if (a < 0) {
        if (bc == BC_REFLECTING) {
            a = -1 - a;
            flip = true;
        } else {
            a = 0;
        }
    } else if (a >= N) {
        if (bc == BC_REFLECTING) {
            a = 2 * N - 1 - a;
            flip = true;
        } else {
            a = N - 1;
        }
    }
    return a < 0 ? 0 : (a >= N ? N - 1 : a);
}

__device__ __forceinline__ int clamp_int(int a, int lo, int hi) {
    return a < lo ? lo : (a > hi ? hi : a);
}

}  // namespace swe
