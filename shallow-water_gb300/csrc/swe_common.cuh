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
    float gf, half_gf, inv_dxf, inv_dyf;  // FP32 images for the FP32-mixed form
    double cfl_min_dxdy;         // cfl * min(dx, dy) (compute_stable_dt numerator)
    double dt_fixed;             // > 0: fixed dt; otherwise adaptive from speed slot
    unsigned long long *speed;   // two max-wave-speed slots (double bit patterns)
    int slot_read;               // slot holding max speed of U^n (adaptive dt)
    int slot_write;              // slot receiving max speed of U^(n+1) (stage 3)
    double *t_accum;             // simulation time, += dt once per step (stage 3)
    double *dt_log;              // optional per-step dt record
    int log_index;               // index into dt_log for this step
    int *flags;                  // FLAG_* bits
    unsigned char *mask;         // optional: 1 where positivity clamped the cell (adjoint)
    int halo_lo, halo_hi;        // x sides whose ghost rows a neighbour slab supplies
    int tile_row0;               // first tile row of a launch over a band of tile rows
};

// Ensemble of independent grids (one per instance) in shared field pools.
struct EnsInst {
    long long off;            // element offset of the instance in every field pool
    int Nx, Ny;
    long long pitch;
    int tiles_j;              // tiles along y for the launched tile shape
    int tile_base;            // first global work-list index of the instance
    double inv_dx, inv_dy;
    int kx, ky;
    float inv_dxf, inv_dyf;
    double cfl_min_dxdy;
};

struct EnsParams {
    const void *src[3];       // stage source pools (h or eta, hu, hv)
    const void *n[3];         // U^n pools
    void *out[3];             // output pools
    const void *B;            // bathymetry pool
    const EnsInst *inst;      // per instance
    const int *tile_inst;     // work item -> instance
    int total_tiles;
    int bc;
    double g, half_g;
    float gf, half_gf;
    double dt_fixed;          // > 0: all instances use it
    unsigned long long *speed;  // 2 slots per instance
    int slot_read, slot_write;
    double *t;                // per-instance time
    double *dt_last;          // per-instance dt of the last step
    int *flags;
    int elem;                 // element size (8: FP64, 4: FP32)
    // FP32 form: TMA maps of the current tile shape, per instance and stage source:
    // maps[(q * 3 + s) * 4 + f], s = 0 U^n, 1 U^(1), 2 U^(2); f = eta, hu, hv, B (null:
    // every tile uses the mirrored-index loader).  CUtensorMap is 128 bytes.
    const void *maps;
};

enum : int { SHAPE_8x32 = 0, SHAPE_8x16 = 1, SHAPE_4x64 = 2, SHAPE_16x32 = 3, SHAPE_8x64 = 4,
             SHAPE_COLS = 5, SHAPE_STRIP = 6 };
// SHAPE_COLS (FP32 form): a work item is a strip of F32_STRIP_ROWS rows by F32_COL_BLOCK
// columns, swept by column warps (swe_fp32.cu).
constexpr int F32_STRIP_ROWS = 64, F32_COL_BLOCK = 112;
// SHAPE_STRIP (FP64 form): a work item is a strip of F64_STRIP_TILES 8x32 tiles along x,
// walked by one CTA that carries each tile's last x-face row into the next (swe_fp64.cu).
constexpr int F64_STRIP_TILES = 6;

// StageParams of instance q inside an ensemble launch.
__device__ __forceinline__ StageParams ens_view(const EnsParams &e, int q) {
    const EnsInst &I = e.inst[q];
    const long long off = I.off * e.elem;
    StageParams p{};  // every field defined (halo sides, mask, log: none)
    p.hs = static_cast<const char *>(e.src[0]) + off;
    p.hus = static_cast<const char *>(e.src[1]) + off;
    p.hvs = static_cast<const char *>(e.src[2]) + off;
    p.hn = static_cast<const char *>(e.n[0]) + off;
    p.hun = static_cast<const char *>(e.n[1]) + off;
    p.hvn = static_cast<const char *>(e.n[2]) + off;
    p.B = static_cast<const char *>(e.B) + off;
    p.ho = static_cast<char *>(e.out[0]) + off;
    p.huo = static_cast<char *>(e.out[1]) + off;
    p.hvo = static_cast<char *>(e.out[2]) + off;
    p.Nx = I.Nx;
    p.Ny = I.Ny;
    p.pitch = I.pitch;
    p.bc = e.bc;
    p.inv_dx = I.inv_dx;
    p.inv_dy = I.inv_dy;
    p.kx = I.kx;
    p.ky = I.ky;
    p.g = e.g;
    p.half_g = e.half_g;
    p.gf = e.gf;
    p.half_gf = e.half_gf;
    p.inv_dxf = I.inv_dxf;
    p.inv_dyf = I.inv_dyf;
    p.cfl_min_dxdy = I.cfl_min_dxdy;
    p.dt_fixed = e.dt_fixed;
    p.speed = e.speed + 2 * q;
    p.slot_read = e.slot_read;
    p.slot_write = e.slot_write;
    p.t_accum = nullptr;
    p.dt_log = nullptr;
    p.log_index = 0;
    p.flags = e.flags;
    p.mask = nullptr;
    return p;
}

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

// Row coordinate of a stencil cell: ghost rows on a slab-interface side are read where
// they lie (they hold the neighbour's rows); other ghosts follow the wall rule.
__device__ __forceinline__ int map_row(int a, int N, int bc, bool halo_lo, bool halo_hi,
                                       bool &flip) {
    if ((a < 0 && halo_lo) || (a >= N && halo_hi)) {
        flip = false;
        return a;
    }
    return map_coord(a, N, bc, flip);
}

__device__ __forceinline__ int clamp_int(int a, int lo, int hi) {
    return a < lo ? lo : (a > hi ? hi : a);
}

}  // namespace swe
