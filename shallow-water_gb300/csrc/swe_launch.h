// Internal launchers shared between the kernel translation units and the C ABI.
#pragma once

#include <cuda_runtime.h>

#include "swe_common.cuh"
#include "swe_tma.cuh"

namespace swe {

// FP64 drop-in (swe_fp64.cu, compiled with --fmad=false).
// maps (optional): TMA maps of the stage source (h, hu, hv, B) for interior tiles.
// Tile rows [tile_row0, tile_row1) only (tile_row1 < 0: to the last).  Stage 0 stores
// L(U^n) in p.ho/huo/hvo; launch_combine1_f64 then forms U^(1) into (h, hu, hv) with the
// step's dt, bitwise as stage 1.
cudaError_t launch_stage_f64(int stage, const StageParams &p, const StageMaps *maps,
                             cudaStream_t s, int tile_row0 = 0, int tile_row1 = -1);
cudaError_t launch_combine1_f64(const StageParams &p, void *h, void *hu, void *hv, int num_sms,
                                cudaStream_t s);
// Max wave speed of interior rows [i0, i1) into slot (atomic max).
cudaError_t launch_max_speed_rows_f64(const void *h, const void *hu, const void *hv, int i0,
                                      int i1, int Ny, long long pitch, double g,
                                      unsigned long long *slot, int num_sms, cudaStream_t s);
// Ghosts of ghosted rows [r0, r1) by the wall rule (no slab sides).
cudaError_t launch_fill_ghost_band_f64(void *h, void *hu, void *hv, int Nx, int Ny,
                                       long long pitch, int bc, int r0, int r1, cudaStream_t s);
constexpr int TILE_I_F64 = 8, TILE_J_F64 = 32;
// Ensemble stage over the work list; shape is SHAPE_* (8x32, 8x16, 4x64 for FP64).
cudaError_t launch_ens_stage_f64(int shape, int stage, const EnsParams &e, int grid,
                                 cudaStream_t s);
// CTAs of each ensemble tile shape that fit on one SM at once (the minimum over the three
// stage kernels; 0 if the occupancy query fails).
int ens_resident_per_sm_f64(int shape);
int ens_resident_per_sm_f32(int shape);
cudaError_t launch_max_speed_f64(const void *h, const void *hu, const void *hv, int Nx, int Ny,
                                 long long pitch, double g, unsigned long long *slot,
                                 int num_sms, cudaStream_t s);
// Ghost refresh by the wall rule; x-ghost rows on slab-interface sides are left as stored.
cudaError_t launch_fill_ghosts_f64(void *h, void *hu, void *hv, int Nx, int Ny, long long pitch,
                                   int bc, cudaStream_t s, int halo_lo = 0, int halo_hi = 0);

// FP32-mixed form (swe_fp32.cu): state (eta = h + B, hu, hv) and B in FP32.
// Single-grid FP32 tile shape (rows x columns); the TMA box is (TI + 4) x (TJ + 4).
#ifndef SWE_TILE_I_F32
#define SWE_TILE_I_F32 8
#endif
constexpr int TILE_I_F32 = SWE_TILE_I_F32, TILE_J_F32 = 32;
// maps: TMA maps of the stage source (NULL: every tile uses the mirrored-index loader).
cudaError_t launch_stage_f32(int stage, const StageParams &p, const StageMaps *maps,
                             cudaStream_t s);
// Ensemble stage (FP32-mixed); shape is SHAPE_8x32, SHAPE_16x32 or SHAPE_8x64.
cudaError_t launch_ens_stage_f32(int shape, int stage, const EnsParams &e, int grid,
                                 cudaStream_t s);
cudaError_t launch_max_speed_f32(const void *e, const void *hu, const void *hv, const void *B,
                                 int Nx, int Ny, long long pitch, double g,
                                 unsigned long long *slot, int num_sms, cudaStream_t s);
cudaError_t launch_f64_to_f32(const void *src, const void *add, void *dst, int rows, int cols,
                              long long pitch, int num_sms, cudaStream_t s);
cudaError_t launch_f32_to_f64(const void *src, const void *sub, void *dst, int rows, int cols,
                              long long pitch, int num_sms, cudaStream_t s);
cudaError_t launch_fill_ghosts_f32(void *e, void *hu, void *hv, const void *B, int Nx, int Ny,
                                   long long pitch, int bc, cudaStream_t s);

// Compensated totals (swe_reduce.cu): out[0..2] = (sum h, sum hu, sum hv) * dxdy.
// partial needs 6 * totals_blocks(num_sms) doubles.
int totals_blocks(int num_sms);
cudaError_t launch_totals_blocks(const void *h, const void *hu, const void *hv, const void *B,
                                 bool f32, int Nx, int Ny, long long pitch, double dxdy,
                                 double *partial, double *out, int blocks, cudaStream_t s);
// The modular solver (swe_modular.cu, --fmad=false): one fused stage of
// SerialSolver<ReflectingWalls, recon, riemann, SSPRK3, bathymetry on / off>.
struct ModularStage {
    const void *hs, *hus, *hvs;  // stage source
    const void *hn, *hun, *hvn;  // U^n
    const void *B;
    void *ho, *huo, *hvo;
    int Nx, Ny;
    long long pitch;
    double g, dx, dy, dt;
    int recon, riemann, bathy;  // 0 / 1 PiecewiseConst / MUSCL; 0 / 1 / 2 HLL / Rusanov / ROE
    int kx, ky;                 // log2 of 1 / dx and 1 / dy when powers of two, else 127
    int *flags;                 // FLAG_NONFINITE, FLAG_MODULAR_HLL
};
constexpr int FLAG_MODULAR_HLL = 4;  // HLL could not provide a dissipation speed
cudaError_t launch_stage_modular(int stage, const ModularStage &m, cudaStream_t s);
// time_utils.hpp's compute_stable_dt into *out (as double bits); h < 0 sets FLAG_NONFINITE.
cudaError_t launch_modular_stable_dt(const void *h, const void *hu, const void *hv, int Nx, int Ny,
                                     long long pitch, double g, double cfl, double dx, double dy,
                                     unsigned long long *out, int *flags, int num_sms,
                                     cudaStream_t s);

// Sanity reductions (mass, energy, h_min, first negative index) into out[0..3];
// partial holds 6 doubles per block, num_sms * 4 blocks.
cudaError_t launch_sanity(const void *h, const void *hu, const void *hv, const void *B, bool f32,
                          int Nx, int Ny, long long pitch, double g, double dxdy,
                          double *partial, double *out, int num_sms, cudaStream_t s);
cudaError_t launch_totals(const void *h, const void *hu, const void *hv, const void *B, bool f32,
                          int Nx, int Ny, long long pitch, double dxdy, double *partial,
                          double *out, int num_sms, cudaStream_t s);

}  // namespace swe
