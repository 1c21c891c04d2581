// Internal launchers shared between the kernel translation units and the C ABI.
#pragma once

#include <cuda_runtime.h>

#include "swe_common.cuh"

namespace swe {

// FP64 drop-in (swe_fp64.cu, compiled with --fmad=false).
cudaError_t launch_stage_f64(int stage, const StageParams &p, cudaStream_t s);
cudaError_t launch_max_speed_f64(const void *h, const void *hu, const void *hv, int Nx, int Ny,
                                 long long pitch, double g, unsigned long long *slot,
                                 int num_sms, cudaStream_t s);
cudaError_t launch_fill_ghosts_f64(void *h, void *hu, void *hv, int Nx, int Ny, long long pitch,
                                   int bc, cudaStream_t s);

}  // namespace swe
