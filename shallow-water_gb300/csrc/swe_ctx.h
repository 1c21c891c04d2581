// Internal definition of the single-grid context (swe_ctx in include/swe_gb300.h),
// shared by the C ABI (swe_api.cu) and the adjoint driver (swe_adjoint.cu).
#pragma once

#include <cuda_runtime.h>

#include <string>

#include "../../include/swe_gb300.h"
#include "swe_tma.cuh"

struct swe_ctx {
    swe_params p{};
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    long long pitch = 0;       // device row pitch, elements
    size_t field_elems = 0;    // (Nx + 4) * pitch
    void *base = nullptr;      // single device allocation
    void *Un[3]{}, *U1[3]{}, *U2[3]{}, *B = nullptr;
    void *stage64[2]{};        // FP32 form: FP64 staging (B as given, scratch) in device layout
    double *partial = nullptr; // totals: per-block compensated pairs, then the 3 results
    unsigned long long *speed = nullptr;  // [2]
    double *t_accum = nullptr;
    int *flags = nullptr;
    double *dt_log = nullptr;
    int dt_log_cap = 0;
    int last_steps = 0;
    long long steps_done = 0;  // selects the speed slot parity
    bool uploaded = false;
    double dx = 0, dy = 0, inv_dx = 0, inv_dy = 0, cfl_min_dxdy = 0;
    long long launches = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // bracket the stage launches of swe_step
    // swe_step_host: a transfer stream, a second compute stream for alternate bands, and
    // one event per band of rows (uploaded / finished) plus two joins, created on first
    // use.
    cudaStream_t xfer = nullptr, aux = nullptr;
    cudaEvent_t band_ev[130]{};
    int n_band_ev = 0;
    double last_ms = 0.0;
    double modular_dt = 0.0;   // the modular scheme's fixed dt of the last swe_step
    swe::StageMaps maps[3]{};  // FP32 form: TMA maps of U^n, U^(1), U^(2) (stage sources)
    bool maps_ok = false;
    bool preset_timeout = false;  // swe_test_preset_timeout: the next stepping call's flag
    std::string err;
};

namespace swe {
// k with x == 2^k when x is a normal power of two with |k| <= 64, else 127.
int pow2_exponent(double x);
// Launch parameters shared by every stage of a context (buffers, slots and log index are
// set per stage by the caller); dt > 0 fixes the step, otherwise it is adaptive.
StageParams ctx_stage_params(swe_ctx *c, double dt);
}  // namespace swe
