// C ABI of the GB300 shallow-water backend (declared in include/swe_gb300.h).
//
// Owns the device state of one grid: U^n, U^(1), U^(2) (h, hu, hv each), the
// bathymetry, two max-wave-speed slots, the time accumulator, a per-step dt record
// and an error-flag word, all in one allocation.  Every call runs on the context's
// own stream and synchronises before returning; no exception crosses the boundary.
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "../../include/swe_gb300.h"
#include "swe_launch.h"

using namespace swe;

#include "swe_ctx.h"

namespace {

int fail(swe_ctx *c, int status, const char *fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return status;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return fail(c, SWE_ERR_CUDA, "%s failed: %s (%s:%d)", #call,                      \
                        cudaGetErrorString(e_), __FILE__, __LINE__);                          \
    } while (0)

size_t elem_size(const swe_ctx *c) {
    return c->p.precision == SWE_PRECISION_FP64 ? sizeof(double) : sizeof(float);
}

int set_device(swe_ctx *c) {
    CK(cudaSetDevice(c->p.device));
    return SWE_OK;
}

// Clears the error-flag word at the start of a stepping call.  After
// swe_test_preset_timeout, the call's flag word starts with FLAG_TIMEOUT set instead (its
// low byte; the word is little-endian), as if a wait of an earlier launch had given up.
int clear_flags(swe_ctx *c) {
    CK(cudaMemsetAsync(c->flags, 0, sizeof(int), c->stream));
    if (c->preset_timeout) {
        c->preset_timeout = false;
        CK(cudaMemsetAsync(c->flags, FLAG_TIMEOUT, 1, c->stream));
    }
    return SWE_OK;
}

}  // namespace

bool swe::encode_tile_map(CUtensorMap *m, const void *base, int rows, int cols,
                          long long pitch, int box_rows, int box_cols, int elem) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                             cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            cudaGetLastError();
            return false;
        }
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch * (cuuint64_t)elem};
    const cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUtensorMapDataType type =
        elem == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    return encode(m, type, 2, const_cast<void *>(base), dims, strides,
                  box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// k with x == 2^k when x is a normal power of two with |k| <= 64, else 127.
int swe::pow2_exponent(double x) {
    int k = 0;
    const double m = std::frexp(x, &k);  // x = m * 2^k, m in [0.5, 1)
    if (m != 0.5 || !(x > 0.0) || k - 1 < -64 || k - 1 > 64) return 127;
    return k - 1;
}

namespace {

bool fp32(const swe_ctx *c) { return c->p.precision == SWE_PRECISION_FP32_MIXED; }
bool modular(const swe_ctx *c) { return c->p.scheme == SWE_SCHEME_MODULAR; }
int refresh_speed(swe_ctx *c);

// One stage of the modular solver from buffer set src into dst (stage 1: U^n -> U^(1),
// 2: U^(1) -> U^(2), 3: U^(2) -> U^n).
cudaError_t launch_modular(swe_ctx *c, int stage, double dt, void *const *src, void *const *dst) {
    ModularStage m{};
    m.hs = src[0]; m.hus = src[1]; m.hvs = src[2];
    m.hn = c->Un[0]; m.hun = c->Un[1]; m.hvn = c->Un[2];
    m.B = c->B;
    m.ho = dst[0]; m.huo = dst[1]; m.hvo = dst[2];
    m.Nx = c->p.Nx;
    m.Ny = c->p.Ny;
    m.pitch = c->pitch;
    m.g = c->p.g;
    m.dx = c->dx;
    m.dy = c->dy;
    m.dt = dt;
    m.recon = c->p.reconstruction;
    m.riemann = c->p.riemann;
    m.bathy = c->p.bathymetry;
    m.kx = pow2_exponent(1.0 / c->dx);
    m.ky = pow2_exponent(1.0 / c->dy);
    m.flags = c->flags;
    return launch_stage_modular(stage, m, c->stream);
}

// swe_step of the modular scheme: SerialSolver::run's step loop with fixed dt; the time
// accumulates on the host in step order (serial_solver.hpp:220).
int step_modular(swe_ctx *c, int n_steps, double dt, double *t_inout) {
    if (!(dt > 0.0))
        return fail(c, SWE_ERR_UNSUPPORTED, "swe_step: the modular scheme takes a fixed dt > 0");
    CK(cudaMemsetAsync(c->flags, 0, sizeof(int), c->stream));
    CK(cudaEventRecord(c->ev0, c->stream));
    for (int s = 0; s < n_steps; ++s) {
        CK(launch_modular(c, 1, dt, c->Un, c->U1));
        CK(launch_modular(c, 2, dt, c->U1, c->U2));
        CK(launch_modular(c, 3, dt, c->U2, c->Un));
        c->launches += 3;
        ++c->steps_done;
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    const int st = refresh_speed(c);  // keeps swe_max_wave_speed current
    if (st) return st;
    int flags = 0;
    CK(cudaMemcpyAsync(&flags, c->flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_ms = ms;
    c->last_steps = n_steps;
    c->modular_dt = dt;
    if (t_inout)
        for (int s = 0; s < n_steps; ++s) *t_inout += dt;
    if (flags & FLAG_MODULAR_HLL)
        return fail(c, SWE_ERR_NONFINITE, "HLL could not provide dissipation speed.");
    if (flags & FLAG_NONFINITE)
        return fail(c, SWE_ERR_NONFINITE, "non-finite state detected in positivity correction");
    return SWE_OK;
}

}  // namespace

// Launch parameters shared by every stage of a context (buffers set per stage).
StageParams swe::ctx_stage_params(swe_ctx *c, double dt) {
    StageParams sp{};
    sp.B = c->B;
    sp.Nx = c->p.Nx;
    sp.Ny = c->p.Ny;
    sp.pitch = c->pitch;
    sp.bc = c->p.bc;
    sp.inv_dx = c->inv_dx;
    sp.inv_dy = c->inv_dy;
    sp.kx = pow2_exponent(c->inv_dx);
    sp.ky = pow2_exponent(c->inv_dy);
    sp.g = c->p.g;
    sp.half_g = 0.5 * c->p.g;
    sp.gf = (float)sp.g;
    sp.half_gf = (float)sp.half_g;
    sp.inv_dxf = (float)sp.inv_dx;
    sp.inv_dyf = (float)sp.inv_dy;
    sp.cfl_min_dxdy = c->cfl_min_dxdy;
    sp.dt_fixed = dt > 0.0 ? dt : 0.0;
    sp.speed = c->speed;
    sp.t_accum = c->t_accum;
    sp.dt_log = c->dt_log;
    sp.flags = c->flags;
    sp.halo_lo = c->p.x_halo_lo;
    sp.halo_hi = c->p.x_halo_hi;
    return sp;
}

namespace {

// Max wave speed of U^n into the slot the next step reads.
int refresh_speed(swe_ctx *c) {
    unsigned long long *slot = c->speed + (c->steps_done & 1);
    CK(cudaMemsetAsync(slot, 0, sizeof(unsigned long long), c->stream));
    if (fp32(c)) {
        CK(launch_max_speed_f32(c->Un[0], c->Un[1], c->Un[2], c->B, c->p.Nx, c->p.Ny, c->pitch,
                                c->p.g, slot, c->num_sms, c->stream));
    } else {
        CK(launch_max_speed_f64(c->Un[0], c->Un[1], c->Un[2], c->p.Nx, c->p.Ny, c->pitch,
                                c->p.g, slot, c->num_sms, c->stream));
    }
    ++c->launches;
    return SWE_OK;
}

// Room for one dt per step of a call in the device dt record.
int ensure_dt_log(swe_ctx *c, int n_steps) {
    if (c->dt_log_cap >= n_steps) return SWE_OK;
    if (c->dt_log) CK(cudaFree(c->dt_log));
    c->dt_log = nullptr;
    c->dt_log_cap = 0;
    const int cap = std::max(n_steps, 1024);
    CK(cudaMalloc(&c->dt_log, (size_t)cap * sizeof(double)));
    c->dt_log_cap = cap;
    return SWE_OK;
}

cudaError_t launch_stage(swe_ctx *c, int stage, const StageParams &sp) {
    if (fp32(c))
        return launch_stage_f32(stage, sp, c->maps_ok ? &c->maps[stage - 1] : nullptr, c->stream);
    return launch_stage_f64(stage, sp, c->maps_ok ? &c->maps[stage - 1] : nullptr, c->stream);
}

// TMA maps of the three stage sources of a context (box = tile + 2-cell halo): the FP32
// form's (eta, hu, hv, B) or the FP64 form's (h, hu, hv, B).  Any failure leaves maps_ok
// false and every tile on the mirrored-index loader.
void build_maps(swe_ctx *c) {
    c->maps_ok = false;
    const char *off = std::getenv("SWE_GB300_NO_TMA");
    if (off && off[0] == '1') return;
    const int rows = c->p.Nx + 4, cols = c->p.Ny + 4;
    const bool f32 = fp32(c);
    const int bi = (f32 ? TILE_I_F32 : TILE_I_F64) + 4, bj = (f32 ? TILE_J_F32 : TILE_J_F64) + 4;
    const int el = f32 ? 4 : 8;
    void *const *src[3] = {c->Un, c->U1, c->U2};
    for (int s = 0; s < 3; ++s) {
        StageMaps &m = c->maps[s];
        if (!encode_tile_map(&m.e, src[s][0], rows, cols, c->pitch, bi, bj, el) ||
            !encode_tile_map(&m.u, src[s][1], rows, cols, c->pitch, bi, bj, el) ||
            !encode_tile_map(&m.v, src[s][2], rows, cols, c->pitch, bi, bj, el) ||
            !encode_tile_map(&m.b, c->B, rows, cols, c->pitch, bi, bj, el))
            return;
    }
    c->maps_ok = true;
}

}  // namespace

extern "C" {

size_t swe_params_size(void) { return sizeof(swe_params); }
size_t swe_snapshot_params_size(void) { return sizeof(swe_snapshot_params); }

void swe_params_default(swe_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->nG = 2;
    p->Lx = p->Ly = 1.0;
    p->g = 9.80665;
    p->cfl = 0.45;
    p->bc = SWE_BC_REFLECTING;
    p->precision = SWE_PRECISION_FP64;
    p->device = 0;
    p->scheme = SWE_SCHEME_FUSED;
    p->reconstruction = SWE_RECON_MUSCL;
    p->riemann = SWE_RIEMANN_HLL;
    p->bathymetry = 1;
}

const char *swe_status_string(int s) {
    switch (s) {
        case SWE_OK: return "ok";
        case SWE_ERR_BAD_ARG: return "bad argument";
        case SWE_ERR_CUDA: return "CUDA error";
        case SWE_ERR_NONFINITE: return "non-finite state detected";
        case SWE_ERR_CFL: return "time step above the CFL limit";
        case SWE_ERR_TIMEOUT: return "device wait timed out";
        case SWE_ERR_NO_DEVICE: return "no CUDA device";
        case SWE_ERR_UNSUPPORTED: return "unsupported option";
        case SWE_ERR_IO: return "output file error";
        default: return "unknown status";
    }
}

const char *swe_last_error(const swe_ctx *c) { return c ? c->err.c_str() : "null context"; }

long long swe_kernel_launches(const swe_ctx *c) { return c ? c->launches : 0; }

int swe_create(const swe_params *pin, swe_ctx **out) {
    if (!pin || !out) return SWE_ERR_BAD_ARG;
    *out = nullptr;
    swe_params p = *pin;
    if (p.g <= 0.0) p.g = 9.80665;
    if (p.nG != 2 || p.Nx < 2 || p.Ny < 2 || !(p.Lx > 0.0) || !(p.Ly > 0.0) ||
        !(p.cfl > 0.0) || (p.bc != SWE_BC_REFLECTING && p.bc != SWE_BC_TRANSMISSIVE))
        return SWE_ERR_BAD_ARG;
    if (p.reserved != 0 || !(p.dx >= 0.0) || !(p.dy >= 0.0)) return SWE_ERR_BAD_ARG;
    p.x_halo_lo = p.x_halo_lo != 0;
    p.x_halo_hi = p.x_halo_hi != 0;
    // Device indices are int: keep (Nx + 4) * pitch below 2^31 per field.
    if ((long long)(p.Nx + 4) * (long long)(p.Ny + 36) >= (1ll << 31)) return SWE_ERR_BAD_ARG;
    if (p.precision != SWE_PRECISION_FP64 && p.precision != SWE_PRECISION_FP32_MIXED)
        return SWE_ERR_UNSUPPORTED;
    if ((p.x_halo_lo || p.x_halo_hi) && p.precision != SWE_PRECISION_FP64)
        return SWE_ERR_UNSUPPORTED;  // slabs are an FP64 drop-in feature
    if (p.scheme != SWE_SCHEME_FUSED && p.scheme != SWE_SCHEME_MODULAR) return SWE_ERR_BAD_ARG;
    if (p.scheme == SWE_SCHEME_MODULAR) {
        if (p.reconstruction < 0 || p.reconstruction > 1 || p.riemann < 0 || p.riemann > 2)
            return SWE_ERR_BAD_ARG;
        p.bathymetry = p.bathymetry != 0;
        // SerialSolver: FP64, ReflectingWalls only (the reference has no other boundary)
        if (p.precision != SWE_PRECISION_FP64 || p.bc != SWE_BC_REFLECTING || p.x_halo_lo ||
            p.x_halo_hi)
            return SWE_ERR_UNSUPPORTED;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= p.device || p.device < 0) {
        cudaGetLastError();
        return SWE_ERR_NO_DEVICE;
    }
    swe_ctx *c = new (std::nothrow) swe_ctx();
    if (!c) return SWE_ERR_BAD_ARG;
    c->p = p;
    int st = set_device(c);
    if (st != SWE_OK) {
        delete c;
        return st;
    }
    // HPC_solver.hpp:91-93 and include/core/grid.hpp:19-20; 1.0 / dx as apply_divergence.
    c->dx = p.dx > 0.0 ? p.dx : p.Lx / p.Nx;
    c->dy = p.dy > 0.0 ? p.dy : p.Ly / p.Ny;
    c->inv_dx = 1.0 / c->dx;
    c->inv_dy = 1.0 / c->dy;
    c->cfl_min_dxdy = p.cfl * std::min(c->dx, c->dy);
    c->pitch = ((long long)(p.Ny + 4) + 31) / 32 * 32;
    c->field_elems = (size_t)(p.Nx + 4) * (size_t)c->pitch;
    const size_t fb = c->field_elems * elem_size(c);
    const size_t aux = 256;  // speed slots, time, flags
    const size_t staging = (p.precision == SWE_PRECISION_FP32_MIXED)
                               ? 2 * c->field_elems * sizeof(double) : 0;
    auto cleanup = [&](int s) {
        if (c->base) cudaFree(c->base);
        if (c->ev0) cudaEventDestroy(c->ev0);
        if (c->ev1) cudaEventDestroy(c->ev1);
        if (c->stream) cudaStreamDestroy(c->stream);
        cudaGetLastError();
        delete c;
        return s;
    };
    cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, p.device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&c->base, 10 * fb + aux + staging);
    if (e != cudaSuccess) {
        const int s = (e == cudaErrorMemoryAllocation) ? SWE_ERR_BAD_ARG : SWE_ERR_CUDA;
        return cleanup(s);
    }
    char *b = static_cast<char *>(c->base);
    for (int f = 0; f < 3; ++f) {
        c->Un[f] = b + (0 + f) * fb;
        c->U1[f] = b + (3 + f) * fb;
        c->U2[f] = b + (6 + f) * fb;
    }
    c->B = b + 9 * fb;
    char *a = b + 10 * fb;
    c->speed = reinterpret_cast<unsigned long long *>(a);
    c->t_accum = reinterpret_cast<double *>(a + 16);
    c->flags = reinterpret_cast<int *>(a + 24);
    if (staging) {
        c->stage64[0] = a + aux;
        c->stage64[1] = a + aux + c->field_elems * sizeof(double);
    }
    // Zero everything once so untouched ghosts and padding are defined.
    e = cudaMemsetAsync(c->base, 0, 10 * fb + aux + staging, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cleanup(SWE_ERR_CUDA);
    build_maps(c);
    *out = c;
    return SWE_OK;
}

void swe_destroy(swe_ctx *c) {
    if (!c) return;
    cudaSetDevice(c->p.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->dt_log) cudaFree(c->dt_log);
    if (c->partial) cudaFree(c->partial);
    if (c->base) cudaFree(c->base);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (int i = 0; i < c->n_band_ev; ++i) cudaEventDestroy(c->band_ev[i]);
    if (c->xfer) cudaStreamDestroy(c->xfer);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->stream) cudaStreamDestroy(c->stream);
    cudaGetLastError();
    delete c;
}

int swe_upload(swe_ctx *c, const double *h, const double *hu, const double *hv, const double *B) {
    if (!c || !h || !hu || !hv) return fail(c, SWE_ERR_BAD_ARG, "swe_upload: null argument");
    if (!c->uploaded && !B) return fail(c, SWE_ERR_BAD_ARG, "swe_upload: first upload needs B");
    int st = set_device(c);
    if (st) return st;
    const size_t row = (size_t)(c->p.Ny + 4) * sizeof(double);
    const size_t dpitch = (size_t)c->pitch * sizeof(double);
    const size_t rows = (size_t)(c->p.Nx + 4);
    if (fp32(c)) {
        // B as given stays in stage64[0]; eta = RN32(h + B), the rest rounded to FP32.
        const int R = c->p.Nx + 4, C = c->p.Ny + 4;
        if (B) {
            CK(cudaMemcpy2DAsync(c->stage64[0], dpitch, B, row, row, rows,
                                 cudaMemcpyHostToDevice, c->stream));
            CK(launch_f64_to_f32(c->stage64[0], nullptr, c->B, R, C, c->pitch, c->num_sms,
                                 c->stream));
            ++c->launches;
        }
        const double *src[3] = {h, hu, hv};
        for (int f = 0; f < 3; ++f) {
            CK(cudaMemcpy2DAsync(c->stage64[1], dpitch, src[f], row, row, rows,
                                 cudaMemcpyHostToDevice, c->stream));
            CK(launch_f64_to_f32(c->stage64[1], f == 0 ? c->stage64[0] : nullptr, c->Un[f], R,
                                 C, c->pitch, c->num_sms, c->stream));
            ++c->launches;
        }
    } else {
        const double *src[4] = {h, hu, hv, B};
        void *dst[4] = {c->Un[0], c->Un[1], c->Un[2], c->B};
        for (int f = 0; f < 4; ++f) {
            if (!src[f]) continue;
            CK(cudaMemcpy2DAsync(dst[f], dpitch, src[f], row, row, rows,
                                 cudaMemcpyHostToDevice, c->stream));
        }
    }
    c->steps_done = 0;
    st = refresh_speed(c);
    if (st) return st;
    CK(cudaStreamSynchronize(c->stream));
    c->uploaded = true;
    return SWE_OK;
}

int swe_download(swe_ctx *c, double *h, double *hu, double *hv) {
    if (!c || !h || !hu || !hv) return fail(c, SWE_ERR_BAD_ARG, "swe_download: null argument");
    if (!c->uploaded) return fail(c, SWE_ERR_BAD_ARG, "swe_download: no state uploaded");
    int st = set_device(c);
    if (st) return st;
    const size_t row = (size_t)(c->p.Ny + 4) * sizeof(double);
    const size_t spitch = (size_t)c->pitch * sizeof(double);
    double *dst[3] = {h, hu, hv};
    if (fp32(c)) {
        CK(launch_fill_ghosts_f32(c->Un[0], c->Un[1], c->Un[2], c->B, c->p.Nx, c->p.Ny,
                                  c->pitch, c->p.bc, c->stream));
        ++c->launches;
        for (int f = 0; f < 3; ++f) {
            // h = eta - B (exact in FP64); hu, hv widened.  The scratch staging buffer is
            // reused, so each field's copy completes before the next conversion.
            CK(launch_f32_to_f64(c->Un[f], f == 0 ? c->B : nullptr, c->stage64[1],
                                 c->p.Nx + 4, c->p.Ny + 4, c->pitch, c->num_sms, c->stream));
            ++c->launches;
            CK(cudaMemcpy2DAsync(dst[f], row, c->stage64[1], spitch, row,
                                 (size_t)(c->p.Nx + 4), cudaMemcpyDeviceToHost, c->stream));
        }
    } else {
        CK(launch_fill_ghosts_f64(c->Un[0], c->Un[1], c->Un[2], c->p.Nx, c->p.Ny, c->pitch,
                                  c->p.bc, c->stream, c->p.x_halo_lo, c->p.x_halo_hi));
        ++c->launches;
        for (int f = 0; f < 3; ++f)
            CK(cudaMemcpy2DAsync(dst[f], row, c->Un[f], spitch, row, (size_t)(c->p.Nx + 4),
                                 cudaMemcpyDeviceToHost, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return SWE_OK;
}

int swe_step(swe_ctx *c, int n_steps, double dt, double *t_inout) {
    if (!c || n_steps < 0) return fail(c, SWE_ERR_BAD_ARG, "swe_step: bad argument");
    if (!c->uploaded) return fail(c, SWE_ERR_BAD_ARG, "swe_step: no state uploaded");
    if (!(dt == dt)) return fail(c, SWE_ERR_BAD_ARG, "swe_step: dt is NaN");
    c->last_steps = 0;
    if (n_steps == 0) return SWE_OK;
    int st = set_device(c);
    if (st) return st;
    if (modular(c)) return step_modular(c, n_steps, dt, t_inout);
    st = ensure_dt_log(c, n_steps);
    if (st) return st;
    const double t0 = t_inout ? *t_inout : 0.0;
    CK(cudaMemcpyAsync(c->t_accum, &t0, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    st = clear_flags(c);
    if (st) return st;

    StageParams sp = ctx_stage_params(c, dt);
    CK(cudaEventRecord(c->ev0, c->stream));
    for (int s = 0; s < n_steps; ++s) {
        sp.slot_read = (int)(c->steps_done & 1);
        sp.slot_write = sp.slot_read ^ 1;
        sp.log_index = s;
        // Stage 1: U1 = Un + dt L(Un)
        sp.hs = c->Un[0]; sp.hus = c->Un[1]; sp.hvs = c->Un[2];
        sp.hn = c->Un[0]; sp.hun = c->Un[1]; sp.hvn = c->Un[2];
        sp.ho = c->U1[0]; sp.huo = c->U1[1]; sp.hvo = c->U1[2];
        CK(launch_stage(c, 1, sp));
        // Stage 2: U2 = 3/4 Un + 1/4 (U1 + dt L(U1))
        sp.hs = c->U1[0]; sp.hus = c->U1[1]; sp.hvs = c->U1[2];
        sp.ho = c->U2[0]; sp.huo = c->U2[1]; sp.hvo = c->U2[2];
        CK(launch_stage(c, 2, sp));
        // Stage 3: Un = 1/3 Un + 2/3 (U2 + dt L(U2)), in place; max speed -> next slot
        sp.hs = c->U2[0]; sp.hus = c->U2[1]; sp.hvs = c->U2[2];
        sp.ho = c->Un[0]; sp.huo = c->Un[1]; sp.hvo = c->Un[2];
        CK(launch_stage(c, 3, sp));
        c->launches += 3;
        ++c->steps_done;
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    int flags = 0;
    double t1 = 0.0;
    CK(cudaMemcpyAsync(&flags, c->flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&t1, c->t_accum, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_ms = ms;
    c->last_steps = n_steps;
    if (t_inout) *t_inout = t1;
    if (flags & FLAG_TIMEOUT)
        return fail(c, SWE_ERR_TIMEOUT, "a tile's TMA copy did not complete (state undefined)");
    if (flags & FLAG_NONFINITE)
        return fail(c, SWE_ERR_NONFINITE, "non-finite state detected in GB300 solver");
    return SWE_OK;
}

// swe_step_host: bands of about SWE_HOST_BAND_TILE_ROWS tile rows, at most kMaxBands.
#ifndef SWE_HOST_BAND_TILE_ROWS
#define SWE_HOST_BAND_TILE_ROWS 64
#endif
constexpr int kBandTileRows = SWE_HOST_BAND_TILE_ROWS, kMaxBands = 64;

int swe_step_host(swe_ctx *c, const double *h, const double *hu, const double *hv,
                  const double *B, double *h_out, double *hu_out, double *hv_out, int n_steps,
                  double dt, double *t_inout) {
    if (!c || !h || !hu || !hv || !h_out || !hu_out || !hv_out || n_steps < 0)
        return fail(c, SWE_ERR_BAD_ARG, "swe_step_host: bad argument");
    if (!(dt == dt)) return fail(c, SWE_ERR_BAD_ARG, "swe_step_host: dt is NaN");
    if (!c->uploaded && !B) return fail(c, SWE_ERR_BAD_ARG, "swe_step_host: first upload needs B");
    int st = set_device(c);
    if (st) return st;
    // The overlapped schedule is the FP64 fused drop-in's on one grid; the other forms run
    // the same three calls back to back.
    // The band schedule fills and copies out a band's ghost rows while other bands
    // still compute; that holds only for wall rules whose x-ghost rows mirror or copy
    // rows of the first or last band (swe_bc).
    const bool band_safe_bc = c->p.bc == SWE_BC_REFLECTING || c->p.bc == SWE_BC_TRANSMISSIVE;
    if (fp32(c) || modular(c) || c->p.x_halo_lo || c->p.x_halo_hi || n_steps == 0 ||
        !band_safe_bc) {
        st = swe_upload(c, h, hu, hv, B);
        if (st) return st;
        st = swe_step(c, n_steps, dt, t_inout);
        if (st) return st;
        return swe_download(c, h_out, hu_out, hv_out);
    }
    st = ensure_dt_log(c, n_steps);
    if (st) return st;
    constexpr int kEvents = 2 * kMaxBands + 2;
    static_assert(kEvents <= (int)(sizeof(c->band_ev) / sizeof(c->band_ev[0])), "events");
    if (!c->xfer) CK(cudaStreamCreateWithFlags(&c->xfer, cudaStreamNonBlocking));
    if (!c->aux) CK(cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking));
    while (c->n_band_ev < kEvents) {
        CK(cudaEventCreateWithFlags(&c->band_ev[c->n_band_ev], cudaEventDisableTiming));
        ++c->n_band_ev;
    }
    // On an early error return, no copy or kernel of this call stays in flight.
    struct Drain {
        cudaStream_t a, b;
        ~Drain() {
            cudaStreamSynchronize(a);
            cudaStreamSynchronize(b);
        }
    } drain{c->xfer, c->aux};
    const int Nx = c->p.Nx, Ny = c->p.Ny, R = Nx + 2 * NG;
    const int tile_rows = (Nx + TILE_I_F64 - 1) / TILE_I_F64;
    // Band b: tile rows [T(b), T(b + 1)).  Its stage needs ghosted rows below
    // T(b + 1) * TI + 4 (the tile, its 2-row halo and the wall ghosts); its interior rows
    // end at ghosted row T(b + 1) * TI + 2.  On large grids the first and the last band
    // are a quarter of the others: nothing overlaps the first band's upload or the last
    // band's download.
    const int edge = tile_rows >= 4 * kBandTileRows ? kBandTileRows / 4 : 0;
    const int mid_rows = tile_rows - 2 * edge;
    const int nmid = std::min(kMaxBands - 2, std::max(1, (mid_rows + kBandTileRows - 1) / kBandTileRows));
    const int nb = nmid + (edge ? 2 : 0);
    auto T = [&](int b) {
        if (!edge) return (int)((long long)tile_rows * b / nb);
        if (b == 0) return 0;
        if (b == nb) return tile_rows;
        return edge + (int)((long long)mid_rows * (b - 1) / nmid);
    };
    auto upto = [&](int b) { return b == nb ? R : std::min(R, T(b) * TILE_I_F64 + 4); };
    auto done_to = [&](int b) { return b == nb ? R : std::min(R, T(b) * TILE_I_F64 + NG); };
    const size_t row = (size_t)(Ny + 4) * sizeof(double);
    const size_t dpitch = (size_t)c->pitch * sizeof(double);
    cudaEvent_t *up = c->band_ev, *fin = c->band_ev + kMaxBands;
    cudaEvent_t join = c->band_ev[2 * kMaxBands], fork = c->band_ev[2 * kMaxBands + 1];
    // Consecutive bands alternate between the two compute streams: bands are
    // independent of each other, and one band's last wave of CTAs then overlaps the next
    // band's first instead of leaving SMs idle.
    auto band_stream = [&](int b) { return (b & 1) ? c->aux : c->stream; };

    const double t0 = t_inout ? *t_inout : 0.0;
    CK(cudaMemcpyAsync(c->t_accum, &t0, sizeof(double), cudaMemcpyHostToDevice, c->stream));
    st = clear_flags(c);
    if (st) return st;
    c->steps_done = 0;
    CK(cudaMemsetAsync(c->speed, 0, sizeof(unsigned long long), c->stream));  // slot 0
    CK(cudaEventRecord(c->ev0, c->stream));
    CK(cudaStreamWaitEvent(c->xfer, c->ev0, 0));  // nothing in flight reads U^n any more
    CK(cudaStreamWaitEvent(c->aux, c->ev0, 0));   // the speed slot is reset

    // Upload by bands on the transfer stream; as each band lands, the compute stream
    // reduces its max wave speed and computes L(U^n) on the tile rows it completes.
    const double *src[4] = {h, hu, hv, B};
    void *dst[4] = {c->Un[0], c->Un[1], c->Un[2], c->B};
    StageParams sp = ctx_stage_params(c, dt);
    sp.slot_read = 0;
    sp.slot_write = 1;
    sp.log_index = 0;
    sp.hs = c->Un[0]; sp.hus = c->Un[1]; sp.hvs = c->Un[2];
    sp.hn = c->Un[0]; sp.hun = c->Un[1]; sp.hvn = c->Un[2];
    sp.ho = c->U2[0]; sp.huo = c->U2[1]; sp.hvo = c->U2[2];  // L(U^n), free until stage 2
    for (int b = 0; b < nb; ++b) {
        const int r0 = b == 0 ? 0 : upto(b), r1 = upto(b + 1);
        for (int f = 0; f < 4; ++f) {
            if (!src[f] || r1 <= r0) continue;
            CK(cudaMemcpy2DAsync(static_cast<char *>(dst[f]) + (size_t)r0 * dpitch, dpitch,
                                 src[f] + (size_t)r0 * (Ny + 4), row, row, (size_t)(r1 - r0),
                                 cudaMemcpyHostToDevice, c->xfer));
        }
        CK(cudaEventRecord(up[b], c->xfer));
        cudaStream_t S = band_stream(b);
        CK(cudaStreamWaitEvent(S, up[b], 0));
        const int i0 = std::max(r0, NG) - NG, i1 = std::min(r1, Nx + NG) - NG;
        CK(launch_max_speed_rows_f64(c->Un[0], c->Un[1], c->Un[2], i0, i1, Ny, c->pitch,
                                     c->p.g, c->speed, c->num_sms, S));
        CK(launch_stage_f64(0, sp, c->maps_ok ? &c->maps[0] : nullptr, S, T(b), T(b + 1)));
        c->launches += 2;
    }
    CK(cudaEventRecord(join, c->aux));
    CK(cudaStreamWaitEvent(c->stream, join, 0));  // every band's speed and L
    c->uploaded = true;
    CK(launch_combine1_f64(sp, c->U1[0], c->U1[1], c->U1[2], c->num_sms, c->stream));
    ++c->launches;

    for (int s = 0; s < n_steps; ++s) {
        sp.slot_read = (int)(c->steps_done & 1);
        sp.slot_write = sp.slot_read ^ 1;
        sp.log_index = s;
        if (s > 0) {
            sp.hs = c->Un[0]; sp.hus = c->Un[1]; sp.hvs = c->Un[2];
            sp.ho = c->U1[0]; sp.huo = c->U1[1]; sp.hvo = c->U1[2];
            CK(launch_stage(c, 1, sp));
            ++c->launches;
        }
        sp.hs = c->U1[0]; sp.hus = c->U1[1]; sp.hvs = c->U1[2];
        sp.ho = c->U2[0]; sp.huo = c->U2[1]; sp.hvo = c->U2[2];
        CK(launch_stage(c, 2, sp));
        sp.hs = c->U2[0]; sp.hus = c->U2[1]; sp.hvs = c->U2[2];
        sp.ho = c->Un[0]; sp.huo = c->Un[1]; sp.hvo = c->Un[2];
        c->launches += 1;
        if (s + 1 < n_steps) {
            CK(launch_stage(c, 3, sp));
            ++c->launches;
        } else {
            // Last stage by bands; each finished band's ghosts are filled and the band
            // copied out while the next band computes.  A band's ghosts come from its own
            // rows (band 0 and the last band hold the rows the x-ghosts mirror).
            CK(cudaEventRecord(fork, c->stream));
            CK(cudaStreamWaitEvent(c->aux, fork, 0));  // stage 2 is complete
            for (int b = 0; b < nb; ++b) {
                cudaStream_t S = band_stream(b);
                CK(launch_stage_f64(3, sp, c->maps_ok ? &c->maps[2] : nullptr, S, T(b),
                                    T(b + 1)));
                const int r0 = b == 0 ? 0 : done_to(b), r1 = done_to(b + 1);
                CK(launch_fill_ghost_band_f64(c->Un[0], c->Un[1], c->Un[2], Nx, Ny, c->pitch,
                                              c->p.bc, r0, r1, S));
                c->launches += 2;
                CK(cudaEventRecord(fin[b], S));
                CK(cudaStreamWaitEvent(c->xfer, fin[b], 0));
                double *out[3] = {h_out, hu_out, hv_out};
                for (int f = 0; f < 3; ++f) {
                    if (r1 <= r0) continue;
                    CK(cudaMemcpy2DAsync(out[f] + (size_t)r0 * (Ny + 4), row,
                                         static_cast<const char *>(c->Un[f]) + (size_t)r0 * dpitch,
                                         dpitch, row, (size_t)(r1 - r0), cudaMemcpyDeviceToHost,
                                         c->xfer));
                }
            }
        }
        ++c->steps_done;
    }
    CK(cudaEventRecord(join, c->aux));
    CK(cudaStreamWaitEvent(c->stream, join, 0));
    CK(cudaEventRecord(c->ev1, c->stream));
    int flags = 0;
    double t1 = 0.0;
    CK(cudaMemcpyAsync(&flags, c->flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&t1, c->t_accum, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->xfer));
    CK(cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_ms = ms;
    c->last_steps = n_steps;
    if (t_inout) *t_inout = t1;
    if (flags & FLAG_TIMEOUT)
        return fail(c, SWE_ERR_TIMEOUT, "a tile's TMA copy did not complete (state undefined)");
    if (flags & FLAG_NONFINITE)
        return fail(c, SWE_ERR_NONFINITE, "non-finite state detected in GB300 solver");
    return SWE_OK;
}

int swe_stage(swe_ctx *c, int stage, double dt) {
    if (!c || stage < 1 || stage > 3 || !(dt > 0.0))
        return fail(c, SWE_ERR_BAD_ARG, "swe_stage: stage must be 1..3 and dt > 0");
    if (!c->uploaded) return fail(c, SWE_ERR_BAD_ARG, "swe_stage: no state uploaded");
    if (modular(c)) return fail(c, SWE_ERR_UNSUPPORTED, "swe_stage: fused scheme only");
    int st = set_device(c);
    if (st) return st;
    StageParams sp = ctx_stage_params(c, dt);
    sp.slot_read = (int)(c->steps_done & 1);
    sp.slot_write = sp.slot_read ^ 1;
    sp.t_accum = nullptr;
    sp.dt_log = nullptr;
    sp.hn = c->Un[0]; sp.hun = c->Un[1]; sp.hvn = c->Un[2];
    void *const *src = stage == 1 ? c->Un : (stage == 2 ? c->U1 : c->U2);
    void *const *dst = stage == 1 ? c->U1 : (stage == 2 ? c->U2 : c->Un);
    sp.hs = src[0]; sp.hus = src[1]; sp.hvs = src[2];
    sp.ho = dst[0]; sp.huo = dst[1]; sp.hvo = dst[2];
    st = clear_flags(c);
    if (st) return st;
    CK(launch_stage(c, stage, sp));
    ++c->launches;
    if (stage == 3) ++c->steps_done;  // the stage wrote the new state's max speed
    int flags = 0;
    CK(cudaMemcpyAsync(&flags, c->flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (flags & FLAG_TIMEOUT)
        return fail(c, SWE_ERR_TIMEOUT, "a tile's TMA copy did not complete (state undefined)");
    if (flags & FLAG_NONFINITE)
        return fail(c, SWE_ERR_NONFINITE, "non-finite state detected in GB300 solver");
    return SWE_OK;
}

int swe_halo(swe_ctx *c, int buffer, int side, int op, double *rows) {
    if (!c || !rows || buffer < 0 || buffer > 2 || side < 0 || side > 1 || op < 0 || op > 1)
        return fail(c, SWE_ERR_BAD_ARG, "swe_halo: bad argument");
    if (fp32(c)) return fail(c, SWE_ERR_UNSUPPORTED, "swe_halo: slabs are FP64 only");
    int st = set_device(c);
    if (st) return st;
    void *const *buf = buffer == 0 ? c->Un : (buffer == 1 ? c->U1 : c->U2);
    // ghosted row index of the first of the two rows
    const int r0 = op == 0 ? (side == 0 ? NG : c->p.Nx) : (side == 0 ? 0 : c->p.Nx + NG);
    const size_t row = (size_t)(c->p.Ny + 4) * sizeof(double);
    const size_t dp = (size_t)c->pitch * sizeof(double);
    for (int f = 0; f < 3; ++f) {
        double *dev = static_cast<double *>(buf[f]) + (size_t)r0 * c->pitch;
        double *hst = rows + (size_t)f * 2 * (c->p.Ny + 4);
        if (op == 0)
            CK(cudaMemcpy2DAsync(hst, row, dev, dp, row, 2, cudaMemcpyDefault, c->stream));
        else
            CK(cudaMemcpy2DAsync(dev, dp, hst, row, row, 2, cudaMemcpyDefault, c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return SWE_OK;
}

int swe_max_wave_speed(swe_ctx *c, double *out) {
    if (!c || !out) return fail(c, SWE_ERR_BAD_ARG, "swe_max_wave_speed: null argument");
    if (!c->uploaded) return fail(c, SWE_ERR_BAD_ARG, "swe_max_wave_speed: no state uploaded");
    int st = set_device(c);
    if (st) return st;
    unsigned long long bits = 0;
    CK(cudaMemcpyAsync(&bits, c->speed + (c->steps_done & 1), sizeof bits,
                       cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    std::memcpy(out, &bits, sizeof(double));
    return SWE_OK;
}

int swe_stable_dt(swe_ctx *c, double *out) {
    if (!out) return fail(c, SWE_ERR_BAD_ARG, "swe_stable_dt: null argument");
    if (c && modular(c)) {
        if (!c->uploaded) return fail(c, SWE_ERR_BAD_ARG, "swe_stable_dt: no state uploaded");
        int st = set_device(c);
        if (st) return st;
        unsigned long long *slot = c->speed + (c->steps_done & 1);
        CK(cudaMemsetAsync(c->flags, 0, sizeof(int), c->stream));
        CK(launch_modular_stable_dt(c->Un[0], c->Un[1], c->Un[2], c->p.Nx, c->p.Ny, c->pitch,
                                    c->p.g, c->p.cfl, c->dx, c->dy, slot, c->flags, c->num_sms,
                                    c->stream));
        ++c->launches;
        unsigned long long bits = 0;
        int flags = 0;
        CK(cudaMemcpyAsync(&bits, slot, sizeof bits, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(&flags, c->flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        st = refresh_speed(c);  // the slot held the max wave speed
        if (st) return st;
        CK(cudaStreamSynchronize(c->stream));
        if (flags & FLAG_NONFINITE)
            return fail(c, SWE_ERR_BAD_ARG,
                        "Could not perform stability check for dt because h <= 0!");
        std::memcpy(out, &bits, sizeof(double));
        return SWE_OK;
    }
    double ms = 0.0;
    int st = swe_max_wave_speed(c, &ms);
    if (st) return st;
    *out = (ms <= 1.0e-8) ? 1.0e100 : c->cfl_min_dxdy / ms;  // HPC_kernels.hpp:296-297
    return SWE_OK;
}

int swe_totals(swe_ctx *c, double *mass, double *mx, double *my) {
    if (!c || !mass || !mx || !my) return fail(c, SWE_ERR_BAD_ARG, "swe_totals: null argument");
    if (!c->uploaded) return fail(c, SWE_ERR_BAD_ARG, "swe_totals: no state uploaded");
    int st = set_device(c);
    if (st) return st;
    if (!c->partial)
        CK(cudaMalloc(&c->partial, (6 * (size_t)totals_blocks(c->num_sms) + 4) * sizeof(double)));
    double *out = c->partial + 6 * totals_blocks(c->num_sms);
    CK(launch_totals(c->Un[0], c->Un[1], c->Un[2], c->B, fp32(c), c->p.Nx, c->p.Ny, c->pitch,
                     c->dx * c->dy, c->partial, out, c->num_sms, c->stream));
    c->launches += 2;
    double r[3];
    CK(cudaMemcpyAsync(r, out, sizeof r, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *mass = r[0];
    *mx = r[1];
    *my = r[2];
    return SWE_OK;
}

int swe_sanity(swe_ctx *c, double *mass, double *h_min, long long *first_negative,
               double *energy) {
    if (!c || !mass || !h_min || !first_negative || !energy)
        return fail(c, SWE_ERR_BAD_ARG, "swe_sanity: null argument");
    if (!c->uploaded) return fail(c, SWE_ERR_BAD_ARG, "swe_sanity: no state uploaded");
    int st = set_device(c);
    if (st) return st;
    if (!c->partial)
        CK(cudaMalloc(&c->partial, (6 * (size_t)totals_blocks(c->num_sms) + 4) * sizeof(double)));
    double *out = c->partial + 6 * totals_blocks(c->num_sms);
    CK(launch_sanity(c->Un[0], c->Un[1], c->Un[2], c->B, fp32(c), c->p.Nx, c->p.Ny, c->pitch,
                     c->p.g, c->dx * c->dy, c->partial, out, c->num_sms, c->stream));
    c->launches += 2;
    double r[4];
    CK(cudaMemcpyAsync(r, out, sizeof r, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *mass = r[0];
    *energy = r[1];
    *h_min = r[2];
    std::memcpy(first_negative, &r[3], sizeof(long long));
    return SWE_OK;
}

int swe_test_preset_timeout(swe_ctx *c) {
    if (!c) return SWE_ERR_BAD_ARG;
    c->preset_timeout = true;
    return SWE_OK;
}

int swe_last_step_ms(const swe_ctx *c, double *ms) {
    if (!c || !ms) return SWE_ERR_BAD_ARG;
    *ms = c->last_ms;
    return SWE_OK;
}

int swe_dt_log(swe_ctx *c, double *out, int n, int *written) {
    if (!c || !out || n < 0) return fail(c, SWE_ERR_BAD_ARG, "swe_dt_log: bad argument");
    const int m = std::min(n, c->last_steps);
    if (written) *written = m;
    if (m == 0) return SWE_OK;
    if (modular(c)) {  // fixed dt
        for (int k = 0; k < m; ++k) out[k] = c->modular_dt;
        return SWE_OK;
    }
    CK(cudaMemcpyAsync(out, c->dt_log, (size_t)m * sizeof(double), cudaMemcpyDeviceToHost,
                       c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return SWE_OK;
}

}  // extern "C"
