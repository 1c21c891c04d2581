// One grid split into x-slabs over one or several GPUs of this process, with the halo
// exchange and the CFL reduction kept on the devices (C ABI: swe_slabs_* in
// include/swe_gb300.h).
//
// The reference's 4-GPU backend (include/backend/cuda/four_gpu/cuda_solver_4gpu.hpp)
// splits the rows into contiguous slabs (build_subdomains, :281-304) and, around every
// stage, synchronises all devices and copies nG ghost rows between neighbours with
// cudaMemcpyPeer (exchange_one_array, :480-505).  Here every slab is an swe_ctx with
// x_halo set on its interface sides, and a step is enqueued without a host round trip:
//
//  - stage s of every slab first runs on its inner tile rows, which read no ghost rows
//    (inner_end);
//  - each slab's stream then waits for the events of its neighbours' copies into the
//    ghost rows of the stage source, and runs the edge tile rows (the first, and the one
//    or two at the end);
//  - after the stage, each slab copies its two interface rows of the buffer it wrote
//    (three fields, 2 x pitch contiguous doubles each) into its neighbours' ghost rows
//    with cudaMemcpyPeerAsync on its own stream, and records an event;
//  - after stage 3, each slab publishes the max wave speed it reduced, and every slab
//    gathers all of them (8-byte peer copies) and writes their max into its own slot,
//    so every slab computes the same dt from the same global max.
//
// The copies of one stage overlap the inner tile rows of the next.  The result is
// bitwise that of one context over the whole grid: every interface sees the same
// stencil values, and the global max is exact.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/swe_gb300.h"
#include "swe_ctx.h"
#include "swe_launch.h"

using namespace swe;

namespace {

__global__ void k_max_of_slots(const unsigned long long *gathered, int n,
                               unsigned long long *slot) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned long long m = 0;  // bit patterns of non-negative doubles order as the values
    for (int j = 0; j < n; ++j) m = gathered[j] > m ? gathered[j] : m;
    *slot = m;
}

}  // namespace

struct swe_slabs {
    swe_params p{};                  // the whole grid
    int parts = 0;
    std::vector<int> r0, r1;         // interior row range of each slab
    std::vector<swe_ctx *> s;
    std::vector<cudaEvent_t> sent;   // per slab: its copies of the last stage are done
    // per slab, on its device: [0, 2) the published max speed by step parity, [2, 2 + parts)
    // the gathered values
    std::vector<unsigned long long *> words;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;  // on slab 0's stream
    double last_ms = 0.0;
    long long launches = 0;
    std::string err;
};

namespace {

int sfail(swe_slabs *g, int status, const std::string &msg) {
    if (g) g->err = msg;
    return status;
}

#define SCK(call)                                                                             \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return sfail(g, SWE_ERR_CUDA, std::string(#call " failed: ") +                    \
                                              cudaGetErrorString(e_));                         \
    } while (0)

void *const *buffer(swe_ctx *c, int b) { return b == 0 ? c->Un : (b == 1 ? c->U1 : c->U2); }

int tile_rows(const swe_ctx *c) { return (c->p.Nx + TILE_I_F64 - 1) / TILE_I_F64; }

// End of the inner tile rows [1, inner_end): tile row t reads rows 8t - 2 .. 8t + 9, so it
// reads no ghost row when t >= 1 and 8t + 9 <= Nx - 1.
int inner_end(const swe_ctx *c) {
    return std::min(tile_rows(c), std::max(1, (c->p.Nx - 2) / TILE_I_F64));
}

// Copies slab k's two interface rows of buffer b into its neighbours' ghost rows, on
// slab k's stream, and records its `sent` event.
int send_halos(swe_slabs *g, int k, int b) {
    swe_ctx *c = g->s[k];
    const size_t rows2 = 2 * (size_t)c->pitch * sizeof(double);
    for (int side = 0; side < 2; ++side) {
        const int m = side == 0 ? k - 1 : k + 1;
        if (m < 0 || m >= g->parts) continue;
        swe_ctx *d = g->s[m];
        // ghosted row of the first of the two rows, in k (source) and m (destination)
        const size_t src_row = side == 0 ? NG : (size_t)c->p.Nx;
        const size_t dst_row = side == 0 ? (size_t)d->p.Nx + NG : 0;
        for (int f = 0; f < 3; ++f) {
            const char *src = static_cast<const char *>(buffer(c, b)[f]) +
                              src_row * c->pitch * sizeof(double);
            char *dst = static_cast<char *>(buffer(d, b)[f]) + dst_row * d->pitch * sizeof(double);
            SCK(cudaMemcpyPeerAsync(dst, d->p.device, src, c->p.device, rows2, c->stream));
        }
    }
    SCK(cudaEventRecord(g->sent[k], c->stream));
    return SWE_OK;
}

// Every slab's speed slot `slot` := the max over all slabs (published by parity `par`).
int global_speed(swe_slabs *g, int slot, int par) {
    for (int j = 0; j < g->parts; ++j) {
        swe_ctx *c = g->s[j];
        SCK(cudaSetDevice(c->p.device));
        SCK(cudaMemcpyAsync(g->words[j] + par, c->speed + slot, sizeof(unsigned long long),
                            cudaMemcpyDeviceToDevice, c->stream));
        SCK(cudaEventRecord(g->sent[j], c->stream));
    }
    for (int k = 0; k < g->parts; ++k) {
        swe_ctx *c = g->s[k];
        SCK(cudaSetDevice(c->p.device));
        for (int j = 0; j < g->parts; ++j) {
            if (j != k) SCK(cudaStreamWaitEvent(c->stream, g->sent[j], 0));
            SCK(cudaMemcpyPeerAsync(g->words[k] + 2 + j, c->p.device, g->words[j] + par,
                                    g->s[j]->p.device, sizeof(unsigned long long), c->stream));
        }
        k_max_of_slots<<<1, 32, 0, c->stream>>>(g->words[k] + 2, g->parts, c->speed + slot);
        SCK(cudaGetLastError());
        ++g->launches;
    }
    // the gathers read other slabs' words: every later write to them (the next step's
    // publication on the other parity, the one after on this one) follows a global max
    // that waits for this one on every slab
    for (int j = 0; j < g->parts; ++j) {
        SCK(cudaSetDevice(g->s[j]->p.device));
        SCK(cudaEventRecord(g->sent[j], g->s[j]->stream));
    }
    return SWE_OK;
}

int sync_all(swe_slabs *g) {
    for (swe_ctx *c : g->s) {
        SCK(cudaSetDevice(c->p.device));
        SCK(cudaStreamSynchronize(c->stream));
    }
    return SWE_OK;
}

}  // namespace

extern "C" {

int swe_slabs_create(const swe_params *pin, int parts, const int *devices, swe_slabs **out) try {
    if (!pin || !out || parts < 1) return SWE_ERR_BAD_ARG;
    *out = nullptr;
    swe_params p = *pin;
    if (p.g <= 0.0) p.g = 9.80665;
    if (p.precision != SWE_PRECISION_FP64 || p.scheme != SWE_SCHEME_FUSED || p.x_halo_lo ||
        p.x_halo_hi)
        return SWE_ERR_UNSUPPORTED;  // slabs are an FP64 drop-in feature
    if (p.Nx < 2 * parts || p.Ny < 2 || !(p.Lx > 0.0) || !(p.Ly > 0.0)) return SWE_ERR_BAD_ARG;
    swe_slabs *g = new (std::nothrow) swe_slabs();
    if (!g) return SWE_ERR_BAD_ARG;
    g->p = p;
    g->parts = parts;
    const double dx = p.dx > 0.0 ? p.dx : p.Lx / p.Nx, dy = p.dy > 0.0 ? p.dy : p.Ly / p.Ny;
    auto cleanup = [&](int st) {
        swe_slabs_destroy(g);
        return st;
    };
    for (int k = 0; k < parts; ++k) {
        // rows split as evenly as possible (build_subdomains, cuda_solver_4gpu.hpp:281-304)
        const int a = (int)((long long)k * p.Nx / parts), b = (int)((long long)(k + 1) * p.Nx / parts);
        g->r0.push_back(a);
        g->r1.push_back(b);
        swe_params q = p;
        q.Nx = b - a;
        q.Lx = dx * q.Nx;
        q.dx = dx;  // the whole grid's cell sizes, bit for bit
        q.dy = dy;
        q.x_halo_lo = k > 0;
        q.x_halo_hi = k < parts - 1;
        q.device = devices ? devices[k] : p.device;
        swe_ctx *c = nullptr;
        const int st = swe_create(&q, &c);
        if (st != SWE_OK) return cleanup(st);
        g->s.push_back(c);
        cudaEvent_t ev = nullptr;
        unsigned long long *w = nullptr;
        if (cudaSetDevice(q.device) != cudaSuccess ||
            cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
            return cleanup(SWE_ERR_CUDA);
        g->sent.push_back(ev);
        if (cudaMalloc(&w, (2 + (size_t)parts) * sizeof(unsigned long long)) != cudaSuccess ||
            cudaMemset(w, 0, (2 + (size_t)parts) * sizeof(unsigned long long)) != cudaSuccess) {
            cudaGetLastError();
            return cleanup(SWE_ERR_CUDA);
        }
        g->words.push_back(w);
    }
    // direct peer copies between neighbouring devices where the hardware allows them (the
    // driver stages through the host otherwise)
    for (int k = 0; k + 1 < parts; ++k) {
        const int a = g->s[k]->p.device, b = g->s[k + 1]->p.device;
        if (a == b) continue;
        for (int dir = 0; dir < 2; ++dir) {
            const int from = dir ? b : a, to = dir ? a : b;
            int can = 0;
            if (cudaDeviceCanAccessPeer(&can, from, to) == cudaSuccess && can) {
                cudaSetDevice(from);
                const cudaError_t e = cudaDeviceEnablePeerAccess(to, 0);
                if (e != cudaSuccess && e != cudaErrorPeerAccessAlreadyEnabled)
                    return cleanup(SWE_ERR_CUDA);
            }
            cudaGetLastError();
        }
    }
    if (cudaSetDevice(g->s[0]->p.device) != cudaSuccess || cudaEventCreate(&g->ev0) != cudaSuccess ||
        cudaEventCreate(&g->ev1) != cudaSuccess)
        return cleanup(SWE_ERR_CUDA);
    *out = g;
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

void swe_slabs_destroy(swe_slabs *g) {
    if (!g) return;
    for (size_t k = 0; k < g->s.size(); ++k) {
        cudaSetDevice(g->s[k]->p.device);
        cudaStreamSynchronize(g->s[k]->stream);
        if (k < g->sent.size() && g->sent[k]) cudaEventDestroy(g->sent[k]);
        if (k < g->words.size() && g->words[k]) cudaFree(g->words[k]);
        swe_destroy(g->s[k]);
    }
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    cudaGetLastError();
    delete g;
}

int swe_slabs_upload(swe_slabs *g, const double *h, const double *hu, const double *hv,
                     const double *B) try {
    if (!g || !h || !hu || !hv || !B) return sfail(g, SWE_ERR_BAD_ARG, "swe_slabs_upload: null argument");
    const size_t W = (size_t)g->p.Ny + 4;
    for (int k = 0; k < g->parts; ++k) {
        // the slab's rows plus two on either side (its neighbours' rows or the grid's ghosts)
        const size_t off = (size_t)g->r0[k] * W;
        const int st = swe_upload(g->s[k], h + off, hu + off, hv + off, B + off);
        if (st) return sfail(g, st, std::string("swe_slabs_upload: ") + swe_last_error(g->s[k]));
    }
    // every slab's slot 0 holds its own max speed; make it the grid's
    int st = global_speed(g, 0, 0);
    if (st) return st;
    return sync_all(g);
} catch (...) {
    return SWE_ERR_BAD_ARG;
}

int swe_slabs_download(swe_slabs *g, double *h, double *hu, double *hv) try {
    if (!g || !h || !hu || !hv) return sfail(g, SWE_ERR_BAD_ARG, "swe_slabs_download: null argument");
    const size_t W = (size_t)g->p.Ny + 4;
    std::vector<double> a, b, c;
    for (int k = 0; k < g->parts; ++k) {
        const size_t n = (size_t)(g->r1[k] - g->r0[k] + 4) * W;
        a.resize(n);
        b.resize(n);
        c.resize(n);
        const int st = swe_download(g->s[k], a.data(), b.data(), c.data());
        if (st) return sfail(g, st, std::string("swe_slabs_download: ") + swe_last_error(g->s[k]));
        // rows of the slab; the first slab also gives the low ghosts, the last the high ones
        const int lo = k == 0 ? 0 : NG;
        const int hi = g->r1[k] - g->r0[k] + (k == g->parts - 1 ? 2 * NG : NG);
        const size_t dst = ((size_t)g->r0[k] + lo) * W, src = (size_t)lo * W, len = (size_t)(hi - lo) * W;
        std::memcpy(h + dst, a.data() + src, len * sizeof(double));
        std::memcpy(hu + dst, b.data() + src, len * sizeof(double));
        std::memcpy(hv + dst, c.data() + src, len * sizeof(double));
    }
    return SWE_OK;
} catch (...) {
    return SWE_ERR_BAD_ARG;
}

int swe_slabs_step(swe_slabs *g, int n_steps, double dt, double *t_inout) try {
    if (!g || n_steps < 0 || !(dt == dt)) return sfail(g, SWE_ERR_BAD_ARG, "swe_slabs_step: bad argument");
    for (swe_ctx *c : g->s)
        if (!c->uploaded) return sfail(g, SWE_ERR_BAD_ARG, "swe_slabs_step: no state uploaded");
    if (n_steps == 0) return SWE_OK;
    const double t0 = t_inout ? *t_inout : 0.0;
    for (swe_ctx *c : g->s) {
        SCK(cudaSetDevice(c->p.device));
        SCK(cudaMemcpyAsync(c->t_accum, &t0, sizeof(double), cudaMemcpyHostToDevice, c->stream));
        SCK(cudaMemsetAsync(c->flags, 0, sizeof(int), c->stream));
    }
    SCK(cudaSetDevice(g->s[0]->p.device));
    SCK(cudaEventRecord(g->ev0, g->s[0]->stream));
    for (int k = 1; k < g->parts; ++k) {  // slab 0's timing covers every slab's work
        SCK(cudaSetDevice(g->s[k]->p.device));
        SCK(cudaStreamWaitEvent(g->s[k]->stream, g->ev0, 0));
    }
    for (int n = 0; n < n_steps; ++n) {
        const int slot_read = (int)(g->s[0]->steps_done & 1);
        for (int stage = 1; stage <= 3; ++stage) {
            const int src = stage - 1, dst = stage % 3;
            std::vector<StageParams> sp(g->parts);
            for (int k = 0; k < g->parts; ++k) {
                swe_ctx *c = g->s[k];
                sp[k] = ctx_stage_params(c, dt);
                sp[k].slot_read = slot_read;
                sp[k].slot_write = slot_read ^ 1;
                sp[k].dt_log = nullptr;
                sp[k].hn = c->Un[0]; sp[k].hun = c->Un[1]; sp[k].hvn = c->Un[2];
                sp[k].hs = buffer(c, src)[0]; sp[k].hus = buffer(c, src)[1]; sp[k].hvs = buffer(c, src)[2];
                sp[k].ho = buffer(c, dst)[0]; sp[k].huo = buffer(c, dst)[1]; sp[k].hvo = buffer(c, dst)[2];
            }
            // inner tile rows: their stencils read no ghost row
            for (int k = 0; k < g->parts; ++k) {
                swe_ctx *c = g->s[k];
                const int e = inner_end(c);
                if (e <= 1) continue;
                SCK(cudaSetDevice(c->p.device));
                SCK(launch_stage_f64(stage, sp[k], c->maps_ok ? &c->maps[src] : nullptr,
                                     c->stream, 1, e));
                ++g->launches;
            }
            // edge tile rows (the first, and those from inner_end on), once the neighbours'
            // rows of the source have landed
            for (int k = 0; k < g->parts; ++k) {
                swe_ctx *c = g->s[k];
                const int T = tile_rows(c), e = inner_end(c);
                SCK(cudaSetDevice(c->p.device));
                if (k > 0) SCK(cudaStreamWaitEvent(c->stream, g->sent[k - 1], 0));
                if (k + 1 < g->parts) SCK(cudaStreamWaitEvent(c->stream, g->sent[k + 1], 0));
                const StageMaps *m = c->maps_ok ? &c->maps[src] : nullptr;
                if (e <= 1) {
                    SCK(launch_stage_f64(stage, sp[k], m, c->stream, 0, T));
                    ++g->launches;
                } else {
                    SCK(launch_stage_f64(stage, sp[k], m, c->stream, 0, 1));
                    if (e < T) {
                        SCK(launch_stage_f64(stage, sp[k], m, c->stream, e, T));
                        ++g->launches;
                    }
                    ++g->launches;
                }
            }
            // the rows this stage wrote, to the neighbours
            for (int k = 0; k < g->parts; ++k) {
                SCK(cudaSetDevice(g->s[k]->p.device));
                const int st = send_halos(g, k, dst);
                if (st) return st;
            }
        }
        for (swe_ctx *c : g->s) ++c->steps_done;
        // publication parity by the step count, so that consecutive steps alternate across
        // calls too (a call ends with every stream synchronised)
        const int st = global_speed(g, slot_read ^ 1, (int)(g->s[0]->steps_done & 1));
        if (st) return st;
    }
    for (int k = 1; k < g->parts; ++k) {
        SCK(cudaSetDevice(g->s[k]->p.device));
        SCK(cudaEventRecord(g->sent[k], g->s[k]->stream));
        SCK(cudaSetDevice(g->s[0]->p.device));
        SCK(cudaStreamWaitEvent(g->s[0]->stream, g->sent[k], 0));
    }
    SCK(cudaSetDevice(g->s[0]->p.device));
    SCK(cudaEventRecord(g->ev1, g->s[0]->stream));
    int st = sync_all(g);
    if (st) return st;
    float ms = 0.f;
    SCK(cudaEventElapsedTime(&ms, g->ev0, g->ev1));
    g->last_ms = ms;
    int flags = 0;
    double t1 = 0.0;
    for (swe_ctx *c : g->s) {
        int f = 0;
        SCK(cudaSetDevice(c->p.device));
        SCK(cudaMemcpy(&f, c->flags, sizeof(int), cudaMemcpyDeviceToHost));
        flags |= f;
        c->last_steps = n_steps;
    }
    SCK(cudaSetDevice(g->s[0]->p.device));
    SCK(cudaMemcpy(&t1, g->s[0]->t_accum, sizeof(double), cudaMemcpyDeviceToHost));
    if (t_inout) *t_inout = t1;
    if (flags & FLAG_TIMEOUT)
        return sfail(g, SWE_ERR_TIMEOUT, "a tile's TMA copy did not complete (state undefined)");
    if (flags & FLAG_NONFINITE)
        return sfail(g, SWE_ERR_NONFINITE, "non-finite state detected in GB300 solver");
    return SWE_OK;
} catch (...) {
    return SWE_ERR_BAD_ARG;
}

int swe_slabs_last_step_ms(const swe_slabs *g, double *ms) {
    if (!g || !ms) return SWE_ERR_BAD_ARG;
    *ms = g->last_ms;
    return SWE_OK;
}

long long swe_slabs_kernel_launches(const swe_slabs *g) { return g ? g->launches : 0; }

const char *swe_slabs_last_error(const swe_slabs *g) { return g ? g->err.c_str() : "null slabs"; }

}  // extern "C"
