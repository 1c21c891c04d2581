// Batched ensemble of independent grids of uneven sizes (C ABI in include/swe_gb300.h).
//
// Every instance's h/eta, hu, hv (three state sets) and B live at its own offset in ten
// shared field pools.  One launch per RK stage covers all instances: the work list
// holds every (instance, tile) pair, CTAs stride over it, and each tile reads its
// instance's dt from that instance's max-speed slot (per-instance CFL).  A whole RK3
// step (three launches) is captured once per slot parity in a CUDA graph and replayed.
// The tile shape and the number of CTAs are chosen by swe_ens_tune, which times every
// candidate on the actual ensemble and restores the state afterwards.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/swe_gb300.h"
#include "swe_launch.h"

using namespace swe;

struct swe_ens {
    swe_params base{};
    int n = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 0;
    int resident[8] = {-1, -1, -1, -1, -1, -1, -1, -1};  // CTAs per SM by shape, -1: not queried
    bool f32 = false;
    size_t elem = 8;
    std::vector<EnsInst> inst;  // host copy (tiles_j / tile_base for the current shape)
    std::vector<double> Lx, Ly;
    size_t pool_elems = 0;
    void *base_ptr = nullptr;
    void *Un[3]{}, *U1[3]{}, *U2[3]{}, *B = nullptr;
    void *snap = nullptr;          // tuner snapshot of U^n pools + per-instance scalars
    EnsInst *d_inst = nullptr;
    int *d_tile_inst = nullptr;
    int total_tiles = 0;
    CUtensorMap *d_maps = nullptr;  // FP32: per instance and stage source, current shape
    unsigned long long *d_speed = nullptr;  // 2 per instance
    double *d_t = nullptr, *d_dt = nullptr;
    int *d_flags = nullptr;
    void *stage64[2]{};            // FP32: FP64 staging for the largest instance
    long long max_field = 0;
    std::vector<char> uploaded;
    long long steps_done = 0;
    int shape = SHAPE_8x32;
    int grid = 0;                  // CTAs; 0 = one per tile
    cudaGraphExec_t graph[2]{};    // by slot parity
    double graph_dt = -1.0;
    int graph_shape = -1, graph_grid = -1;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    double last_ms = 0.0;
    long long launches = 0;
    bool preset_timeout = false;   // swe_ens_test_preset_timeout: the next step's flag
    std::string err;
};

namespace {

int efail(swe_ens *c, int status, const char *fmt, ...) {
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

#define ECK(call)                                                                             \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess)                                                                \
            return efail(c, SWE_ERR_CUDA, "%s failed: %s (%s:%d)", #call,                     \
                         cudaGetErrorString(e_), __FILE__, __LINE__);                         \
    } while (0)

int pow2_exp(double x) {
    int k = 0;
    const double m = std::frexp(x, &k);
    if (m != 0.5 || !(x > 0.0) || k - 1 < -64 || k - 1 > 64) return 127;
    return k - 1;
}

void shape_dims(int shape, int &TI, int &TJ) {
    switch (shape) {
        case SHAPE_8x16: TI = 8; TJ = 16; break;
        case SHAPE_4x64: TI = 4; TJ = 64; break;
        case SHAPE_16x32: TI = 16; TJ = 32; break;
        case SHAPE_8x64: TI = 8; TJ = 64; break;
        case SHAPE_COLS: TI = F32_STRIP_ROWS; TJ = F32_COL_BLOCK; break;
        case SHAPE_STRIP: TI = 8 * F64_STRIP_TILES; TJ = 32; break;
        default: TI = 8; TJ = 32; break;
    }
}

bool shape_ok(const swe_ens *c, int shape) {
    if (c->f32)
        return shape == SHAPE_8x32 || shape == SHAPE_16x32 || shape == SHAPE_8x64 ||
               shape == SHAPE_COLS;
    return shape == SHAPE_8x32 || shape == SHAPE_8x16 || shape == SHAPE_4x64 ||
           shape == SHAPE_STRIP;
}

void destroy_graphs(swe_ens *c) {
    for (auto &g : c->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    c->graph_shape = -1;
}

// FP32 form: TMA maps of every instance's three stage sources for a TI x TJ tile (box
// (TI + 4) x (TJ + 4)).  Instances too small for an interior tile never use theirs (a
// failed encode leaves it zero); any other failure, or SWE_GB300_NO_TMA=1, leaves every
// tile on the mirrored-index loader.
void build_maps(swe_ens *c, int TI, int TJ) {
    if (c->d_maps) cudaFree(c->d_maps);
    c->d_maps = nullptr;
    const char *off = std::getenv("SWE_GB300_NO_TMA");
    if (off && off[0] == '1') return;
    std::vector<CUtensorMap> maps((size_t)c->n * 12);
    std::memset(maps.data(), 0, maps.size() * sizeof(CUtensorMap));
    void *const *src[3] = {c->Un, c->U1, c->U2};
    for (int q = 0; q < c->n; ++q) {
        const EnsInst &I = c->inst[q];
        const bool used = I.Nx >= TI + 4 && I.Ny >= TJ + 4;  // can hold an interior tile
        const size_t o = (size_t)I.off * c->elem;
        for (int s = 0; s < 3; ++s) {
            const void *base[4] = {static_cast<char *>(src[s][0]) + o,
                                   static_cast<char *>(src[s][1]) + o,
                                   static_cast<char *>(src[s][2]) + o,
                                   static_cast<char *>(c->B) + o};
            for (int f = 0; f < 4; ++f) {
                CUtensorMap &m = maps[((size_t)q * 3 + s) * 4 + f];
                if (!encode_tile_map(&m, base[f], I.Nx + 4, I.Ny + 4, I.pitch, TI + 4, TJ + 4,
                                     (int)c->elem)) {
                    if (used) return;
                    std::memset(&m, 0, sizeof m);
                }
            }
        }
    }
    if (cudaMalloc(&c->d_maps, maps.size() * sizeof(CUtensorMap)) != cudaSuccess) {
        cudaGetLastError();
        c->d_maps = nullptr;
        return;
    }
    if (cudaMemcpy(c->d_maps, maps.data(), maps.size() * sizeof(CUtensorMap),
                   cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(c->d_maps);
        c->d_maps = nullptr;
    }
}

// Work list for the current tile shape (instances in order, tiles row-major).
int build_tiles(swe_ens *c) {
    int TI, TJ;
    shape_dims(c->shape, TI, TJ);
    std::vector<int> tile_inst;
    long long total = 0;
    for (int q = 0; q < c->n; ++q) {
        EnsInst &I = c->inst[q];
        const int ti = (I.Nx + TI - 1) / TI, tj = (I.Ny + TJ - 1) / TJ;
        I.tiles_j = tj;
        I.tile_base = (int)total;
        total += (long long)ti * tj;
        if (total >= (1ll << 31)) return efail(c, SWE_ERR_BAD_ARG, "ensemble too large");
    }
    tile_inst.resize((size_t)total);
    for (int q = 0; q < c->n; ++q) {
        const EnsInst &I = c->inst[q];
        const int ntiles = ((I.Nx + TI - 1) / TI) * I.tiles_j;
        std::fill(tile_inst.begin() + I.tile_base, tile_inst.begin() + I.tile_base + ntiles, q);
    }
    if (c->d_tile_inst) ECK(cudaFree(c->d_tile_inst));
    c->d_tile_inst = nullptr;
    ECK(cudaMalloc(&c->d_tile_inst, tile_inst.size() * sizeof(int)));
    ECK(cudaMemcpyAsync(c->d_tile_inst, tile_inst.data(), tile_inst.size() * sizeof(int),
                        cudaMemcpyHostToDevice, c->stream));
    ECK(cudaMemcpyAsync(c->d_inst, c->inst.data(), c->inst.size() * sizeof(EnsInst),
                        cudaMemcpyHostToDevice, c->stream));
    ECK(cudaStreamSynchronize(c->stream));
    c->total_tiles = (int)total;
    destroy_graphs(c);
    if (c->f32 && c->shape != SHAPE_COLS) {
        build_maps(c, TI, TJ);
    } else if (c->d_maps) {  // the column sweeps read global memory directly
        cudaFree(c->d_maps);
        c->d_maps = nullptr;
    }
    return SWE_OK;
}

EnsParams stage_params(const swe_ens *c, int stage, int slot_read, double dt_fixed) {
    EnsParams e{};
    void *const *src = stage == 1 ? c->Un : (stage == 2 ? c->U1 : c->U2);
    void *const *out = stage == 1 ? c->U1 : (stage == 2 ? c->U2 : c->Un);
    for (int f = 0; f < 3; ++f) {
        e.src[f] = src[f];
        e.n[f] = c->Un[f];
        e.out[f] = out[f];
    }
    e.B = c->B;
    e.inst = c->d_inst;
    e.tile_inst = c->d_tile_inst;
    e.total_tiles = c->total_tiles;
    e.bc = c->base.bc;
    e.g = c->base.g;
    e.half_g = 0.5 * c->base.g;
    e.gf = (float)e.g;
    e.half_gf = (float)e.half_g;
    e.dt_fixed = dt_fixed > 0.0 ? dt_fixed : 0.0;
    e.speed = c->d_speed;
    e.slot_read = slot_read;
    e.slot_write = slot_read ^ 1;
    e.t = c->d_t;
    e.dt_last = c->d_dt;
    e.flags = c->d_flags;
    e.elem = (int)c->elem;
    e.maps = c->d_maps;
    return e;
}

// CTAs per SM of a shape (the occupancy query, once per shape and ensemble).
int resident_per_sm(swe_ens *c, int shape) {
    if (shape < 0 || shape >= 8) return 0;
    if (c->resident[shape] < 0)
        c->resident[shape] = c->f32 ? ens_resident_per_sm_f32(shape) : ens_resident_per_sm_f64(shape);
    return c->resident[shape];
}

// CTAs of the current shape resident on the whole GPU at once (0: unknown).
int resident_ctas(swe_ens *c) { return resident_per_sm(c, c->shape) * c->num_sms; }

// A persistent schedule never asks for more CTAs than fit at once: with every CTA
// resident, equal shares of the work list finish together instead of in waves.
int grid_ctas(swe_ens *c) {
    const int tiles = std::max(c->total_tiles, 1);
    if (c->grid <= 0) return tiles;
    int g = std::min(c->grid, tiles);
    const int r = resident_ctas(c);
    if (r > 0 && g > r) g = r;
    return g;
}

int launch_step(swe_ens *c, int slot_read, double dt_fixed) {
    const int grid = grid_ctas(c);
    for (int stage = 1; stage <= 3; ++stage) {
        const EnsParams e = stage_params(c, stage, slot_read, dt_fixed);
        ECK(c->f32 ? launch_ens_stage_f32(c->shape, stage, e, grid, c->stream)
                   : launch_ens_stage_f64(c->shape, stage, e, grid, c->stream));
    }
    return SWE_OK;
}

// CUDA graphs of one RK3 step for each slot parity; recaptured when the schedule or
// the fixed dt changes.
int ensure_graphs(swe_ens *c, double dt_fixed) {
    if (c->graph_shape == c->shape && c->graph_grid == c->grid && c->graph_dt == dt_fixed &&
        c->graph[0] && c->graph[1])
        return SWE_OK;
    destroy_graphs(c);
    for (int parity = 0; parity < 2; ++parity) {
        cudaGraph_t g = nullptr;
        ECK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int st = launch_step(c, parity, dt_fixed);
        cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (st != SWE_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        ECK(e);
        e = cudaGraphInstantiate(&c->graph[parity], g, 0);
        cudaGraphDestroy(g);
        ECK(e);
    }
    c->graph_shape = c->shape;
    c->graph_grid = c->grid;
    c->graph_dt = dt_fixed;
    return SWE_OK;
}

int refresh_speed_inst(swe_ens *c, int q) {
    const EnsInst &I = c->inst[q];
    const size_t off = (size_t)I.off * c->elem;
    unsigned long long *slot = c->d_speed + 2 * q + (c->steps_done & 1);
    ECK(cudaMemsetAsync(slot, 0, sizeof(unsigned long long), c->stream));
    auto at = [&](void *p) { return static_cast<char *>(p) + off; };
    if (c->f32) {
        ECK(launch_max_speed_f32(at(c->Un[0]), at(c->Un[1]), at(c->Un[2]), at(c->B), I.Nx, I.Ny,
                                 I.pitch, c->base.g, slot, c->num_sms, c->stream));
    } else {
        ECK(launch_max_speed_f64(at(c->Un[0]), at(c->Un[1]), at(c->Un[2]), I.Nx, I.Ny, I.pitch,
                                 c->base.g, slot, c->num_sms, c->stream));
    }
    ++c->launches;
    return SWE_OK;
}

int run_steps(swe_ens *c, int n_steps, double dt_fixed) {
    int st = ensure_graphs(c, dt_fixed);
    if (st) return st;
    for (int s = 0; s < n_steps; ++s) {
        ECK(cudaGraphLaunch(c->graph[c->steps_done & 1], c->stream));
        c->launches += 3;
        ++c->steps_done;
    }
    return SWE_OK;
}

}  // namespace

extern "C" {

int swe_ens_create(const swe_params *base, int n, const int *Nx, const int *Ny, const double *Lx,
                   const double *Ly, swe_ens **out) try {
    if (!base || !out || n <= 0 || !Nx || !Ny) return SWE_ERR_BAD_ARG;
    *out = nullptr;
    swe_params b = *base;
    if (b.g <= 0.0) b.g = 9.80665;
    if (b.nG != 2 || !(b.cfl > 0.0) || (b.bc != SWE_BC_REFLECTING && b.bc != SWE_BC_TRANSMISSIVE) ||
        (b.precision != SWE_PRECISION_FP64 && b.precision != SWE_PRECISION_FP32_MIXED))
        return SWE_ERR_BAD_ARG;
    if (b.scheme != SWE_SCHEME_FUSED) return SWE_ERR_UNSUPPORTED;  // the fused stage only
    for (int q = 0; q < n; ++q) {
        if (Nx[q] < 2 || Ny[q] < 2) return SWE_ERR_BAD_ARG;
        if ((Lx && !(Lx[q] > 0.0)) || (Ly && !(Ly[q] > 0.0))) return SWE_ERR_BAD_ARG;
        if ((long long)(Nx[q] + 4) * (Ny[q] + 36) >= (1ll << 31)) return SWE_ERR_BAD_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || b.device < 0 || b.device >= ndev) {
        cudaGetLastError();
        return SWE_ERR_NO_DEVICE;
    }
    swe_ens *c = new (std::nothrow) swe_ens();
    if (!c) return SWE_ERR_BAD_ARG;
    c->base = b;
    c->n = n;
    c->f32 = b.precision == SWE_PRECISION_FP32_MIXED;
    c->elem = c->f32 ? sizeof(float) : sizeof(double);
    c->inst.resize(n);
    c->uploaded.assign(n, 0);
    size_t off = 0;
    for (int q = 0; q < n; ++q) {
        EnsInst &I = c->inst[q];
        const double lx = Lx ? Lx[q] : 1.0, ly = Ly ? Ly[q] : 1.0;
        I.Nx = Nx[q];
        I.Ny = Ny[q];
        I.pitch = ((long long)(Ny[q] + 4) + 31) / 32 * 32;
        I.off = (long long)off;
        const double dx = lx / Nx[q], dy = ly / Ny[q];
        I.inv_dx = 1.0 / dx;
        I.inv_dy = 1.0 / dy;
        I.kx = pow2_exp(I.inv_dx);
        I.ky = pow2_exp(I.inv_dy);
        I.inv_dxf = (float)I.inv_dx;
        I.inv_dyf = (float)I.inv_dy;
        I.cfl_min_dxdy = b.cfl * std::min(dx, dy);
        const long long field = (long long)(Nx[q] + 4) * I.pitch;
        c->max_field = std::max(c->max_field, field);
        off += (size_t)field;
    }
    c->pool_elems = off;
    auto cleanup = [&](int s) {
        swe_ens_destroy(c);
        return s;
    };
    if (cudaSetDevice(b.device) != cudaSuccess) return cleanup(SWE_ERR_CUDA);
    cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, b.device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    const size_t fb = c->pool_elems * c->elem;
    const size_t staging = c->f32 ? 2 * (size_t)c->max_field * sizeof(double) : 0;
    if (e == cudaSuccess) e = cudaMalloc(&c->base_ptr, 10 * fb + staging);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_inst, n * sizeof(EnsInst));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_speed, 2 * n * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_t, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_dt, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&c->d_flags, sizeof(int));
    if (e != cudaSuccess) return cleanup(SWE_ERR_CUDA);
    char *p = static_cast<char *>(c->base_ptr);
    for (int f = 0; f < 3; ++f) {
        c->Un[f] = p + (0 + f) * fb;
        c->U1[f] = p + (3 + f) * fb;
        c->U2[f] = p + (6 + f) * fb;
    }
    c->B = p + 9 * fb;
    if (staging) {
        c->stage64[0] = p + 10 * fb;
        c->stage64[1] = p + 10 * fb + (size_t)c->max_field * sizeof(double);
    }
    e = cudaMemsetAsync(c->base_ptr, 0, 10 * fb + staging, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_speed, 0, 2 * n * sizeof(unsigned long long), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_t, 0, n * sizeof(double), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_dt, 0, n * sizeof(double), c->stream);
    if (e != cudaSuccess) return cleanup(SWE_ERR_CUDA);
    c->shape = SHAPE_8x32;
    c->grid = 0;
    if (build_tiles(c) != SWE_OK) return cleanup(SWE_ERR_CUDA);
    *out = c;
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

void swe_ens_destroy(swe_ens *c) try {
    if (!c) return;
    cudaSetDevice(c->base.device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    destroy_graphs(c);
    for (void *p : {(void *)c->base_ptr, (void *)c->snap, (void *)c->d_inst, (void *)c->d_tile_inst,
                    (void *)c->d_speed, (void *)c->d_t, (void *)c->d_dt, (void *)c->d_flags,
                    (void *)c->d_maps})
        if (p) cudaFree(p);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    cudaGetLastError();
    delete c;
} catch (...) {  // host allocation failures do not cross the C ABI
}

const char *swe_ens_last_error(const swe_ens *c) { return c ? c->err.c_str() : "null ensemble"; }

int swe_ens_upload(swe_ens *c, int q, const double *h, const double *hu, const double *hv,
                   const double *B) try {
    if (!c || q < 0 || q >= c->n || !h || !hu || !hv || !B)
        return efail(c, SWE_ERR_BAD_ARG, "swe_ens_upload: bad argument");
    ECK(cudaSetDevice(c->base.device));
    const EnsInst &I = c->inst[q];
    const size_t row = (size_t)(I.Ny + 4) * sizeof(double);
    const size_t rows = (size_t)(I.Nx + 4);
    const size_t off = (size_t)I.off * c->elem;
    auto at = [&](void *p) { return static_cast<char *>(p) + off; };
    if (c->f32) {
        const size_t dp = (size_t)I.pitch * sizeof(double);
        ECK(cudaMemcpy2DAsync(c->stage64[0], dp, B, row, row, rows, cudaMemcpyHostToDevice,
                              c->stream));
        ECK(launch_f64_to_f32(c->stage64[0], nullptr, at(c->B), I.Nx + 4, I.Ny + 4, I.pitch,
                              c->num_sms, c->stream));
        const double *src[3] = {h, hu, hv};
        for (int f = 0; f < 3; ++f) {
            ECK(cudaMemcpy2DAsync(c->stage64[1], dp, src[f], row, row, rows,
                                  cudaMemcpyHostToDevice, c->stream));
            ECK(launch_f64_to_f32(c->stage64[1], f == 0 ? c->stage64[0] : nullptr, at(c->Un[f]),
                                  I.Nx + 4, I.Ny + 4, I.pitch, c->num_sms, c->stream));
        }
        c->launches += 4;
    } else {
        const size_t dp = (size_t)I.pitch * sizeof(double);
        const double *src[4] = {h, hu, hv, B};
        void *dst[4] = {at(c->Un[0]), at(c->Un[1]), at(c->Un[2]), at(c->B)};
        for (int f = 0; f < 4; ++f)
            ECK(cudaMemcpy2DAsync(dst[f], dp, src[f], row, row, rows, cudaMemcpyHostToDevice,
                                  c->stream));
    }
    const double zero = 0.0;
    ECK(cudaMemcpyAsync(c->d_t + q, &zero, sizeof zero, cudaMemcpyHostToDevice, c->stream));
    int st = refresh_speed_inst(c, q);
    if (st) return st;
    ECK(cudaStreamSynchronize(c->stream));
    c->uploaded[q] = 1;
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

int swe_ens_download(swe_ens *c, int q, double *h, double *hu, double *hv) try {
    if (!c || q < 0 || q >= c->n || !h || !hu || !hv)
        return efail(c, SWE_ERR_BAD_ARG, "swe_ens_download: bad argument");
    ECK(cudaSetDevice(c->base.device));
    const EnsInst &I = c->inst[q];
    const size_t row = (size_t)(I.Ny + 4) * sizeof(double);
    const size_t rows = (size_t)(I.Nx + 4);
    const size_t off = (size_t)I.off * c->elem;
    auto at = [&](void *p) { return static_cast<char *>(p) + off; };
    double *dst[3] = {h, hu, hv};
    if (c->f32) {
        ECK(launch_fill_ghosts_f32(at(c->Un[0]), at(c->Un[1]), at(c->Un[2]), at(c->B), I.Nx, I.Ny,
                                   I.pitch, c->base.bc, c->stream));
        for (int f = 0; f < 3; ++f) {
            ECK(launch_f32_to_f64(at(c->Un[f]), f == 0 ? at(c->B) : nullptr, c->stage64[1],
                                  I.Nx + 4, I.Ny + 4, I.pitch, c->num_sms, c->stream));
            ECK(cudaMemcpy2DAsync(dst[f], row, c->stage64[1], (size_t)I.pitch * sizeof(double),
                                  row, rows, cudaMemcpyDeviceToHost, c->stream));
        }
        c->launches += 4;
    } else {
        ECK(launch_fill_ghosts_f64(at(c->Un[0]), at(c->Un[1]), at(c->Un[2]), I.Nx, I.Ny, I.pitch,
                                   c->base.bc, c->stream));
        ++c->launches;
        for (int f = 0; f < 3; ++f)
            ECK(cudaMemcpy2DAsync(dst[f], row, at(c->Un[f]), (size_t)I.pitch * sizeof(double),
                                  row, rows, cudaMemcpyDeviceToHost, c->stream));
    }
    ECK(cudaStreamSynchronize(c->stream));
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

int swe_ens_step(swe_ens *c, int n_steps, double dt) try {
    if (!c || n_steps < 0 || !(dt == dt)) return efail(c, SWE_ERR_BAD_ARG, "swe_ens_step: bad argument");
    for (int q = 0; q < c->n; ++q)
        if (!c->uploaded[q]) return efail(c, SWE_ERR_BAD_ARG, "swe_ens_step: instance %d not uploaded", q);
    if (n_steps == 0) return SWE_OK;
    ECK(cudaSetDevice(c->base.device));
    ECK(cudaMemsetAsync(c->d_flags, 0, sizeof(int), c->stream));
    if (c->preset_timeout) {  // the flag word's low byte (little-endian int)
        c->preset_timeout = false;
        ECK(cudaMemsetAsync(c->d_flags, FLAG_TIMEOUT, 1, c->stream));
    }
    ECK(cudaEventRecord(c->ev0, c->stream));
    int st = run_steps(c, n_steps, dt > 0.0 ? dt : 0.0);
    if (st) return st;
    ECK(cudaEventRecord(c->ev1, c->stream));
    int flags = 0;
    ECK(cudaMemcpyAsync(&flags, c->d_flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    ECK(cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    ECK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    c->last_ms = ms;
    if (flags & FLAG_TIMEOUT)
        return efail(c, SWE_ERR_TIMEOUT, "a tile's TMA copy did not complete (state undefined)");
    if (flags & FLAG_NONFINITE)
        return efail(c, SWE_ERR_NONFINITE, "non-finite state detected in GB300 ensemble");
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

int swe_ens_times(swe_ens *c, double *t) try {
    if (!c || !t) return efail(c, SWE_ERR_BAD_ARG, "swe_ens_times: bad argument");
    ECK(cudaMemcpyAsync(t, c->d_t, c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    ECK(cudaStreamSynchronize(c->stream));
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

int swe_ens_last_dt(swe_ens *c, double *dt) try {
    if (!c || !dt) return efail(c, SWE_ERR_BAD_ARG, "swe_ens_last_dt: bad argument");
    ECK(cudaMemcpyAsync(dt, c->d_dt, c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    ECK(cudaStreamSynchronize(c->stream));
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

int swe_ens_last_step_ms(const swe_ens *c, double *ms) try {
    if (!c || !ms) return SWE_ERR_BAD_ARG;
    *ms = c->last_ms;
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

long long swe_ens_kernel_launches(const swe_ens *c) { return c ? c->launches : 0; }

int swe_ens_test_preset_timeout(swe_ens *c) {
    if (!c) return SWE_ERR_BAD_ARG;
    c->preset_timeout = true;
    return SWE_OK;
}

int swe_ens_set_schedule(swe_ens *c, int shape, int grid) try {
    if (!c || grid < 0 || !shape_ok(c, shape))
        return efail(c, SWE_ERR_BAD_ARG, "swe_ens_set_schedule: unsupported shape %d", shape);
    ECK(cudaSetDevice(c->base.device));
    c->grid = grid;
    if (shape != c->shape) {
        c->shape = shape;
        return build_tiles(c);
    }
    destroy_graphs(c);
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

int swe_ens_get_schedule(const swe_ens *c, int *shape, int *grid, int *total_tiles) try {
    if (!c) return SWE_ERR_BAD_ARG;
    if (shape) *shape = c->shape;
    if (grid) *grid = c->grid;
    if (total_tiles) *total_tiles = c->total_tiles;
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

int swe_ens_tune(swe_ens *c, int steps, double *best_ms) try {
    if (!c || steps <= 0) return efail(c, SWE_ERR_BAD_ARG, "swe_ens_tune: bad argument");
    for (int q = 0; q < c->n; ++q)
        if (!c->uploaded[q]) return efail(c, SWE_ERR_BAD_ARG, "swe_ens_tune: instance %d not uploaded", q);
    ECK(cudaSetDevice(c->base.device));
    ECK(cudaMemsetAsync(c->d_flags, 0, sizeof(int), c->stream));
    // Snapshot U^n, speed slots, times and the step parity; every candidate starts there.
    const size_t fb = c->pool_elems * c->elem;
    if (!c->snap) ECK(cudaMalloc(&c->snap, 3 * fb + 4 * c->n * sizeof(double)));
    char *sp = static_cast<char *>(c->snap);
    for (int f = 0; f < 3; ++f)
        ECK(cudaMemcpyAsync(sp + f * fb, c->Un[f], fb, cudaMemcpyDeviceToDevice, c->stream));
    ECK(cudaMemcpyAsync(sp + 3 * fb, c->d_speed, 2 * c->n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    ECK(cudaMemcpyAsync(sp + 3 * fb + 2 * c->n * sizeof(double), c->d_t, c->n * sizeof(double),
                        cudaMemcpyDeviceToDevice, c->stream));
    const long long steps0 = c->steps_done;
    auto restore = [&]() -> int {
        for (int f = 0; f < 3; ++f)
            ECK(cudaMemcpyAsync(c->Un[f], sp + f * fb, fb, cudaMemcpyDeviceToDevice, c->stream));
        ECK(cudaMemcpyAsync(c->d_speed, sp + 3 * fb, 2 * c->n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        ECK(cudaMemcpyAsync(c->d_t, sp + 3 * fb + 2 * c->n * sizeof(double), c->n * sizeof(double),
                            cudaMemcpyDeviceToDevice, c->stream));
        c->steps_done = steps0;
        return SWE_OK;
    };
    const int shapes64[] = {SHAPE_STRIP, SHAPE_8x32, SHAPE_8x16, SHAPE_4x64};
    const int shapes32[] = {SHAPE_COLS, SHAPE_8x32, SHAPE_16x32, SHAPE_8x64};
    const int *shapes = c->f32 ? shapes32 : shapes64;
    const int n_shapes = 4;
    // 0: one CTA per tile; 1 / 2: a persistent grid of every resident CTA / half of them
    const int grids[] = {0, 1, 2};
    double best = 1e300;
    int best_shape = c->shape, best_grid = c->grid;
    for (int si = 0; si < n_shapes; ++si) {
        for (int gm : grids) {
            int g = 0;
            if (gm > 0) {
                const int per_sm = resident_per_sm(c, shapes[si]);
                if (per_sm <= 0 || (gm == 2 && per_sm < 2)) continue;
                g = (gm == 1 ? per_sm : per_sm / 2) * c->num_sms;
            }
            int st = swe_ens_set_schedule(c, shapes[si], g);
            if (st) return st;
            st = run_steps(c, 1, 0.0);  // warm-up (also captures the graphs)
            if (st) return st;
            ECK(cudaEventRecord(c->ev0, c->stream));
            st = run_steps(c, steps, 0.0);
            if (st) return st;
            ECK(cudaEventRecord(c->ev1, c->stream));
            ECK(cudaEventSynchronize(c->ev1));
            float ms = 0.f;
            ECK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            if (ms < best) {
                best = ms;
                best_shape = shapes[si];
                best_grid = g;
            }
            st = restore();
            if (st) return st;
        }
    }
    int st = swe_ens_set_schedule(c, best_shape, best_grid);
    if (st) return st;
    int flags = 0;
    ECK(cudaMemcpyAsync(&flags, c->d_flags, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    ECK(cudaStreamSynchronize(c->stream));
    if (flags & FLAG_TIMEOUT)  // the timings after the failed wait mean nothing
        return efail(c, SWE_ERR_TIMEOUT, "swe_ens_tune: a tile's TMA copy did not complete");
    if (best_ms) *best_ms = best / steps;
    return SWE_OK;
} catch (...) {  // host allocation failures do not cross the C ABI
    return SWE_ERR_BAD_ARG;
}

}  // extern "C"
