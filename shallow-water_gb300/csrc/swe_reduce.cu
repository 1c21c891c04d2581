// Compensated global totals of the state: mass = sum h dx dy, momentum = sum hu dx dy,
// sum hv dx dy over the interior (the quantity the reference's MassConservation check
// accumulates naively, tests/sanity_checks/mass_conservation.hpp:45-56).
//
// Each thread sums a fixed grid-stride set of cells in chunks of CHUNK cells: a plain
// FP64 sum per chunk, then an error-free TwoSum of the chunk into the thread's
// compensated (sum, compensation) pair - one FP64 add per value plus 6/CHUNK, where a
// TwoSum per value would make the reduction FP64-bound on GB300.  Warps and blocks
// combine pairs with TwoSum; a second one-block kernel adds the per-block pairs in
// block order.  The result is deterministic (fixed assignment and order); its error is
// that of the CHUNK-term chunk sums, about CHUNK roundings of a chunk, plus one
// rounding of the total.  Works on both forms (FP32 eta - B is exact in FP64).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <climits>
#include <mutex>

#include "../../include/swe_gb300.h"
#include "swe_common.cuh"
#include "swe_soft_f64.cuh"
#include "swe_launch.h"

namespace swe {
namespace {

struct Comp {
    double s, c;
};

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ void add(Comp &x, double v) {
    double s, e;
    two_sum(x.s, v, s, e);
    x.s = s;
    x.c += e;
}

__device__ __forceinline__ Comp merge(Comp x, Comp y) {
    Comp r;
    double e;
    two_sum(x.s, y.s, r.s, e);
    r.c = x.c + y.c + e;
    return r;
}

constexpr int BT = 256;
constexpr int CHUNK = 8;

template <bool F32>
__global__ void __launch_bounds__(BT) k_totals_partial(const void *h, const void *hu,
                                                       const void *hv, const void *B, int Nx,
                                                       int Ny, long long P, double *partial) {
    Comp acc[3] = {{0, 0}, {0, 0}, {0, 0}};
    double part[3] = {0.0, 0.0, 0.0};
    int in_chunk = 0;
    const long long n = (long long)Nx * Ny;
    for (long long t = blockIdx.x * (long long)BT + threadIdx.x; t < n;
         t += (long long)gridDim.x * BT) {
        const int i = (int)(t / Ny), j = (int)(t - (t / Ny) * Ny);
        const long long k = (long long)(i + NG) * P + (j + NG);
        double v0, v1, v2;
        if (F32) {
            v0 = (double)static_cast<const float *>(h)[k] - (double)static_cast<const float *>(B)[k];
            v1 = static_cast<const float *>(hu)[k];
            v2 = static_cast<const float *>(hv)[k];
        } else {
            v0 = static_cast<const double *>(h)[k];
            v1 = static_cast<const double *>(hu)[k];
            v2 = static_cast<const double *>(hv)[k];
        }
        part[0] += v0;
        part[1] += v1;
        part[2] += v2;
        if (++in_chunk == CHUNK) {
            for (int q = 0; q < 3; ++q) {
                add(acc[q], part[q]);
                part[q] = 0.0;
            }
            in_chunk = 0;
        }
    }
    for (int q = 0; q < 3; ++q) add(acc[q], part[q]);
    __shared__ Comp red[3][BT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = 0; q < 3; ++q) {
        Comp x = acc[q];
        for (int o = 16; o > 0; o >>= 1) {
            Comp y;
            y.s = __shfl_down_sync(0xffffffffu, x.s, o);
            y.c = __shfl_down_sync(0xffffffffu, x.c, o);
            x = merge(x, y);
        }
        if (lane == 0) red[q][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        Comp x = red[threadIdx.x][0];
        for (int w = 1; w < BT / 32; ++w) x = merge(x, red[threadIdx.x][w]);
        partial[(blockIdx.x * 3 + threadIdx.x) * 2 + 0] = x.s;
        partial[(blockIdx.x * 3 + threadIdx.x) * 2 + 1] = x.c;
    }
}

__global__ void k_totals_final(const double *partial, int blocks, double scale, double *out) {
    if (threadIdx.x >= 3) return;
    Comp x{0, 0};
    for (int b = 0; b < blocks; ++b)
        x = merge(x, Comp{partial[(b * 3 + threadIdx.x) * 2], partial[(b * 3 + threadIdx.x) * 2 + 1]});
    out[threadIdx.x] = (x.s + x.c) * scale;
}

// Sanity reductions of one state in one pass (the reference's MassConservation,
// Positivity and Debug checks, tests/sanity_checks/*.hpp, computed on the device):
// compensated sums of h and of the energy density
//   e = (hu^2 + hv^2) / (2 h) (h > 1e-8, else 0) + g h^2 / 2 + g h B,
// the minimum h (NaN ignored, as `h < h_min` never selects it) and the smallest
// row-major interior index i * Ny + j with h < 0 (the cell Positivity reports first).
// Per block: mass pair, energy pair, h_min, first index (as a double's bits).
template <bool F32>
__global__ void __launch_bounds__(BT) k_sanity_partial(const void *h, const void *hu,
                                                       const void *hv, const void *B, int Nx,
                                                       int Ny, long long P, double g,
                                                       double *partial) {
    Comp mass{0, 0}, energy{0, 0};
    double pm = 0.0, pe = 0.0;  // chunk sums
    int in_chunk = 0;
    double hmin = __longlong_as_double(0x7FF0000000000000LL);  // +inf
    long long first = LLONG_MAX;
    const double half_g = 0.5 * g;
    const long long n = (long long)Nx * Ny;
    for (long long t = blockIdx.x * (long long)BT + threadIdx.x; t < n;
         t += (long long)gridDim.x * BT) {
        const int i = (int)(t / Ny), j = (int)(t - (t / Ny) * Ny);
        const long long k = (long long)(i + NG) * P + (j + NG);
        double hh, u, v, b;
        if (F32) {
            b = static_cast<const float *>(B)[k];
            hh = (double)static_cast<const float *>(h)[k] - b;
            u = static_cast<const float *>(hu)[k];
            v = static_cast<const float *>(hv)[k];
        } else {
            hh = static_cast<const double *>(h)[k];
            u = static_cast<const double *>(hu)[k];
            v = static_cast<const double *>(hv)[k];
            b = static_cast<const double *>(B)[k];
        }
        // the division and the comparisons run on the integer pipe (correctly rounded /
        // exact), the rest is one FP64 chunk sum per quantity
        const double kin = x64::lt(1.0e-8, hh) ? sf::div_rn(x64::halve(u * u + v * v), hh) : 0.0;
        pm += hh;
        pe += kin + half_g * hh * hh + g * hh * b;
        if (++in_chunk == CHUNK) {
            add(mass, pm);
            add(energy, pe);
            pm = pe = 0.0;
            in_chunk = 0;
        }
        if (x64::lt(hh, hmin)) hmin = hh;  // NaN never selected, as `h < h_min`
        if (x64::lt(hh, 0.0) && t < first) first = t;
    }
    add(mass, pm);
    add(energy, pe);
    __shared__ Comp red[2][BT / 32];
    __shared__ double rmin[BT / 32];
    __shared__ long long rfirst[BT / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        Comp y;
        y.s = __shfl_down_sync(0xffffffffu, mass.s, o);
        y.c = __shfl_down_sync(0xffffffffu, mass.c, o);
        mass = merge(mass, y);
        y.s = __shfl_down_sync(0xffffffffu, energy.s, o);
        y.c = __shfl_down_sync(0xffffffffu, energy.c, o);
        energy = merge(energy, y);
        const double hm2 = __shfl_down_sync(0xffffffffu, hmin, o);
        if (x64::lt(hm2, hmin)) hmin = hm2;
        const long long f2 = __shfl_down_sync(0xffffffffu, first, o);
        first = f2 < first ? f2 : first;
    }
    if (lane == 0) {
        red[0][warp] = mass;
        red[1][warp] = energy;
        rmin[warp] = hmin;
        rfirst[warp] = first;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        Comp m = red[0][0], e = red[1][0];
        double hm = rmin[0];
        long long f = rfirst[0];
        for (int w = 1; w < BT / 32; ++w) {
            m = merge(m, red[0][w]);
            e = merge(e, red[1][w]);
            if (x64::lt(rmin[w], hm)) hm = rmin[w];
            f = rfirst[w] < f ? rfirst[w] : f;
        }
        double *o = partial + (size_t)blockIdx.x * 6;
        o[0] = m.s;
        o[1] = m.c;
        o[2] = e.s;
        o[3] = e.c;
        o[4] = hm;
        o[5] = __longlong_as_double(f);
    }
}

// out: mass * dxdy, energy * dxdy, h_min, first index (-1: none; as a double's bits).
__global__ void k_sanity_final(const double *partial, int blocks, double dxdy, double *out) {
    if (threadIdx.x != 0) return;
    Comp m{0, 0}, e{0, 0};
    double hm = __longlong_as_double(0x7FF0000000000000LL);
    long long f = LLONG_MAX;
    for (int b = 0; b < blocks; ++b) {
        const double *o = partial + (size_t)b * 6;
        m = merge(m, Comp{o[0], o[1]});
        e = merge(e, Comp{o[2], o[3]});
        if (x64::lt(o[4], hm)) hm = o[4];
        const long long fb = __double_as_longlong(o[5]);
        f = fb < f ? fb : f;
    }
    out[0] = (m.s + m.c) * dxdy;
    out[1] = (e.s + e.c) * dxdy;
    out[2] = hm;
    out[3] = __longlong_as_double(f == LLONG_MAX ? -1LL : f);
}

}  // namespace

cudaError_t launch_sanity(const void *h, const void *hu, const void *hv, const void *B, bool f32,
                          int Nx, int Ny, long long pitch, double g, double dxdy,
                          double *partial, double *out, int num_sms, cudaStream_t s) {
    const int blocks = num_sms * 4;
    if (f32)
        k_sanity_partial<true><<<blocks, BT, 0, s>>>(h, hu, hv, B, Nx, Ny, pitch, g, partial);
    else
        k_sanity_partial<false><<<blocks, BT, 0, s>>>(h, hu, hv, B, Nx, Ny, pitch, g, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_sanity_final<<<1, 32, 0, s>>>(partial, blocks, dxdy, out);
    return cudaGetLastError();
}

int totals_blocks(int num_sms) { return num_sms * 4; }

cudaError_t launch_totals_blocks(const void *h, const void *hu, const void *hv, const void *B,
                                 bool f32, int Nx, int Ny, long long pitch, double dxdy,
                                 double *partial, double *out, int blocks, cudaStream_t s) {
    if (f32)
        k_totals_partial<true><<<blocks, BT, 0, s>>>(h, hu, hv, B, Nx, Ny, pitch, partial);
    else
        k_totals_partial<false><<<blocks, BT, 0, s>>>(h, hu, hv, B, Nx, Ny, pitch, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_totals_final<<<1, 32, 0, s>>>(partial, blocks, dxdy, out);
    return cudaGetLastError();
}

cudaError_t launch_totals(const void *h, const void *hu, const void *hv, const void *B, bool f32,
                          int Nx, int Ny, long long pitch, double dxdy, double *partial,
                          double *out, int num_sms, cudaStream_t s) {
    const int blocks = totals_blocks(num_sms);
    if (f32)
        k_totals_partial<true><<<blocks, BT, 0, s>>>(h, hu, hv, B, Nx, Ny, pitch, partial);
    else
        k_totals_partial<false><<<blocks, BT, 0, s>>>(h, hu, hv, B, Nx, Ny, pitch, partial);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_totals_final<<<1, 32, 0, s>>>(partial, blocks, dxdy, out);
    return cudaGetLastError();
}

}  // namespace swe

// ---- Allocation-free variant ------------------------------------------------------------
//
// Scratch for swe_totals_noalloc: the per-block compensated partial sums (6 doubles per
// block) and nothing else.  A file-scope device array, so the entry point never calls
// cudaMalloc; every GPU that loads this library holds it (48 KiB) until the process exits.
// In host code the name is only a stand-in for the device copy: its device address comes
// from cudaGetSymbolAddress, taken once per device with that device current.
static __device__ __align__(256) double g_totals_noalloc_scratch[6 * SWE_TOTALS_NOALLOC_MAX_BLOCKS];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
double *g_noalloc_ptr[kMaxDevices] = {};
CUcontext g_noalloc_ctx[kMaxDevices] = {};  // the context each address was looked up in

// The context current on the calling thread (the driver's cuCtxGetCurrent, reached
// through the runtime's entry-point query so that nothing links libcuda directly).
bool current_context(CUcontext *ctx) {
    static PFN_cuCtxGetCurrent_v4000 get = nullptr;
    if (!get) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || !fn) {
            cudaGetLastError();
            return false;
        }
        get = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(fn);
    }
    return get(ctx) == CUDA_SUCCESS;
}

// Address of the scratch array in the current context of `device`: looked up on the first
// call per device, and again whenever the current context is not the one it was looked
// up in (the array has one copy per context that loaded the library's module).
int noalloc_scratch(int device, double **out) {
    if (device < 0 || device >= kMaxDevices) return SWE_ERR_BAD_ARG;
    // NULL on a thread the runtime has not used yet; the look-up below makes the device's
    // primary context current there.
    CUcontext ctx = nullptr;
    if (!current_context(&ctx)) return SWE_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!ctx || !g_noalloc_ptr[device] || g_noalloc_ctx[device] != ctx) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_totals_noalloc_scratch);
        if (e != cudaSuccess || !ptr || !current_context(&ctx) || !ctx) {
            cudaGetLastError();
            return SWE_ERR_CUDA;
        }
        g_noalloc_ptr[device] = static_cast<double *>(ptr);
        g_noalloc_ctx[device] = ctx;
    }
    *out = g_noalloc_ptr[device];
    return SWE_OK;
}

}  // namespace

extern "C" int swe_totals_noalloc(const void *h, const void *hu, const void *hv, const void *B,
                                  int precision, int Nx, int Ny, long long pitch, double dxdy,
                                  int blocks, double *out, void *stream) {
    using namespace swe;
    const bool f32 = precision == SWE_PRECISION_FP32_MIXED;
    if (!h || !hu || !hv || !out || (f32 && !B)) return SWE_ERR_BAD_ARG;
    if (precision != SWE_PRECISION_FP64 && !f32) return SWE_ERR_BAD_ARG;
    if (Nx < 1 || Ny < 1 || pitch < (long long)Ny + 4 || blocks < 0) return SWE_ERR_BAD_ARG;
    int device = 0, sms = 0;
    if (cudaGetDevice(&device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        cudaGetLastError();
        return SWE_ERR_NO_DEVICE;
    }
    if (blocks == 0) blocks = std::min(totals_blocks(sms), SWE_TOTALS_NOALLOC_MAX_BLOCKS);
    if (blocks > SWE_TOTALS_NOALLOC_MAX_BLOCKS) return SWE_ERR_BAD_ARG;  // beyond the scratch
    double *scratch = nullptr;
    const int st = noalloc_scratch(device, &scratch);
    if (st != SWE_OK) return st;
    const cudaError_t e =
        launch_totals_blocks(h, hu, hv, B, f32, Nx, Ny, pitch, dxdy, scratch, out, blocks,
                             static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? SWE_OK : SWE_ERR_CUDA;
}

