// Device self-tests.
//  - The integer-pipe binary64 division, square root, multiplication and addition
//    (swe_soft_f64.cuh) against the GPU's own IEEE round-to-nearest operations, on
//    hashed operands: raw bit patterns (every class), physical-scale values, near-equal
//    pairs and exact quotients with their neighbours.
//  - The give-up path of the stage kernels' bounded TMA waits (swe_tma.cuh), on a
//    barrier that is armed for bytes no copy delivers.
#include <cuda_runtime.h>

#include "../../include/swe_gb300.h"
#include "swe_soft_f64.cuh"
#include "swe_tma.cuh"

namespace swe {
namespace {

using sf::u64;

__device__ __forceinline__ u64 mix64(u64 z) {  // SplitMix64 finaliser
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ bool same(double got, double want) {
    if (want != want) return got != got;
    return __double_as_longlong(got) == __double_as_longlong(want);
}

// A double with a random significand and sign and a biased exponent 1023 + [lo, lo + 63].
__device__ __forceinline__ double scaled(u64 r, int lo) {
    const u64 e = (u64)(1023 + lo + (int)(r >> 58));
    return __longlong_as_double((long long)((r & (sf::MANT_BITS | sf::SIGN_BIT)) | (e << 52)));
}

__global__ void k_selftest_soft(long long n, u64 seed, unsigned long long *bad) {
    unsigned long long local = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const u64 r1 = mix64(seed + 2 * (u64)i), r2 = mix64(seed + 2 * (u64)i + 1);
        double x, y;
        switch (i & 3) {
            case 0:  // raw patterns: zeros, subnormals, infinities, NaN, extremes
                x = __longlong_as_double((long long)r1);
                y = __longlong_as_double((long long)r2);
                break;
            case 1:  // physical scales
                x = scaled(r1, -32);
                y = scaled(r2, -32);
                break;
            case 2:  // near-equal operands
                x = scaled(r1, -20);
                y = __longlong_as_double(__double_as_longlong(x) ^ (long long)(r2 & 0xFFF));
                break;
            default: {  // exact quotient q = x / y with short significands, then a neighbour
                const double q = (double)(r1 >> 38) * 0x1p-20;
                y = (double)((r2 >> 37) | 1) * 0x1p-13;
                x = __dmul_rn(q, y);
                if (r2 & 1) x = __longlong_as_double(__double_as_longlong(x) + ((r2 & 2) ? 1 : -1));
            }
        }
        local += !same(sf::div_rn(x, y), __ddiv_rn(x, y));
        local += !same(sf::div_rn(1.0, y), __ddiv_rn(1.0, y));
        local += !same(sf::mul_rn(x, y), __dmul_rn(x, y));
        local += !same(sf::add_rn(x, y), __dadd_rn(x, y));
        local += !same(sf::sub_rn(x, y), __dsub_rn(x, y));
        const double ax = fabs(x);
        local += !same(sf::sqrt_rn(ax), __dsqrt_rn(ax));
        local += !same(sf::sqrt_rn(x), __dsqrt_rn(x));
    }
    if (local) atomicAdd(bad, local);
}

// Each block does what a stage tile does before its stencil: read the flag word under a
// block barrier and return if a wait already gave up, else arm its barrier and wait
// through tma::stage_in.  The barrier expects `bytes` that nothing delivers, so the wait
// gives up after deadline_ns, sets FLAG_TIMEOUT, waits once more for (absent) copies and
// returns; blocks that start after that return at the flag check.
__global__ void k_selftest_wait_timeout(int *flags, unsigned long long deadline_ns,
                                        unsigned long long *waited) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ int s_abort;
    if (threadIdx.x == 0) {
        tma::mbar_init(&bar, 1);
        s_abort = tma::timeout_set(flags);
    }
    __syncthreads();
    if (s_abort) return;
    if (threadIdx.x == 0) atomicAdd(waited, 1ull);
    tma::Pipe pipe{&bar, 0u};
    tma::stage_in(pipe, flags, 1024u, [] {}, deadline_ns);
}

}  // namespace
}  // namespace swe

extern "C" int swe_selftest_soft_f64(long long n, unsigned long long seed, long long *mismatches) {
    if (n < 0 || !mismatches) return SWE_ERR_BAD_ARG;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) return SWE_ERR_NO_DEVICE;
    unsigned long long *d_bad = nullptr, h_bad = 0;
    if (cudaMalloc(&d_bad, sizeof *d_bad) != cudaSuccess) return SWE_ERR_CUDA;
    int st = SWE_OK;
    if (cudaMemset(d_bad, 0, sizeof *d_bad) != cudaSuccess) st = SWE_ERR_CUDA;
    if (st == SWE_OK) {
        swe::k_selftest_soft<<<1216, 256>>>(n, seed, d_bad);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(&h_bad, d_bad, sizeof h_bad, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = SWE_ERR_CUDA;
    }
    cudaFree(d_bad);
    *mismatches = (long long)h_bad;
    return st;
}

extern "C" int swe_selftest_wait_timeout(int ctas, double deadline_ms, long long *waited_ctas,
                                         double *elapsed_ms) {
    if (ctas < 1 || ctas > (1 << 20) || !(deadline_ms > 0.0) || deadline_ms > 1000.0 ||
        !waited_ctas || !elapsed_ms)
        return SWE_ERR_BAD_ARG;
    int dev_count = 0;
    if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) return SWE_ERR_NO_DEVICE;
    struct Words {
        unsigned long long waited;
        int flags;
    } *d = nullptr, h{};
    if (cudaMalloc(&d, sizeof *d) != cudaSuccess) return SWE_ERR_CUDA;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int st = SWE_OK;
    if (cudaMemset(d, 0, sizeof *d) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess)
        st = SWE_ERR_CUDA;
    float ms = 0.f;
    if (st == SWE_OK) {
        const unsigned long long ns = (unsigned long long)(deadline_ms * 1.0e6);
        cudaEventRecord(e0);
        swe::k_selftest_wait_timeout<<<ctas, 64>>>(&d->flags, ns, &d->waited);
        cudaEventRecord(e1);
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess ||
            cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = SWE_ERR_CUDA;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(d);
    if (st != SWE_OK) return st;
    *waited_ctas = (long long)h.waited;
    *elapsed_ms = ms;
    return (h.flags & swe::FLAG_TIMEOUT) ? SWE_ERR_TIMEOUT : SWE_OK;
}
