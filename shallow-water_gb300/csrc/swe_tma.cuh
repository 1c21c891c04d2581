// Tensor-memory-accelerator (TMA) tile loads for the stage kernels (sm_90+ PTX:
// cp.async.bulk.tensor with an mbarrier completing on transaction bytes).
//
// A CTA initialises its barrier once (mbar_init at kernel start) and tracks the phase
// parity in a register, flipping it after every completed tile, so a barrier is never
// re-initialised.  For each tile one elected thread arms the barrier with the expected
// byte count and issues the 2-D copies; every thread then waits on the phase.
//
// Every wait is bounded in time (kWaitNs of the GPU's global nanosecond timer), and
// the bound holds per launch, not per tile:
//  - a CTA whose wait gives up sets FLAG_TIMEOUT in the launch's flag word, waits
//    (again bounded) for its own copies to land, so that none is left writing into
//    shared memory that a later CTA reuses, and then returns from the kernel;
//  - every CTA reads the flag word at the start of each tile, folded into a block
//    barrier it already has, and returns at once when FLAG_TIMEOUT is set.
// A launch whose copies never land therefore ends about two deadlines after its first
// resident CTAs start waiting; the CTAs after them return without issuing a copy.
#pragma once

#include <cuda.h>
#include <cstdint>

#include "swe_common.cuh"

namespace swe {
namespace tma {

// Deadline of one wait.  A tile's copies land within microseconds; 50 ms leaves room for
// time-slicing with another context without a false timeout.
constexpr unsigned long long kWaitNs = 50ull * 1000ull * 1000ull;

// The GPU's global timer, in nanoseconds.
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
    // make the initialised barrier visible to the async (TMA) proxy
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait for phase `parity` to complete; false if it has not after deadline_ns.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          unsigned long long deadline_ns = kWaitNs) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        for (int k = 0; k < 32; ++k)
            if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > deadline_ns) return false;
    }
}

// Orders this thread's earlier generic-proxy shared-memory accesses, and those of the
// block ordered before them by a barrier, before its following TMA writes (the async
// proxy): issued by the thread that starts the copies when the buffers are being reused.
__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 2-D tile (x = innermost coordinate, y = row) of `map` into shared memory at dst
// (128-byte aligned); completes `bytes` on bar.  x times the element size must be a
// multiple of 16 bytes.
__device__ __forceinline__ void load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                        uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// The four staged fields of a stage source (eta or h, hu, hv, B).
struct TileMaps {
    const CUtensorMap *e, *u, *v, *b;
};

// A CTA's transaction barrier (initialised once, at kernel start) and the parity of
// the phase its next tile completes.
struct Pipe {
    uint64_t *bar;
    uint32_t phase;
};

// True when FLAG_TIMEOUT is set in the flag word: a wait of this launch, or of an
// earlier launch of the same call, gave up.  Read by one thread, which shares the
// answer through a block barrier so that the whole CTA returns together.
__device__ __forceinline__ bool timeout_set(const int *flags) {
    return (*reinterpret_cast<const volatile int *>(flags) & FLAG_TIMEOUT) != 0;
}

// Stages one tile: thread 0 arms the barrier for `bytes` and runs issue() (the copies),
// then every thread waits for the pipe's phase.  On success the phase flips and true is
// returned.  When the wait gives up, FLAG_TIMEOUT is set, thread 0 waits once more
// (bounded) for this CTA's copies to land, and false is returned to every thread: the
// caller then returns from the kernel without touching the barrier or the buffers
// again.  Called by every thread of the block; the barrier must have been initialised
// and made visible by a block barrier before.
template <class Issue>
__device__ __forceinline__ bool stage_in(Pipe &pp, int *flags, uint32_t bytes, Issue &&issue,
                                         unsigned long long deadline_ns = kWaitNs) {
    if (threadIdx.x == 0) {
        fence_proxy_async();  // earlier generic reads of the buffers before the copies
        mbar_arrive_expect_tx(pp.bar, bytes);
        issue();
    }
    const bool late = !mbar_wait(pp.bar, pp.phase, deadline_ns);
    if (__syncthreads_or(late)) {
        if (threadIdx.x == 0) {
            atomicOr(flags, FLAG_TIMEOUT);
            mbar_wait(pp.bar, pp.phase, deadline_ns);
        }
        __syncthreads();
        return false;
    }
    pp.phase ^= 1u;
    return true;
}

}  // namespace tma

// Host side: tensor maps of one stage source, passed to kernels by value.
struct StageMaps {
    CUtensorMap e, u, v, b;
};

// Encodes a 2-D tiled map over a ghosted (rows x cols) field of FP32 (elem 4) or FP64
// (elem 8) values with row pitch `pitch` elements and a (box_rows x box_cols) box
// (host; defined in swe_api.cu).
bool encode_tile_map(CUtensorMap *m, const void *base, int rows, int cols, long long pitch,
                     int box_rows, int box_cols, int elem);

}  // namespace swe
