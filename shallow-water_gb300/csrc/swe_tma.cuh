// Tensor-memory-accelerator (TMA) tile loads for the stage kernels (sm_90+ PTX:
// cp.async.bulk.tensor with an mbarrier completing on transaction bytes).
//
// One elected thread arms the barrier with the expected byte count and issues the 2-D
// tile copies; every thread waits on the barrier's phase.  The wait is bounded: after
// kSpinLimit polls it gives up, the caller records FLAG_TIMEOUT and skips the tile, so
// a copy that never lands cannot hang the GPU.
#pragma once

#include <cuda.h>
#include <cstdint>

namespace swe {
namespace tma {

// Each failed try_wait may itself suspend for a hardware-defined time (about a
// microsecond), so 2^20 polls bound a copy that never lands near a second per tile,
// far above the microseconds a copy takes.
constexpr uint32_t kSpinLimit = 1u << 20;

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

// Bounded wait for phase `parity`; false if it did not complete within kSpinLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t it = 0; it < kSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
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
