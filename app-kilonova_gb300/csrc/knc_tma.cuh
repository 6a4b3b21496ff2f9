// knc_tma.cuh — tensor-memory-accelerator copies and mbarriers (inline PTX).
//
// The mixed update kernel stages each tile's primitives (with the 2-zone PLM
// halo) and the conserved boxes it reads with cp.async.bulk.tensor: one
// 3-D copy per array per tile, zero-filled outside the block, completing on an
// mbarrier. Tensor maps are encoded on the host per block (P as float
// [5][nr+4][nq], each state buffer as double [5][nr][nq]) and stored in a
// device array indexed by slot.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace knc {

struct TmaMaps {
    CUtensorMap P;      // float  {nq, nr + 4, 5}, box {TILE_Q + 8, TR + 4, 5}
    CUtensorMap U[2];   // double {nq, nr, 5},     box {TILE_Q, TR, 5}
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make initialised mbarriers visible to the asynchronous (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Order this thread's earlier shared-memory accesses (generic proxy) before
// later asynchronous-proxy copies into the same memory.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Wait for phase `parity` of an mbarrier, giving up after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, int limit) {
    for (int n = 0; n < limit; ++n)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 3-D tiled copy global -> shared; x must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace knc
