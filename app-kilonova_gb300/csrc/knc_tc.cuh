// knc_tc.cuh — fifth-generation tensor-core primitives (tcgen05, inline PTX).
//
// Used by the training kernel of the learned c2p guess, the one dense
// contraction of this code. One thread of the CTA issues tcgen05.mma with both
// operands in shared memory and the FP32 accumulator in tensor memory (TMEM);
// completion is signalled on an mbarrier by tcgen05.commit; every warp then
// reads its 32 TMEM lanes (accumulator rows) back with tcgen05.ld.
//
// Operand layout: no swizzle, K-major "core matrices" of 8 rows x 16 bytes
// (8 bf16 along K), each core matrix 128 contiguous bytes with its rows 16
// bytes apart. The shared-memory descriptor gives the byte distance between
// core matrices adjacent along K (leading byte offset) and between groups of 8
// rows along M or N (stride byte offset).
#pragma once

#include <stdint.h>

namespace knc {

// Shared-memory matrix descriptor (sm_100 family): start address, leading and
// stride byte offsets in 16-byte units, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, bf16 A and B, both
// K-major, dense, M x N.
constexpr uint32_t tc_idesc_bf16(int m, int n) {
    return (1u << 4)                      // D format F32
           | (1u << 7)                    // A format BF16
           | (1u << 10)                   // B format BF16
           | ((uint32_t)(n >> 3) << 17)   // N / 8
           | ((uint32_t)(m >> 4) << 24);  // M / 16
}

// D[tmem] (+)= A[smem] . B[smem]^T, K = 16; issued by one thread.
__device__ __forceinline__ void tc_mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                            uint32_t accumulate) {
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on an mbarrier once every tcgen05.mma this thread issued so far has
// completed.
__device__ __forceinline__ void tc_commit(uint32_t bar_saddr) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar_saddr)
                 : "memory");
}

// TMEM allocation by one whole warp; the address is written to shared memory.
__device__ __forceinline__ void tc_alloc(uint32_t slot_saddr, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_saddr), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes
// 32 w .. 32 w + 31; lane field in bits 31:16 of the address).
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 64 FP32 columns starting at column `col` of this warp's lanes.
__device__ __forceinline__ void tc_ld64(uint32_t tmem, int col, float (&v)[64]) {
    const uint32_t base = tmem + ((uint32_t)(threadIdx.x & ~31u) << 16) + (uint32_t)col;
    float t[16];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        tc_ld16(base + 16u * c, t);
        tc_wait_ld();
#pragma unroll
        for (int k = 0; k < 16; ++k) v[16 * c + k] = t[k];
    }
}

}  // namespace knc
