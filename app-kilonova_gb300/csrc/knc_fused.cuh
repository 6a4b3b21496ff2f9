// knc_fused.cuh — one RK stage as one persistent, cooperative launch.
//
// The separate form of a stage is four launches (ghost rows, recovery, halo
// remaps, update). The fused form runs the same per-zone and per-tile device
// functions inside one kernel whose CTAs are all resident (cooperative
// launch), with a grid-wide barrier where one phase consumes the previous
// one's output:
//   A  ghost rows of both mesh ends, then the primitive recovery of every zone
//      in chunks of NT consecutive zones of one block (each zone pushes its
//      edge rows into same-shaped neighbours' halos, as in the separate form);
//   -- barrier --
//   B  halo remaps across polar-resolution changes (uneven blocks only);
//   -- barrier (only with remaps) --
//   C  the flux / source / update / RK-average tiles (or warp strips).
// Work in each phase is a grid-stride loop over a device list, so one launch
// shape covers every block set of a moving mesh. Because the phases call the
// very functions the separate kernels call, the two forms give bit-identical
// states.
//
// The barrier counts arrivals in DevStatus::bar_count (zeroed by the host with
// the rest of the status); launch n of a fold waits for bar_base + k x grid.
// A wait gives up after a bounded number of polls, sets bar_abort and lets
// the CTA continue without waiting at later barriers; the host then reports
// the stage as failed. Co-residency of all CTAs (cooperative launch with a
// grid no larger than the occupancy bound) means the limit is never reached
// in a correct launch.
#pragma once

#include "knc_halo.cuh"
#include "knc_internal.h"
#include "knc_mlp.cuh"
#include "knc_stage.cuh"

namespace knc {

__device__ __forceinline__ void grid_barrier(DevStatus* st, unsigned long long target, int limit) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&st->bar_count, 1ull);
        if (*(volatile int32_t*)&st->bar_abort == 0) {
            int n = 0;
            while (*(volatile unsigned long long*)&st->bar_count < target) {
                if (++n > limit) {
                    atomicExch(&st->bar_abort, 1);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// A barrier the CTA passes without waiting: it only counts its arrival, so the
// barriers after it keep their targets. For a phase with no work (every CTA
// knows it from the same device value), the next phase may start at once.
__device__ __forceinline__ void grid_arrive(DevStatus* st) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&st->bar_count, 1ull);
    }
}

// Per-thread recovery statistics (summed into DevStatus at the end). 32-bit
// per thread (a thread recovers far fewer than 2^28 zones of at most 16
// iterations each), widened for the warp sums.
struct C2pStats {
    unsigned zones = 0, it64 = 0, it32 = 0, fbs = 0;
    double dtz = 1.7976931348623157e308;
};

// Shared memory of the fused kernel: the update tile's arrays, then (with the
// learned guess) the MLP weights and one activation tile per warp.
template <bool MLP>
constexpr size_t fused_strip_smem_bytes() {
    return MLP ? sizeof(MlpWeights) + STRIP_WARPS * MLP_ACT_ELEMS * sizeof(__nv_bfloat16) : 0;
}

template <class R, int TR, bool MLP>
constexpr size_t fused_smem_bytes() {
    return ((StageSmem<R, TR>::bytes + 15) / 16) * 16 +
           (MLP ? sizeof(MlpWeights) + (update_threads<TR>() / 32) * MLP_ACT_ELEMS * sizeof(__nv_bfloat16) : 0);
}

// C2P provides `static constexpr bool mlp` and
//   __device__ static void zone(const StageArgs&, int slot, const DevBlock&, int i, int j, bool active,
//                               MlpWeights&, __nv_bfloat16* act, C2pStats&)
// which every thread of a warp calls together (the learned guess is a
// warp-wide tensor-core inference).
//
// NT threads per CTA (the tile form needs update_threads<TR>()); STRIPS_ONLY:
// the update phase runs warp strips only and the CTA keeps no tile arrays,
// so small CTAs (4 warps) fit many to an SM.
template <class R, bool MIXED, int TR, class C2P, int NT = update_threads<TR>(), bool STRIPS_ONLY = false>
__device__ __forceinline__ void stage_fused_body(const StageArgs& a, const GhostArgs& g, const FusedArgs& f) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int run_update;
    constexpr size_t W_OFF = STRIPS_ONLY ? 0 : ((StageSmem<R, TR>::bytes + 15) / 16) * 16;
    MlpWeights& W = *reinterpret_cast<MlpWeights*>(smem_raw + W_OFF);
    __nv_bfloat16* act = reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<unsigned char*>(&W) + sizeof(MlpWeights)) +
                         (threadIdx.x >> 5) * MLP_ACT_ELEMS;
    if (C2P::mlp) {
        mlp_load(W, a.mlp);
        __syncthreads();
    }
    // a failure in an earlier stage stops the step (the separate kernels'
    // entry checks); every CTA still takes part in the barriers
    const unsigned long long ek = *(volatile unsigned long long*)&a.status->err_key;
    const bool run = !(ek != NO_ERROR && (uint32_t)(ek >> 48) < (uint32_t)a.stage);
    C2pStats st;

    // ---- A: ghost rows, then recovery chunks {slot, z0, nz, 0}
    const int ng0 = (2 * g.nq[0] + NT - 1) / NT, ng1 = (2 * g.nq[1] + NT - 1) / NT;
    const int nA = ng0 + ng1 + f.nchunks;
    if (run) {
        for (int item = blockIdx.x; item < nA; item += gridDim.x) {
            if (item < ng0) {
                ghost_zone(g, 0, item * NT + threadIdx.x);
            } else if (item < ng0 + ng1) {
                ghost_zone(g, 1, (item - ng0) * NT + threadIdx.x);
            } else {
                const int4 ch = f.chunks[item - ng0 - ng1];
                const DevBlock& B = a.blocks[ch.x];
                const bool active = (int)threadIdx.x < ch.z;
                const int z = ch.y + (active ? (int)threadIdx.x : 0);
                const int i = z / B.nq, j = z - i * B.nq;
                C2P::zone(a, ch.x, B, i, j, active, W, act, st);
            }
        }
    }
    if (a.compute_dt) {
        // the adaptive time step must be complete before phase C reads it
        double dtz = st.dtz;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dtz = fmin(dtz, __shfl_down_sync(0xffffffffu, dtz, o));
        if ((threadIdx.x & 31) == 0) atomicMin(&a.status->dt_bits, (unsigned long long)__double_as_longlong(dtz));
    }
    grid_barrier(a.status, f.bar_base + gridDim.x, f.spin_limit);

    // ---- B: remaps
    if (f.nremap > 0) {
        if (run) {
            const int per = 2 * f.max_nq;
            const int total = f.nremap * per;
            for (int k = blockIdx.x * NT + threadIdx.x; k < total; k += gridDim.x * NT) {
                const int item = k / per;
                remap_zone<R, typename C2P::RemapRec>(a, f.remap[item], k - item * per);
            }
        }
        grid_barrier(a.status, f.bar_base + 2ull * gridDim.x, f.spin_limit);
    }

    // ---- C: update tiles (skipped after any failure, like the separate kernel)
    if (threadIdx.x == 0)
        run_update = *(volatile unsigned long long*)&a.status->err_key == NO_ERROR &&
                     *(volatile int32_t*)&a.status->bar_abort == 0;
    __syncthreads();
    if (run_update) {
        if (STRIPS_ONLY || a.strips) {
            // warp strips: every warp of the grid takes strips on its own
            constexpr int WPC = NT / 32;
            stage_strips<R, MIXED>(a, blockIdx.x * WPC + (int)(threadIdx.x >> 5), gridDim.x * WPC);
        } else if constexpr (!STRIPS_ONLY) {
            // (the next stage's producers run in the next launch: clear its list)
            if constexpr (MIXED) clear_next_hp(a);
            for (int tile = blockIdx.x; tile < a.nutiles; tile += gridDim.x) {
                update_tile<R, MIXED, TR>(a, a.utiles[tile], smem_raw);
                __syncthreads();
            }
        }
        if constexpr (MIXED) {
            if (!(STRIPS_ONLY || a.strips)) drain_hp(a);   // (the strips' form drains its own list)
        }
    }
    warp_reduce_stats(a.status, st.zones, st.it64, st.it32, st.fbs, st.dtz, false);
}

}  // namespace knc
