// knc_mixed.cu — the mixed-precision stage.
//
// Same method as the FP64 stage (src/scheme.rs:16-173), with the precision
// moved per operation:
//   FP32  reconstruction, Riemann fluxes, geometric sources, geometry factors
//         (update_kernel<float, true>), primitive storage;
//   FP64  the conserved state and its RK accumulation, time and excision
//         radius (host), and the cons -> prim recovery of zones whose Lorentz
//         factor exceeds `w_split` — converged to the reference's residual
//         |f| < 1e-12 (D + tau) — and the faces whose stencil reaches such a
//         zone, with the update of the zones they bound (zone_hp,
//         knc_stage.cuh).
// Zones below `w_split` recover in FP32. Every zone first runs the Newton
// iteration in FP32; an FP64 recovery then starts from that root and usually
// needs one or two FP64 iterations instead of the 3-6 the plain guess takes.
//
// The recovery is scale-invariant (U -> k U gives p -> k p), so it runs on the
// volume-integrated state and divides rho and p by dV afterwards: no FP64
// divisions by the cell volume.
#include <map>
#include <mutex>

#include "knc_bits.cuh"
#include "knc_fused.cuh"
#include "knc_halo.cuh"
#include "knc_internal.h"
#include "knc_mlp.cuh"
#include "knc_physics.cuh"
#include "knc_stage.cuh"
#include "knc_tma.cuh"

namespace knc {

// Programmatic dependent launch: a kernel launched this way may be scheduled
// while its predecessor on the stream is still running (after every CTA of
// the predecessor has started and called launch_dependents); it blocks in
// dependency_wait() until the predecessor has completed and its writes are
// visible. The launch latency and the predecessor's tail then overlap.
__device__ __forceinline__ void dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... Params, class... Args>
static cudaError_t launch_chained(void (*k)(Params...), int grid, int block, size_t smem, cudaStream_t s,
                                  Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

// The learned-guess inference out of line: warps run it only when one of
// their zones needs the FP64 recovery, so its register demand stays out of
// the common path.
static __device__ __noinline__ float mlp_guess_call(const MlpWeights& W, __nv_bfloat16* act, float x0, float x1,
                                                    float x2) {
    const float x[3] = {x0, x1, x2};
    return mlp_warp_infer(W, act, x);
}

constexpr int TMA_WAIT_LIMIT = 1 << 22;   // mbarrier polls before a copy counts as lost

// The FP64 recovery of one zone (volume-integrated state m, S_r, S_theta,
// tau; cell volume dV in the stage's length units) from the FP32 root p32 / m
// when the FP32 iteration converged (ok32), else from the plain guess; the
// reference's iteration from the plain guess is the fallback.
struct Fp64Recovery {
    float P[4];
    int kind;
    int it64;
    int fbs;
    int it32;
};

__device__ __forceinline__ Fp64Recovery recover_fp64(const StageArgs& a, double m, double s1, double s2, double tau,
                                                     float dV, bool ok32, float p32) {
    Fp64Recovery r = {{0.f, 0.f, 0.f, 0.f}, HYDRO_NONE, 0, 0, 0};
    const double ss = s1 * s1 + s2 * s2;
    const double tol = NEWTON_TOLERANCE * (m + tau);
    double p64 = 0.0, w64 = 1.0;
    const bool ok = newton_fast<double>(m, ss, tau, a.gm, ok32 ? (double)p32 * m : 0.0, tol, 0.0, NEWTON_ITER_MAX,
                                        p64, w64, r.it64);
    if (!ok) {
        // fallback: the reference's iteration from the plain guess
        r.fbs = 1;
        const double u[4] = {m, s1, s2, tau};
        double Pd[4] = {0.0, 0.0, 0.0, 0.0};
        double bad;
        int itf = 0;
        const int kf = srhd_c2p_newton(a.gm, u, 0.0, Pd, itf, bad);
        r.it64 += itf;
        if (kf == HYDRO_ROOT_FINDER_FAILED) {
            r.kind = kf;
        } else {
            // Pd is the (floored) primitive of the volume-integrated state
            const double inv_dv = a.lscale3_d / (double)dV;
            r.P[0] = (float)(Pd[0] * inv_dv);
            r.P[1] = (float)Pd[1];
            r.P[2] = (float)Pd[2];
            r.P[3] = (float)(Pd[3] * inv_dv);
        }
    } else {
        const double inv_dv = a.lscale3_d / (double)dV;
        const double inv_et = 1.0 / (tau + m + p64);
        const double rho = m / w64 * inv_dv;
        r.P[0] = (float)rho;
        r.P[1] = (float)(w64 * s1 * inv_et);
        r.P[2] = (float)(w64 * s2 * inv_et);
        r.P[3] = p64 < 0.0 ? (float)(PRESSURE_FLOOR * rho) : (float)(p64 * inv_dv);
    }
    return r;
}

// Out of line, for the recovery form that defers these zones: there it runs
// only if the deferral list were full, so it reads the zone's state again
// rather than keep the FP64 values live, and its registers stay out of the
// common path. run32: the FP32 iteration (per unit mass: ssn, taun, from
// guess) has not run yet.
static __device__ __noinline__ Fp64Recovery recover_fp64_call(const StageArgs& a, const DevBlock& B, int i, int j,
                                                              float dV, bool ok32, float p32, bool run32, float ssn,
                                                              float taun, float guess) {
    int it32 = 0;
    if (run32) {
        float w32 = 1.f;
        ok32 = newton_fast<float>(1.0f, ssn, taun, a.gm_f, guess, 2e-7f * taun, 1e-6f, 16, p32, w32, it32);
    }
    const int64_t n = (int64_t)B.nr * B.nq;
    const double* Ub = B.buf[a.sel_in] + (int64_t)i * B.nq + j;
    Fp64Recovery r = recover_fp64(a, Ub[0], Ub[n], Ub[2 * n], Ub[3 * n], dV, ok32, p32);
    r.it32 = it32;
    return r;
}

// A merged zone of a halo remap (volume integrals U over the finer
// neighbour's zones, their summed volume dv) recovered as the mixed stage
// recovers any zone: the FP32 iteration per unit mass, the FP64 recovery from
// its root above the Lorentz-factor split or where it did not converge.
struct MixedRemapRecovery {
    template <class R>
    __device__ static int recover(const StageArgs& a, const double (&U)[5], double dv, R (&v)[NFIELD]) {
        const double m = U[0], tau = U[3];
        if (is_negative(m)) return HYDRO_NEGATIVE_DENSITY;
        if (is_negative(tau)) return HYDRO_NEGATIVE_ENERGY_DENSITY;
        const int de = -a.lscale3;
        const float mf = d2f_rn_exp(m, de), tauf = d2f_rn_exp(tau, de);
        const float s1f = d2f_rn_exp(U[1], de), s2f = d2f_rn_exp(U[2], de);
        const float scalf = d2f_rn_exp(U[4], de);
        const float dV = d2f_rn_exp(dv, de);
        const float im = 1.0f / mf;
        const float s1n = s1f * im, s2n = s2f * im, taun = tauf * im;
        const float ssn = s1n * s1n + s2n * s2n;
        const float x1 = __fdividef(sqrtf(ssn), 1.0f + taun);
        const bool high = x1 * x1 > a.high_thr_f;
        float p32 = 0.f, w32 = 1.f;
        int it32 = 0;
        const bool ok32 = newton_fast<float>(1.0f, ssn, taun, a.gm_f, 0.0f, 2e-7f * taun, 1e-6f, 16, p32, w32, it32);
        float P[4];
        int kind = HYDRO_NONE;
        if (!high && ok32) {
            const float inv_dv = 1.0f / dV;
            const float inv_et = 1.0f / (taun + 1.0f + p32);
            P[0] = mf / w32 * inv_dv;
            P[1] = w32 * s1n * inv_et;
            P[2] = w32 * s2n * inv_et;
            P[3] = p32 * mf * inv_dv;
            if (p32 < 0.f) P[3] = (float)PRESSURE_FLOOR * P[0];
        } else {
            const Fp64Recovery r = recover_fp64(a, m, U[1], U[2], tau, dV, ok32, p32);
#pragma unroll
            for (int q = 0; q < 4; ++q) P[q] = r.P[q];
            kind = r.kind;
        }
        const float wz = sqrtf(__fmaf_rn(P[2], P[2], __fmaf_rn(P[1], P[1], 1.0f)));
#pragma unroll
        for (int q = 0; q < 4; ++q) v[q] = (R)P[q];
        v[4] = (R)(scalf / dV / wz);
        return kind;
    }
};

// Recovery of one zone; every thread of a warp calls zone() together (the
// learned guess is a warp-wide inference).
//
// DEFER: the zones that need the FP64 recovery (Lorentz factor above the
// split, or an FP32 iteration that did not converge) are appended to the
// stage's list (a.high) and left to c2p_high_kernel, which recovers them
// densely, with the learned guess, through the inline form: every zone meets
// the same arithmetic in both forms.
template <bool MLP, bool DEFER = false>
struct MixedC2p {
    static constexpr bool mlp = MLP;
    using RemapRec = MixedRemapRecovery;
    __device__ static void zone(const StageArgs& a, int slot, const DevBlock& B, int i, int j, bool active,
                                MlpWeights& W, __nv_bfloat16* act, C2pStats& st) {
        double U[5] = {1.0, 0.0, 0.0, 1.0, 0.0};
        if (active) {
            const int64_t n = (int64_t)B.nr * B.nq;
            const double* Ub = B.buf[a.sel_in] + (int64_t)i * B.nq + j;
#pragma unroll
            for (int q = 0; q < 5; ++q) U[q] = Ub[q * n];
        }
        zone_state(a, slot, B, i, j, active, U, W, act, st);
    }

    // The same with the zone's state U (D, S_r, S_theta, tau, scalar mass)
    // already loaded. DT: -1 reduce the time step when the stage asks for it
    // (a.compute_dt), 0 never, 1 always (a kernel specialised either way
    // carries no register for the other case).
    template <int DT = -1>
    __device__ static void zone_state(const StageArgs& a, int slot, const DevBlock& B, int i, int j, bool active,
                                      const double (&U)[5], MlpWeights& W, __nv_bfloat16* act, C2pStats& st) {
        const float gmf = a.gm_f;
        const float high_thr = a.high_thr_f;
        const float dV = active ? B.dv_r32[i] * B.dv_q[j].x : 1.0f;
        const double m = U[0], tau = U[3];
        int kind = HYDRO_NONE;
        if (active && is_negative(m)) kind = HYDRO_NEGATIVE_DENSITY;
        else if (active && is_negative(tau)) kind = HYDRO_NEGATIVE_ENERGY_DENSITY;
        // FP32 copies by integer conversion (no FP64-pipe instructions), in
        // the stage's length units: volumes (and so the volume integrals)
        // carry 2^(-3 e) with L = 2^e near the reference radius
        const int de = -a.lscale3;
        const float mf = d2f_rn_exp(m, de), tauf = d2f_rn_exp(tau, de);
        const float s1f = d2f_rn_exp(U[1], de), s2f = d2f_rn_exp(U[2], de);
        const float scalf = d2f_rn_exp(U[4], de);
        // the FP32 iteration runs on the state per unit mass (O(1) numbers,
        // no overflow or underflow of the squares whatever the units); the
        // recovery is scale-invariant, p = (p / m) m
        const float im = 1.0f / mf;
        const float s1n = s1f * im, s2n = s2f * im, taun = tauf * im;
        const float ssn = s1n * s1n + s2n * s2n;
        const float x1 = __fdividef(sqrtf(ssn), 1.0f + taun);   // |S| / (D + tau)
        const bool valid = active && kind == HYDRO_NONE;
        const bool high = valid && x1 * x1 > high_thr;
        float guess = 0.0f;   // p / m
        if (MLP) {
            if (__any_sync(0xffffffffu, high)) {
                float x[3];
                const bool ok = mlp_features(m, U[1] * U[1] + U[2] * U[2], tau, x);
                const float y = mlp_guess_call(W, act, x[0], x[1], x[2]);
                const float gsv = __expf(y);
                // the learned start is for the zones that go on to the FP64
                // recovery; the others start from the plain guess
                guess = (high && ok && gsv > 0.0f) ? fminf(gsv, (gmf - 1.0f) * taun) : 0.0f;
            }
        }
        float p32 = 0.f, w32 = 1.f;
        int it32 = 0;
        bool ok32 = false;
        // stop once the residual is at the rounding level of the energy
        // (|f| < 2e-7 tau / m, about 3 FP32 ulps of tau): further steps move p
        // by rounding noise only (5.6 -> 2.1 iterations per zone on the wind,
        // density L1 unchanged). The deferring form leaves the high zones'
        // iteration to the dense pass.
        if (valid && !(DEFER && high))
            ok32 = newton_fast<float>(1.0f, ssn, taun, gmf, guess, 2e-7f * taun, 1e-6f, 16, p32, w32, it32);
        bool fp64 = valid && (high || !ok32);
        if (DEFER && valid && !fp64 && w32 * w32 > 0.99f * (a.uu_high_f + 1.0f)) {
            // a zone whose stored FP32 four-velocity would be above the split
            // (the estimate from |S| / (D + tau) missed it) goes to the dense
            // pass too, which keeps its FP64 primitive for the update's FP64
            // faces: this kernel stores no zone above the split. (Below 0.99 of
            // the split's W^2 the converged W cannot give such a velocity.)
            const float inv_et = 1.0f / (taun + 1.0f + p32);
            fp64 = high_zone(w32 * s1n * inv_et, w32 * s2n * inv_et, a.uu_high_f);
        }
        if (DEFER) {
            const unsigned full = 0xffffffffu;
            const unsigned mask = __ballot_sync(full, fp64);
            if (mask) {
                const int lane = threadIdx.x & 31;
                unsigned base = 0;
                if (lane == __ffs(mask) - 1) base = atomicAdd(a.high_count, (unsigned)__popc(mask));
                base = __shfl_sync(full, base, __ffs(mask) - 1);
                const unsigned slot_k = base + __popc(mask & ((1u << lane) - 1u));
                // a full list (never reached: capacity = zones) keeps the zone here
                if (fp64 && slot_k < a.high_cap) {
                    a.high[slot_k] = make_int2(slot, (int)((int64_t)i * B.nq + j));
                    return;
                }
            }
        }
        float P[4] = {0.f, 0.f, 0.f, 0.f};
        if (valid) {
            ++st.zones;
            st.it32 += (unsigned)it32;
            if (!fp64) {
                const float inv_dv = 1.0f / dV;
                const float inv_et = 1.0f / (taun + 1.0f + p32);
                P[0] = mf / w32 * inv_dv;
                P[1] = w32 * s1n * inv_et;
                P[2] = w32 * s2n * inv_et;
                P[3] = p32 * mf * inv_dv;
                if (p32 < 0.f) P[3] = (float)PRESSURE_FLOOR * P[0];
            } else {
                // (deferring form: kept here, a high zone has not run the
                // FP32 iteration yet)
                const Fp64Recovery r =
                    DEFER ? recover_fp64_call(a, B, i, j, dV, ok32, p32, high, ssn, taun, guess)
                          : recover_fp64(a, m, U[1], U[2], tau, dV, ok32, p32);
                st.it32 += (unsigned)r.it32;
#pragma unroll
                for (int q = 0; q < 4; ++q) P[q] = r.P[q];
                kind = r.kind;
                st.it64 += (unsigned)r.it64;
                st.fbs += (unsigned)r.fbs;
            }
        }
        if (active) {
            if (kind != HYDRO_NONE) {
                atomicMin(&a.status->err_key, error_key(a.stage, slot, i, j, kind));
                a.status->err_sel = a.sel_in;
            }
            // W = sqrt(1 + u^2) with explicit fused operations: the same
            // products appear in the time-step reduction below, and a kernel
            // with or without that reduction must round W alike
            const float wz = sqrtf(__fmaf_rn(P[2], P[2], __fmaf_rn(P[1], P[1], 1.0f)));
            const float v[NFIELD] = {P[0], P[1], P[2], P[3], scalf / dV / wz};
            store_prim<float>(B, i, j, v);
            // above the split: its FP64 primitive for the update's FP64 faces
            // (the deferring form stores no such zone: it defers every zone
            // above the split, and its list holds every zone of the layout)
            if constexpr (!DEFER) {
                if (high_zone(P[1], P[2], a.uu_high_f)) hp_store(a, slot, B, i, j, v);
            }
            if ((DT < 0 ? a.compute_dt != 0 : DT > 0) && kind == HYDRO_NONE) {
                // State::time_step (src/state.rs:151-160) on this stage's
                // primitives: signal speed in FP32, dl and dl / a in FP64
                PhysT<float> ph;
                ph.srhd = 1;
                ph.hllc = 0;
                ph.gm = a.gm_f;
                ph.gm1 = a.gm1_f;
                ph.gh = a.gh_f;
                ph.theta = a.theta_f;
                const double dr = B.rv[i + 1] - B.rv[i];
                const double dq = B.qv[j + 1] - B.qv[j];
                const double dl = fmin(dr, dq * B.rv[i]);
                const double amax = (double)max_signal_speed(ph, P) * a.cflux;
                st.dtz = fmin(st.dtz, dl / amax);
            }
        }
    }
};

template <bool MLP>
__global__ void __launch_bounds__(TILE_THREADS, 3) c2p_mixed_kernel(StageArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned long long ek = *(volatile unsigned long long*)&a.status->err_key;
    if (ek != NO_ERROR && (uint32_t)(ek >> 48) < (uint32_t)a.stage) return;
    MlpWeights& W = *reinterpret_cast<MlpWeights*>(smem_raw);
    __nv_bfloat16* act = reinterpret_cast<__nv_bfloat16*>(smem_raw + sizeof(MlpWeights)) +
                         (threadIdx.x >> 5) * MLP_ACT_ELEMS;
    if (MLP) {
        mlp_load(W, a.mlp);
        __syncthreads();
    }
    C2pStats st;
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        const int4 t = a.tiles[tile];
        const DevBlock& B = a.blocks[t.x];
        const int i = t.y + threadIdx.x / TILE_Q;
        const int j = t.z + threadIdx.x % TILE_Q;
        MixedC2p<MLP>::zone(a, t.x, B, i, j, i < B.nr && j < B.nq, W, act, st);
    }
    warp_reduce_stats(a.status, st.zones, st.it64, st.it32, st.fbs, st.dtz, a.compute_dt != 0);
}

// ---- recovery by warps walking the rows of a tile -----------------------------
// The recovery's arithmetic between its loads and its stores is long and
// serial, so a zone-per-thread loop keeps few loads in flight and runs
// latency-bound. Here a warp takes a whole recovery tile (TILE_R rows of 32
// zones): the tile's descriptor and block fields are read once instead of once
// per zone, and each lane copies its column's state of the rows C2P_DEPTH - 1
// ahead into shared memory with cp.async (8-byte, L1-allocating) while it
// recovers the current row, so the copies hold no registers. A lane reads
// only the slots it filled (no barrier); cp.async.wait_group orders its own
// copies, and the slot it refills is the one it read a row earlier.
constexpr int C2P_DEPTH = 3;

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// One recovery tile t = {slot, i0, j0, -} walked by the calling warp: its
// TILE_R rows of 32 zones, each lane's column of the next rows copied ahead
// into the warp's staging slots sUw. Zones that need the FP64 recovery go to
// the stage's list (a.high).
template <int DT>
__device__ __forceinline__ void recover_rows_tile(const StageArgs& a, const int4 t, double (*sUw)[NFIELD][32],
                                                  MlpWeights& W, C2pStats& st) {
    const int lane = threadIdx.x & 31;
    const DevBlock& B = a.blocks[t.x];
    const int j = t.z + lane;
    const bool jin = j < B.nq;
    const int rows = min(TILE_R, B.nr - t.y);
    const int64_t n = (int64_t)B.nr * B.nq;
    const double* Ub = B.buf[a.sel_in] + (int64_t)t.y * B.nq + j;
    auto issue = [&](int r) {
        if (jin && r < rows) {
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) cp_async8(&sUw[r % C2P_DEPTH][q][lane], Ub + q * n + (int64_t)r * B.nq);
        }
        cp_async_commit();
    };
#pragma unroll
    for (int r = 0; r < C2P_DEPTH - 1; ++r) issue(r);
    for (int r = 0; r < rows; ++r) {
        issue(r + C2P_DEPTH - 1);
        cp_async_wait<C2P_DEPTH - 1>();
        double U[5] = {1.0, 0.0, 0.0, 1.0, 0.0};
        if (jin) {
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) U[q] = sUw[r % C2P_DEPTH][q][lane];
        }
        MixedC2p<false, true>::zone_state<DT>(a, t.x, B, t.y + r, j, jin, U, W, nullptr, st);
    }
}

template <int DT>
__global__ void __launch_bounds__(TILE_THREADS, 3) c2p_rows_kernel(StageArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int WPC = TILE_THREADS / 32;
    __shared__ __align__(16) double sU[WPC][C2P_DEPTH][NFIELD][32];
    dependency_wait();
    launch_dependents();
    const unsigned long long ek = *(volatile unsigned long long*)&a.status->err_key;
    if (ek != NO_ERROR && (uint32_t)(ek >> 48) < (uint32_t)a.stage) return;
    MlpWeights& W = *reinterpret_cast<MlpWeights*>(smem_raw);   // unused without the learned guess
    const int w = threadIdx.x >> 5;
    C2pStats st;
    for (int tile = blockIdx.x * WPC + w; tile < a.ntiles; tile += gridDim.x * WPC)
        recover_rows_tile<DT>(a, a.tiles[tile], sU[w], W, st);
    cp_async_wait<0>();
    warp_reduce_stats(a.status, st.zones, st.it64, st.it32, st.fbs, st.dtz, a.compute_dt != 0);
}

// The deferred zones (the first `count` of a.high), 32 per warp: warps
// first, first + step, ... of the grid. Every lane of a warp calls it.
template <bool MLP>
__device__ __forceinline__ void recover_high_groups(const StageArgs& a, unsigned count, unsigned first,
                                                    unsigned step, MlpWeights& W, __nv_bfloat16* act,
                                                    C2pStats& st) {
    const unsigned lane = threadIdx.x & 31;
    for (unsigned base = first * 32; base < count; base += step * 32) {
        const unsigned k = base + lane;
        const bool active = k < count;
        const int2 e = a.high[active ? k : base];
        const DevBlock& B = a.blocks[e.x];
        const int i = e.y / B.nq, j = e.y - i * B.nq;
        MixedC2p<MLP>::zone(a, e.x, B, i, j, active, W, act, st);
    }
}

// The deferred zones of this stage ({slot, z} in a.high, *a.high_count of
// them): warps take 32 at a time, so the learned guess and the FP64 recovery
// run on full warps. Clears the other stage parity's counter for the next
// stage (its last reader finished before this launch).
template <bool MLP>
__global__ void __launch_bounds__(TILE_THREADS, 2) c2p_high_kernel(StageArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    dependency_wait();
    launch_dependents();
    const unsigned long long ek = *(volatile unsigned long long*)&a.status->err_key;
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.high_count_next = 0u;
    if (ek != NO_ERROR && (uint32_t)(ek >> 48) < (uint32_t)a.stage) return;
    const unsigned count = min(*(volatile unsigned*)a.high_count, a.high_cap);
    // CTAs without a group of the list stop before loading the network
    if ((unsigned)blockIdx.x * TILE_THREADS >= count) return;
    MlpWeights& W = *reinterpret_cast<MlpWeights*>(smem_raw);
    __nv_bfloat16* act = reinterpret_cast<__nv_bfloat16*>(smem_raw + sizeof(MlpWeights)) +
                         (threadIdx.x >> 5) * MLP_ACT_ELEMS;
    if (MLP) {
        mlp_load(W, a.mlp);
        __syncthreads();
    }
    C2pStats st;
    recover_high_groups<MLP>(a, count, blockIdx.x * (TILE_THREADS / 32) + (threadIdx.x >> 5),
                             gridDim.x * (TILE_THREADS / 32), W, act, st);
    warp_reduce_stats(a.status, st.zones, st.it64, st.it32, st.fbs, st.dtz, a.compute_dt != 0);
}

// ---- the fused stage (mixed) -------------------------------------------------
template <int TR, bool MLP>
__global__ void __launch_bounds__(update_threads<TR>(), MLP ? (TR == 4 ? 3 : TR == 8 ? 2 : 1) : (TR == 4 ? 5 : TR == 8 ? 3 : 2))
    stage_fused_mixed_kernel(StageArgs a, GhostArgs g,
                                                                                    FusedArgs f) {
    stage_fused_body<float, true, TR, MixedC2p<MLP>>(a, g, f);
}

static int g_sms = 0;

static int num_sms() {
    if (!g_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_sms <= 0) g_sms = 1;
    }
    return g_sms;
}

// Resident CTAs of a kernel on the whole device, cached per kernel.
template <class K>
static int resident_grid(K kernel, int threads, size_t smem) {
    static std::mutex mu;
    static std::map<const void*, int> cache;
    std::lock_guard<std::mutex> lock(mu);
    const void* key = reinterpret_cast<const void*>(kernel);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int per_sm = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return cache[key] = per_sm * num_sms();
}

cudaError_t launch_c2p_mixed(const StageArgs& a, cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (a.high) {
        // every zone in FP32; the ones that need the FP64 recovery, densely after
        // one warp per recovery tile
        const int wt = (a.ntiles + TILE_THREADS / 32 - 1) / (TILE_THREADS / 32);
        auto k = a.compute_dt ? c2p_rows_kernel<1> : c2p_rows_kernel<0>;
        const int grid = std::min(wt, resident_grid(k, TILE_THREADS, 0));
        cudaError_t e = launch_chained(k, grid, TILE_THREADS, 0, s, a);
        if (e != cudaSuccess) return e;
        if (a.mlp) {
            const size_t bytes = sizeof(MlpWeights) + 8 * MLP_ACT_ELEMS * sizeof(__nv_bfloat16);
            return launch_chained(c2p_high_kernel<true>, num_sms(), TILE_THREADS, bytes, s, a);
        }
        return launch_chained(c2p_high_kernel<false>, num_sms(), TILE_THREADS, 0, s, a);
    }
    if (a.mlp) {
        const size_t bytes = sizeof(MlpWeights) + 8 * MLP_ACT_ELEMS * sizeof(__nv_bfloat16);
        const int grid = std::min(a.ntiles, resident_grid(c2p_mixed_kernel<true>, TILE_THREADS, bytes));
        c2p_mixed_kernel<true><<<grid, TILE_THREADS, bytes, s>>>(a);
    } else {
        const int grid = std::min(a.ntiles, resident_grid(c2p_mixed_kernel<false>, TILE_THREADS, 0));
        c2p_mixed_kernel<false><<<grid, TILE_THREADS, 0, s>>>(a);
    }
    return cudaGetLastError();
}

// ---- the update with tensor-copy staging ---------------------------------------
// A persistent CTA walks its update tiles with two shared-memory buffers: while
// it computes tile k from one, the tensor copies of tile k + 1 (primitives
// with halo, U_in, U_base) fill the other. Same arithmetic as update_kernel.
template <int TR>
struct TmaSmem {
    static constexpr size_t P_BYTES = (size_t)NFIELD * (TR + 4) * (TILE_Q + 8) * sizeof(float);
    static constexpr size_t U_BYTES = (size_t)NFIELD * TR * TILE_Q * sizeof(double);
    static constexpr size_t BUF = P_BYTES + 2 * U_BYTES;
    static constexpr size_t WORK = ((StageSmem<float, TR>::work_bytes + 127) / 128) * 128;
    static constexpr size_t bytes = 128 + 2 * BUF + WORK + 16;   // alignment slack, buffers, work, 2 mbarriers
};

template <int TR>
__global__ void __launch_bounds__(update_threads<TR>(), 1) update_tma_kernel(StageArgs a) {
    using L = TmaSmem<TR>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned char* base = smem_raw + ((128 - (smem_u32(smem_raw) & 127)) & 127);
    unsigned char* work = base + 2 * L::BUF;
    uint64_t* bar = reinterpret_cast<uint64_t*>(work + L::WORK);
    // a failed recovery in this or an earlier stage stops the step
    if (*(volatile unsigned long long*)&a.status->err_key != NO_ERROR) return;
    const bool avg = a.sel_base >= 0;
    const uint32_t tx = (uint32_t)(L::P_BYTES + L::U_BYTES * (avg ? 2 : 1));
    const TmaMaps* maps = reinterpret_cast<const TmaMaps*>(a.tmaps);
    clear_next_hp(a);
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_barrier_init();
    }
    __syncthreads();
    auto issue = [&](int tile, int b) {
        const int4 t = a.utiles[tile];
        const TmaMaps* m = maps + t.x;
        unsigned char* d = base + b * L::BUF;
        mbar_arrive_expect_tx(&bar[b], tx);
        tma_load_3d(d, &m->P, t.z - 4, t.y, 0, &bar[b]);
        tma_load_3d(d + L::P_BYTES, &m->U[a.sel_in], t.z, t.y, 0, &bar[b]);
        if (avg) tma_load_3d(d + L::P_BYTES + L::U_BYTES, &m->U[a.sel_base], t.z, t.y, 0, &bar[b]);
    };
    int tile = blockIdx.x;
    if (threadIdx.x == 0 && tile < a.nutiles) issue(tile, 0);
    int k = 0;
    bool ok = true;
    for (; tile < a.nutiles; ++k, tile += gridDim.x) {
        const int b = k & 1;
        const int next = tile + gridDim.x;
        if (threadIdx.x == 0 && next < a.nutiles) {
            fence_proxy_async();   // the reads of buffer b ^ 1 (tile k - 1) come first
            issue(next, b ^ 1);
        }
        const bool got = mbar_wait_bounded(&bar[b], (uint32_t)(k >> 1) & 1u, TMA_WAIT_LIMIT);
        if (!__syncthreads_and(got)) {
            ok = false;
            break;
        }
        const unsigned char* d = base + b * L::BUF;
        update_tile<float, true, TR, true>(a, a.utiles[tile], work, reinterpret_cast<const float*>(d),
                                           reinterpret_cast<const double*>(d + L::P_BYTES),
                                           reinterpret_cast<const double*>(d + L::P_BYTES + L::U_BYTES));
        __syncthreads();
    }
    if (!ok && threadIdx.x == 0) {
        // a copy did not complete: record it, and let the copies in flight land
        // (bounded) before the CTA's shared memory is released
        atomicExch(&a.status->bar_abort, 2);
        mbar_wait_bounded(&bar[k & 1], (uint32_t)(k >> 1) & 1u, TMA_WAIT_LIMIT);
        if (tile + gridDim.x < a.nutiles)
            mbar_wait_bounded(&bar[(k + 1) & 1], (uint32_t)((k + 1) >> 1) & 1u, TMA_WAIT_LIMIT);
    }
    if (ok) drain_hp(a);
}

// The bounded mbarrier wait of update_tma_kernel on a barrier that nothing
// arrives on and no copy targets: it must give up after `polls` polls.
__global__ void copy_wait_selftest_kernel(int32_t polls, int32_t* timed_out) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) *timed_out = mbar_wait_bounded(&bar, 0u, polls) ? 0 : 1;
}

template <int TR>
static void update_tma(const StageArgs& a, cudaStream_t s) {
    const int grid = std::min(a.nutiles, resident_grid(update_tma_kernel<TR>, update_threads<TR>(), TmaSmem<TR>::bytes));
    update_tma_kernel<TR><<<grid, update_threads<TR>(), TmaSmem<TR>::bytes, s>>>(a);
}

template <int TR>
static void update_mixed(const StageArgs& a, cudaStream_t s) {
    if (a.tma && a.tmaps) {
        update_tma<TR>(a, s);
        return;
    }
    const size_t smem = StageSmem<float, TR>::bytes;
    const int grid = std::min(a.nutiles, resident_grid(update_kernel<float, true, TR>, update_threads<TR>(), smem));
    update_kernel<float, true, TR><<<grid, update_threads<TR>(), smem, s>>>(a);
}

template <int MB>
static void update_strips(const StageArgs& a, cudaStream_t s) {
    const int want = (a.nstrips + STRIP_WARPS - 1) / STRIP_WARPS;
    const int grid = std::min(want, resident_grid(update_strip_kernel<float, true, MB>, STRIP_WARPS * 32, 0));
    launch_chained(update_strip_kernel<float, true, MB>, grid, STRIP_WARPS * 32, 0, s, a);
}

cudaError_t launch_update_mixed(const StageArgs& a, cudaStream_t s) {
    if (a.strips) {
        if (a.nstrips <= 0) return cudaSuccess;
        switch (a.strip_ctas) {
        case 5: update_strips<5>(a, s); break;
        case 6: update_strips<6>(a, s); break;
        default: update_strips<4>(a, s);
        }
        return cudaGetLastError();
    }
    if (a.nutiles <= 0) return cudaSuccess;
    switch (a.utr) {
    case 4: update_mixed<4>(a, s); break;
    case 16: update_mixed<16>(a, s); break;
    default: update_mixed<8>(a, s);
    }
    return cudaGetLastError();
}

template <int TR>
static cudaError_t configure_update_mixed() {
    cudaError_t e = cudaFuncSetAttribute(update_kernel<float, true, TR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)StageSmem<float, TR>::bytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(update_tma_kernel<TR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)TmaSmem<TR>::bytes);
}

cudaError_t launch_ghost_mixed(const GhostArgs& a, cudaStream_t s) {
    const int nq = a.nq[0] > a.nq[1] ? a.nq[0] : a.nq[1];
    dim3 grid((2 * nq + 127) / 128, 2);
    ghost_kernel<<<grid, 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_remap_mixed(const StageArgs& a, const int4* remap, int nremap, int max_nq, cudaStream_t s) {
    if (nremap <= 0) return cudaSuccess;
    dim3 grid((2 * max_nq + 127) / 128, nremap);
    remap_kernel<float, MixedRemapRecovery><<<grid, 128, 0, s>>>(a, remap);
    return cudaGetLastError();
}

template <int TR, bool MLP>
static cudaError_t fused_mixed(const StageArgs& a, const GhostArgs& g, const FusedArgs& f, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(update_threads<TR>());
    cfg.dynamicSmemBytes = fused_smem_bytes<float, TR, MLP>();
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, stage_fused_mixed_kernel<TR, MLP>, a, g, f);
}

// The fused stage with warp strips only: CTAs of 4 warps, recovery chunks of
// 128 zones.
template <bool MLP>
__global__ void __launch_bounds__(STRIP_WARPS * 32, 5)
    stage_fused_strip_mixed_kernel(StageArgs a, GhostArgs g, FusedArgs f) {
    stage_fused_body<float, true, 8, MixedC2p<MLP>, STRIP_WARPS * 32, true>(a, g, f);
}

// The phases of the fused deferring stage; each sums its recovery statistics
// (and the time-step reduction) like its separate kernel does.
// Phase A of the fused deferring stage, per warp: work items claimed one at a
// time (a.status->item_claim), first the ghost rows of both mesh ends in
// groups of 32 zones, then the recovery tiles. The ghost rows are a long FP64
// latency chain per zone (the separate form hides it on a second stream);
// claimed first and dynamically, they delay no warp's share of the tiles.
template <int DT>
__device__ __forceinline__ void fused_phase_a(const StageArgs& a, const GhostArgs& g, double (*sUw)[NFIELD][32],
                                              MlpWeights& W) {
    const unsigned lane = threadIdx.x & 31;
    const unsigned ng0 = (unsigned)(2 * g.nq[0] + 31) / 32, ng1 = (unsigned)(2 * g.nq[1] + 31) / 32;
    const unsigned total = ng0 + ng1 + (unsigned)a.ntiles;
    C2pStats st;
    for (;;) {
        unsigned item = 0u;
        if (lane == 0) item = atomicAdd(&a.status->item_claim, 1u);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= total) break;
        if (item < ng0) ghost_zone(g, 0, (int)(item * 32 + lane));
        else if (item < ng0 + ng1) ghost_zone(g, 1, (int)((item - ng0) * 32 + lane));
        else recover_rows_tile<DT>(a, a.tiles[item - ng0 - ng1], sUw, W, st);
    }
    cp_async_wait<0>();
    warp_reduce_stats(a.status, st.zones, st.it64, st.it32, st.fbs, st.dtz, a.compute_dt != 0);
}

template <bool MLP, int WARPS>
__device__ __forceinline__ void fused_high_phase(const StageArgs& a, unsigned count, MlpWeights& W,
                                                 __nv_bfloat16* act) {
    C2pStats st;
    recover_high_groups<MLP>(a, count, blockIdx.x * WARPS + (threadIdx.x >> 5), gridDim.x * WARPS, W, act, st);
    warp_reduce_stats(a.status, st.zones, st.it64, st.it32, st.fbs, st.dtz, a.compute_dt != 0);
}

template <int WARPS>
__device__ __forceinline__ void fused_remap_phase(const StageArgs& a, const FusedArgs& f) {
    constexpr int NT = WARPS * 32;
    const int per = 2 * f.max_nq;
    const int total = f.nremap * per;
    for (int k = blockIdx.x * NT + threadIdx.x; k < total; k += gridDim.x * NT) {
        const int item = k / per;
        remap_zone<float, MixedRemapRecovery>(a, f.remap[item], k - item * per);
    }
}

template <int WARPS>
__device__ __forceinline__ void fused_update_phase(const StageArgs& a) {
    stage_strips<float, true>(a, blockIdx.x * WARPS + (int)(threadIdx.x >> 5), gridDim.x * WARPS);
}

// The fused stage with the deferring recovery and warp strips, the separate
// form's five launches in one (CTAs of WARPS warps, all resident):
//   A  work items claimed by warps: ghost rows of both mesh ends in groups of
//      32 zones, then the recovery tiles, rows walked with the next rows copied
//      ahead (recover_rows_tile; zones needing the FP64 recovery are listed);
//   -- barrier --
//   B  the listed zones densely (recover_high_groups, learned guess on the
//      tensor cores); -- barrier, only waited on when the list holds a zone --
//      then the halo remaps across polar-resolution changes (they copy a
//      coarser neighbour's recovered primitives, so they follow the dense
//      pass); -- barrier, only waited on with remaps --
//   C  the warp strips of the update.
// Every launch counts three barrier arrivals per CTA (the host advances its
// barrier epoch by three grids); a barrier whose phase has no work is passed
// with its arrival only. The phases call the functions of the separate
// kernels, so the two forms give bit-identical states.
// Shared memory (dynamic): each warp's staging slots of the recovery, then
// (with the learned guess) the network and one activation tile per warp.
template <bool MLP, int WARPS>
constexpr size_t fused_deferred_smem_bytes() {
    return sizeof(double) * WARPS * C2P_DEPTH * NFIELD * 32 +
           (MLP ? sizeof(MlpWeights) + WARPS * MLP_ACT_ELEMS * sizeof(__nv_bfloat16) : 0);
}

template <bool MLP, int WARPS, int MB>
__global__ void __launch_bounds__(WARPS * 32, MB)
    stage_fused_deferred_kernel(const __grid_constant__ StageArgs a, const __grid_constant__ GhostArgs g,
                                const __grid_constant__ FusedArgs f) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int run_update;
    constexpr int NT = WARPS * 32;
    typedef double Slots[C2P_DEPTH][NFIELD][32];
    Slots* sU = reinterpret_cast<Slots*>(smem_raw);
    unsigned char* mlp_area = smem_raw + sizeof(double) * WARPS * C2P_DEPTH * NFIELD * 32;
    MlpWeights& W = *reinterpret_cast<MlpWeights*>(mlp_area);
    __nv_bfloat16* act = reinterpret_cast<__nv_bfloat16*>(mlp_area + sizeof(MlpWeights)) +
                         (threadIdx.x >> 5) * MLP_ACT_ELEMS;
    // a failure in an earlier stage stops the step; every CTA still arrives
    // at every barrier
    const unsigned long long ek = *(volatile unsigned long long*)&a.status->err_key;
    const bool run = !(ek != NO_ERROR && (uint32_t)(ek >> 48) < (uint32_t)a.stage);

    // ---- A
    if (run) {
        if (a.compute_dt) fused_phase_a<1>(a, g, sU[threadIdx.x >> 5], W);
        else fused_phase_a<0>(a, g, sU[threadIdx.x >> 5], W);
    }
    grid_barrier(a.status, f.bar_base + gridDim.x, f.spin_limit);

    // ---- B: the listed zones, then the remaps
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *a.high_count_next = 0u;       // the next stage's list starts empty
        a.status->item_claim = 0u;     // phase A's items are all claimed: zero for the next launch
    }
    const unsigned count = min(*(volatile unsigned*)a.high_count, a.high_cap);
    if (run && count > 0u && (unsigned)blockIdx.x * NT < count) {
        if (MLP) {
            mlp_load(W, a.mlp);
            __syncthreads();
        }
        fused_high_phase<MLP, WARPS>(a, count, W, act);
    }
    if (count > 0u) grid_barrier(a.status, f.bar_base + 2ull * gridDim.x, f.spin_limit);
    else grid_arrive(a.status);
    if (f.nremap > 0) {
        if (run) fused_remap_phase<WARPS>(a, f);
        grid_barrier(a.status, f.bar_base + 3ull * gridDim.x, f.spin_limit);
    } else {
        grid_arrive(a.status);
    }

    // ---- C: the update's warp strips (skipped after any failure, like the separate kernel)
    if (threadIdx.x == 0)
        run_update = *(volatile unsigned long long*)&a.status->err_key == NO_ERROR &&
                     *(volatile int32_t*)&a.status->bar_abort == 0;
    __syncthreads();
    if (run_update) fused_update_phase<WARPS>(a);
}

// The variants: CTAs of 4 warps built for 4 (no spills) or 5 resident CTAs
// per SM, or one CTA of FUSED_WIDE_WARPS warps per SM (fewer arrivals at each
// grid barrier: one per SM instead of four or five).
constexpr int FUSED_WIDE_WARPS = 20;

template <bool MLP, int WARPS, int MB>
static cudaError_t fused_deferred_configure() {
    return cudaFuncSetAttribute(stage_fused_deferred_kernel<MLP, WARPS, MB>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)fused_deferred_smem_bytes<MLP, WARPS>());
}

template <bool MLP, int WARPS, int MB>
static cudaError_t fused_deferred(const StageArgs& a, const GhostArgs& g, const FusedArgs& f, int grid,
                                  cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(WARPS * 32);
    cfg.dynamicSmemBytes = fused_deferred_smem_bytes<MLP, WARPS>();
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, stage_fused_deferred_kernel<MLP, WARPS, MB>, a, g, f);
}

template <bool MLP, int WARPS, int MB>
static cudaError_t fused_deferred_ctas(int* n) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, stage_fused_deferred_kernel<MLP, WARPS, MB>, WARPS * 32,
                                                         fused_deferred_smem_bytes<MLP, WARPS>());
}

cudaError_t fused_deferred_max_ctas_mixed(bool mlp, int mb, int* n) {
    if (mb == 1)
        return mlp ? fused_deferred_ctas<true, FUSED_WIDE_WARPS, 1>(n) : fused_deferred_ctas<false, FUSED_WIDE_WARPS, 1>(n);
    if (mb == 4) return mlp ? fused_deferred_ctas<true, STRIP_WARPS, 4>(n) : fused_deferred_ctas<false, STRIP_WARPS, 4>(n);
    return mlp ? fused_deferred_ctas<true, STRIP_WARPS, 5>(n) : fused_deferred_ctas<false, STRIP_WARPS, 5>(n);
}

int fused_deferred_threads(int mb) { return (mb == 1 ? FUSED_WIDE_WARPS : STRIP_WARPS) * 32; }

template <bool MLP>
static cudaError_t fused_strip_mixed(const StageArgs& a, const GhostArgs& g, const FusedArgs& f, int grid,
                                     cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(STRIP_WARPS * 32);
    cfg.dynamicSmemBytes = fused_strip_smem_bytes<MLP>();
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, stage_fused_strip_mixed_kernel<MLP>, a, g, f);
}

cudaError_t fused_strip_max_ctas_mixed(bool mlp, int* n) {
    return mlp ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, stage_fused_strip_mixed_kernel<true>,
                                                               STRIP_WARPS * 32, fused_strip_smem_bytes<true>())
               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, stage_fused_strip_mixed_kernel<false>,
                                                               STRIP_WARPS * 32, fused_strip_smem_bytes<false>());
}

cudaError_t launch_stage_fused_mixed(const StageArgs& a, const GhostArgs& g, const FusedArgs& f, int grid,
                                     cudaStream_t s) {
    const bool mlp = a.mlp != nullptr;
    if (a.strips && a.high) {
        // one wide CTA per SM, or 4-warp CTAs built for 4 per SM (no spills) or 5 (more warps)
        if (a.fused_wide)
            return mlp ? fused_deferred<true, FUSED_WIDE_WARPS, 1>(a, g, f, grid, s)
                       : fused_deferred<false, FUSED_WIDE_WARPS, 1>(a, g, f, grid, s);
        if (a.strip_ctas == 4)
            return mlp ? fused_deferred<true, STRIP_WARPS, 4>(a, g, f, grid, s)
                       : fused_deferred<false, STRIP_WARPS, 4>(a, g, f, grid, s);
        return mlp ? fused_deferred<true, STRIP_WARPS, 5>(a, g, f, grid, s)
                   : fused_deferred<false, STRIP_WARPS, 5>(a, g, f, grid, s);
    }
    if (a.strips) return mlp ? fused_strip_mixed<true>(a, g, f, grid, s) : fused_strip_mixed<false>(a, g, f, grid, s);
    switch (fused_tr(a.utr)) {
    case 4: return mlp ? fused_mixed<4, true>(a, g, f, grid, s) : fused_mixed<4, false>(a, g, f, grid, s);
    case 16: return mlp ? fused_mixed<16, true>(a, g, f, grid, s) : fused_mixed<16, false>(a, g, f, grid, s);
    default: return mlp ? fused_mixed<8, true>(a, g, f, grid, s) : fused_mixed<8, false>(a, g, f, grid, s);
    }
}

template <int TR, bool MLP>
static cudaError_t fused_ctas_mixed(int* n) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, stage_fused_mixed_kernel<TR, MLP>, update_threads<TR>(),
                                                         fused_smem_bytes<float, TR, MLP>());
}

cudaError_t fused_max_ctas_mixed(bool mlp, int utr, int* n) {
    switch (fused_tr(utr)) {
    case 4: return mlp ? fused_ctas_mixed<4, true>(n) : fused_ctas_mixed<4, false>(n);
    case 16: return mlp ? fused_ctas_mixed<16, true>(n) : fused_ctas_mixed<16, false>(n);
    default: return mlp ? fused_ctas_mixed<8, true>(n) : fused_ctas_mixed<8, false>(n);
    }
}

template <int TR, bool MLP>
static cudaError_t configure_fused_mixed() {
    return cudaFuncSetAttribute(stage_fused_mixed_kernel<TR, MLP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)fused_smem_bytes<float, TR, MLP>());
}

cudaError_t configure_f64();

// Kernel attributes (shared memory above the default limit), once per device.
cudaError_t configure_kernels() {
    constexpr int MAX_DEVICES = 64;
    static bool done[MAX_DEVICES] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) dev = 0;
    if (done[dev]) return cudaSuccess;
    cudaError_t e = configure_f64();
    if (e == cudaSuccess) e = configure_update_mixed<4>();
    if (e == cudaSuccess) e = configure_update_mixed<8>();
    if (e == cudaSuccess) e = configure_update_mixed<16>();
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(c2p_high_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(MlpWeights) + 8 * MLP_ACT_ELEMS * sizeof(__nv_bfloat16)));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(stage_fused_strip_mixed_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)fused_strip_smem_bytes<true>());
    if (e == cudaSuccess) e = configure_fused_mixed<4, false>();
    if (e == cudaSuccess) e = configure_fused_mixed<8, false>();
    if (e == cudaSuccess) e = configure_fused_mixed<16, false>();
    if (e == cudaSuccess) e = configure_fused_mixed<4, true>();
    if (e == cudaSuccess) e = configure_fused_mixed<8, true>();
    if (e == cudaSuccess) e = configure_fused_mixed<16, true>();
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(c2p_mixed_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(MlpWeights) + 8 * MLP_ACT_ELEMS * sizeof(__nv_bfloat16)));
    if (e == cudaSuccess) e = fused_deferred_configure<false, STRIP_WARPS, 4>();
    if (e == cudaSuccess) e = fused_deferred_configure<true, STRIP_WARPS, 4>();
    if (e == cudaSuccess) e = fused_deferred_configure<false, STRIP_WARPS, 5>();
    if (e == cudaSuccess) e = fused_deferred_configure<true, STRIP_WARPS, 5>();
    if (e == cudaSuccess) e = fused_deferred_configure<false, FUSED_WIDE_WARPS, 1>();
    if (e == cudaSuccess) e = fused_deferred_configure<true, FUSED_WIDE_WARPS, 1>();
    done[dev] = e == cudaSuccess;
    return e;
}

}  // namespace knc

extern "C" int knc_selftest_copy_wait(int32_t polls, int32_t* timed_out) {
    if (polls < 1 || !timed_out) return KNC_ERR_INVALID_ARGUMENT;
    int32_t* d = nullptr;
    if (cudaMalloc(&d, sizeof(int32_t)) != cudaSuccess) return KNC_ERR_OUT_OF_MEMORY;
    cudaError_t e = cudaMemset(d, 0xff, sizeof(int32_t));
    if (e == cudaSuccess) {
        knc::copy_wait_selftest_kernel<<<1, 32>>>(polls, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(timed_out, d, sizeof(int32_t), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? KNC_OK : KNC_ERR_CUDA;
}
