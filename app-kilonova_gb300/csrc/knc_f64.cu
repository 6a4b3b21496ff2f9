// knc_f64.cu — the plain FP64 stage (compiled with --fmad=false).
//
// Kernels of one RK stage on the reference's method in FP64:
//   c2p_f64     BlockState::try_to_primitive + scalar density for every zone
//               (src/state.rs:76-94, src/scheme.rs:32-39); also the adaptive
//               time-step reduction of State::time_step (src/state.rs:151-160)
//   ghost       the two ghost blocks' halo rows from the model at the stage
//               time (src/scheme.rs:45-52 via BlockState::from_model)
//   update      flux / source / update / RK average (knc_stage.cuh)
//   init        State::from_model (src/state.rs:55-69, 107-115)
// Without FMA contraction every expression rounds exactly like the CPU
// oracle's, so this path reproduces the reference arithmetic bit for bit
// wherever the libm-free operations (+ - * / sqrt) are all that is used.
#include "knc_fused.cuh"
#include "knc_halo.cuh"
#include "knc_internal.h"
#include "knc_mlp.cuh"
#include "knc_models.cuh"
#include "knc_physics.cuh"
#include "knc_stage.cuh"

namespace knc {

// ---- c2p -------------------------------------------------------------------
// MLP = true: the Newton recovery starts from the learned pressure guess; the
// plain guess p = 0 is retried when that start does not converge. Every
// thread of a warp calls zone() together (the guess is a warp-wide inference).
template <bool MLP>
struct F64C2p {
    static constexpr bool mlp = MLP;
    using RemapRec = RemapRecoveryF64;
    __device__ static void zone(const StageArgs& a, int slot, const DevBlock& B, int i, int j, bool active,
                                MlpWeights& W, __nv_bfloat16* act, C2pStats& st) {
        const int nr = B.nr, nq = B.nq;
        const int64_t n = (int64_t)nr * nq;
        const int64_t z = (int64_t)i * nq + j;
        double u[4] = {1.0, 0.0, 0.0, 1.0};
        double smass = 0.0, dV = 1.0;
        if (active) {
            const double* U = B.buf[a.sel_in];
            dV = B.dv[z];
#pragma unroll
            for (int q = 0; q < 4; ++q) u[q] = U[q * n + z] / dV;
            smass = U[4 * n + z];
        }
        double guess = 0.0;
        if (MLP && a.srhd) {
            float x[3];
            const bool ok = mlp_features(u[0], u[1] * u[1] + u[2] * u[2], u[3], x);
            const float y = mlp_warp_infer(W, act, x);
            const double g = u[0] * (double)__expf(y);
            const double gmax = (a.gm - 1.0) * u[3];
            guess = (ok && g > 0.0) ? fmin(g, gmax) : 0.0;
        }
        if (!active) return;
        double P[4] = {0.0, 0.0, 0.0, 0.0};
        double bad = 0.0;
        int kind, iters = 0;
        if (a.srhd) {
            kind = srhd_c2p_newton(a.gm, u, guess, P, iters, bad);
            if (MLP && kind == HYDRO_ROOT_FINDER_FAILED && guess != 0.0) {
                int it2 = 0;
                ++st.fbs;
                kind = srhd_c2p_newton(a.gm, u, 0.0, P, it2, bad);
                iters += it2;
            }
        } else {
            kind = newt_c2p(a.gm - 1.0, u, P, bad);
        }
        ++st.zones;
        st.it64 += (unsigned)iters;
        if (kind != HYDRO_NONE && kind != HYDRO_NEGATIVE_PRESSURE) {
            atomicMin(&a.status->err_key, error_key(a.stage, slot, i, j, kind));
            a.status->err_sel = a.sel_in;
        }
        const double w = a.srhd ? sqrt(1.0 + P[1] * P[1] + P[2] * P[2]) : 1.0;
        double v[NFIELD] = {P[0], P[1], P[2], P[3], smass / dV / w};
        store_prim<double>(B, i, j, v);
        if (a.compute_dt) {
            PhysT<double> ph;
            ph.srhd = a.srhd;
            ph.hllc = a.hllc;
            ph.gm = a.gm;
            ph.gm1 = a.gm - 1.0;
            ph.gh = a.gm / ph.gm1;
            ph.theta = a.plm_theta;
            const double dr = B.rv[i + 1] - B.rv[i];
            const double dq = B.qv[j + 1] - B.qv[j];
            const double dl = fmin(dr, dq * B.rv[i]);
            const double amax = max_signal_speed(ph, P) * a.cflux;
            st.dtz = fmin(st.dtz, dl / amax);
        }
    }
};

template <bool MLP>
__global__ void __launch_bounds__(TILE_THREADS) c2p_f64_kernel(StageArgs a) {
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
        F64C2p<MLP>::zone(a, t.x, B, i, j, i < B.nr && j < B.nq, W, act, st);
    }
    warp_reduce_stats(a.status, st.zones, st.it64, 0ull, st.fbs, st.dtz, a.compute_dt != 0);
}

// ---- the fused stage (FP64) ----------------------------------------------------
template <int TR, bool MLP>
__global__ void __launch_bounds__(update_threads<TR>(), TR == 16 ? 1 : 2) stage_fused_f64_kernel(StageArgs a, GhostArgs g,
                                                                                  FusedArgs f) {
    stage_fused_body<double, false, TR, F64C2p<MLP>>(a, g, f);
}

cudaError_t launch_remap_f64(const StageArgs& a, const int4* remap, int nremap, int max_nq, cudaStream_t s) {
    if (nremap <= 0) return cudaSuccess;
    dim3 grid((2 * max_nq + 127) / 128, nremap);
    remap_kernel<double><<<grid, 128, 0, s>>>(a, remap);
    return cudaGetLastError();
}

// ---- initial data -------------------------------------------------------------
__global__ void __launch_bounds__(TILE_THREADS) init_kernel(InitArgs a) {
    const int4 t = a.tiles[blockIdx.x];
    const DevBlock& B = a.blocks[t.x];
    const int i = t.y + threadIdx.x / TILE_Q;
    const int j = t.z + threadIdx.x % TILE_Q;
    const int nr = B.nr, nq = B.nq;
    if (i >= nr || j >= nq) return;
    const int64_t n = (int64_t)nr * nq;
    const int64_t z = (int64_t)i * nq + j;
    double Pm[4];
    double scalar;
    if (a.host_prim) {
        // host-model values, one row of 5 per zone, blocks in slot order
        const double* hp = a.host_prim + ((int64_t)t.w + z) * 5;
        Pm[0] = hp[0];
        Pm[1] = hp[1];
        Pm[2] = hp[2];
        Pm[3] = hp[3];
        scalar = hp[4];
    } else {
        model_eval(a.model, B.rc[i], B.qc[j], a.time, a.noise != 0, B.index, i, j, Pm, scalar);
    }
    PhysT<double> ph;
    ph.srhd = a.srhd;
    ph.hllc = 0;
    ph.gm = a.gm;
    ph.gm1 = a.gm - 1.0;
    ph.gh = a.gm / ph.gm1;
    ph.theta = 1.0;
    double U[4];
    prim_to_cons(ph, Pm, U);
    const double dV = B.dv[z];
    double* out = B.buf[a.sel];
    double d0 = 0.0;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const double v = U[c] * dV;
        out[c * n + z] = v;
        if (c == 0) d0 = v;
    }
    out[4 * n + z] = d0 * scalar;
}

// ---- layout transposes ---------------------------------------------------------
__global__ void aos_to_soa_kernel(const double* __restrict__ aos, const double* __restrict__ scalar,
                                  double* __restrict__ soa, int64_t n) {
    const int64_t z = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= n) return;
    const double4 v = reinterpret_cast<const double4*>(aos)[z];
    soa[z] = v.x;
    soa[n + z] = v.y;
    soa[2 * n + z] = v.z;
    soa[3 * n + z] = v.w;
    soa[4 * n + z] = scalar[z];
}

__global__ void soa_to_aos_kernel(const double* __restrict__ soa, double* __restrict__ aos,
                                  double* __restrict__ scalar, int64_t n) {
    const int64_t z = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= n) return;
    double4 v;
    v.x = soa[z];
    v.y = soa[n + z];
    v.z = soa[2 * n + z];
    v.w = soa[3 * n + z];
    reinterpret_cast<double4*>(aos)[z] = v;
    scalar[z] = soa[4 * n + z];
}

// The whole state <-> the ABI's arrays (blocks in slot order, each
// [nr][nq][4] then [nr][nq] scalar mass), one launch over the recovery tiles
// (t.w = the block's first zone in the whole-state arrays). The host arrays
// may be page-locked host memory read or written directly over the
// CPU-GPU link, or a device staging copy. A shadow block's rows go into both
// of its state buffers: rows its later stages do not update then still hold
// a state that recovers as the first stage's did.
__global__ void __launch_bounds__(TILE_THREADS) state_in_kernel(const DevBlock* __restrict__ blocks,
                                                               const int4* __restrict__ tiles, int sel,
                                                               const double* __restrict__ cons,
                                                               const double* __restrict__ scalar) {
    const int4 t = tiles[blockIdx.x];
    const DevBlock& B = blocks[t.x];
    const int i = t.y + threadIdx.x / TILE_Q, j = t.z + threadIdx.x % TILE_Q;
    if (i >= B.nr || j >= B.nq) return;
    const int64_t n = (int64_t)B.nr * B.nq, z = (int64_t)i * B.nq + j, g = (int64_t)t.w + z;
    const double2 a = reinterpret_cast<const double2*>(cons)[2 * g];
    const double2 b = reinterpret_cast<const double2*>(cons)[2 * g + 1];
    const double sm = scalar[g];
    for (int k = 0; k <= B.shadow; ++k) {
        double* U = B.buf[sel ^ k];
        U[z] = a.x;
        U[n + z] = a.y;
        U[2 * n + z] = b.x;
        U[3 * n + z] = b.y;
        U[4 * n + z] = sm;
    }
}

__global__ void __launch_bounds__(TILE_THREADS) state_out_kernel(const DevBlock* __restrict__ blocks,
                                                                const int4* __restrict__ tiles, int sel,
                                                                double* __restrict__ cons,
                                                                double* __restrict__ scalar) {
    const int4 t = tiles[blockIdx.x];
    const DevBlock& B = blocks[t.x];
    const int i = t.y + threadIdx.x / TILE_Q, j = t.z + threadIdx.x % TILE_Q;
    if (i >= B.nr || j >= B.nq) return;
    const int64_t n = (int64_t)B.nr * B.nq, z = (int64_t)i * B.nq + j, g = (int64_t)t.w + z;
    const double* U = B.buf[sel];
    reinterpret_cast<double2*>(cons)[2 * g] = make_double2(U[z], U[n + z]);
    reinterpret_cast<double2*>(cons)[2 * g + 1] = make_double2(U[2 * n + z], U[3 * n + z]);
    scalar[g] = U[4 * n + z];
}

// Interior rows of a padded double primitive array -> [nr][nq][5], with the
// scalar density divided by rho into a concentration.
__global__ void prims_to_aos_kernel(const double* __restrict__ P, double* __restrict__ out, int64_t nr,
                                    int64_t nq) {
    const int64_t z = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (z >= nr * nq) return;
    const int64_t pn = (nr + 4) * nq;
    const int64_t off = 2 * nq + z;
    double v[5];
    for (int q = 0; q < 5; ++q) v[q] = P[q * pn + off];
    v[4] = v[4] / v[0];
    for (int q = 0; q < 5; ++q) out[z * 5 + q] = v[q];
}

// BlockProducts of a block: the recovered (double) primitives of the padded
// array in AnyPrimitive order, and scalar_mass / lab_frame_mass from the
// volume-integrated state U (src/products.rs:50-58).
__global__ void products_kernel(const double* __restrict__ P, const double* __restrict__ U,
                                double* __restrict__ prim, double* __restrict__ scalar, int64_t nr, int64_t nq) {
    const int64_t z = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = nr * nq;
    if (z >= n) return;
    const int64_t pn = (nr + 4) * nq;
    const int64_t off = 2 * nq + z;
    prim[z * 4 + 0] = P[pn + off];       // velocity_r
    prim[z * 4 + 1] = P[2 * pn + off];   // velocity_q
    prim[z * 4 + 2] = P[off];            // mass_density
    prim[z * 4 + 3] = P[3 * pn + off];   // gas_pressure
    scalar[z] = U[4 * n + z] / U[z];
}

// ---- launchers ---------------------------------------------------------------
cudaError_t launch_products(const void* P, const double* U, double* prim, double* scalar, int64_t nr, int64_t nq,
                            cudaStream_t s) {
    const int64_t n = nr * nq;
    products_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(reinterpret_cast<const double*>(P), U, prim, scalar,
                                                                  nr, nq);
    return cudaGetLastError();
}

cudaError_t launch_prims_to_aos(const void* P, double* out, int64_t nr, int64_t nq, cudaStream_t s) {
    const int64_t n = nr * nq;
    prims_to_aos_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(reinterpret_cast<const double*>(P), out, nr, nq);
    return cudaGetLastError();
}

cudaError_t launch_c2p_f64(const StageArgs& a, cudaStream_t s) {
    if (a.ntiles <= 0) return cudaSuccess;
    if (a.mlp && a.srhd) {
        const size_t bytes = sizeof(MlpWeights) + 8 * MLP_ACT_ELEMS * sizeof(__nv_bfloat16);
        int dev = 0, sms = 1, per_sm = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        // resident CTAs only: a persistent grid larger than that runs a tail wave
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, c2p_f64_kernel<true>, TILE_THREADS, bytes) !=
                cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        const int grid = a.ntiles < sms * per_sm ? a.ntiles : sms * per_sm;
        c2p_f64_kernel<true><<<grid, TILE_THREADS, bytes, s>>>(a);
    } else {
        c2p_f64_kernel<false><<<a.ntiles, TILE_THREADS, 0, s>>>(a);
    }
    return cudaGetLastError();
}

template <int TR>
static void update_f64(const StageArgs& a, cudaStream_t s) {
    update_kernel<double, false, TR><<<a.nutiles, update_threads<TR>(), StageSmem<double, TR>::bytes, s>>>(a);
}

cudaError_t launch_update_f64(const StageArgs& a, cudaStream_t s) {
    if (a.strips) {
        if (a.nstrips <= 0) return cudaSuccess;
        update_strip_kernel<double, false, 2><<<(a.nstrips + STRIP_WARPS - 1) / STRIP_WARPS, STRIP_WARPS * 32, 0, s>>>(a);
        return cudaGetLastError();
    }
    if (a.nutiles <= 0) return cudaSuccess;
    switch (a.utr) {
    case 4: update_f64<4>(a, s); break;
    case 16: update_f64<16>(a, s); break;
    default: update_f64<8>(a, s);
    }
    return cudaGetLastError();
}

template <int TR, bool MLP>
static cudaError_t fused_f64(const StageArgs& a, const GhostArgs& g, const FusedArgs& f, int grid, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(update_threads<TR>());
    cfg.dynamicSmemBytes = fused_smem_bytes<double, TR, MLP>();
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, stage_fused_f64_kernel<TR, MLP>, a, g, f);
}

cudaError_t launch_stage_fused_f64(const StageArgs& a, const GhostArgs& g, const FusedArgs& f, int grid,
                                   cudaStream_t s) {
    const bool mlp = a.mlp && a.srhd;
    switch (fused_tr(a.utr)) {
    case 4: return mlp ? fused_f64<4, true>(a, g, f, grid, s) : fused_f64<4, false>(a, g, f, grid, s);
    case 16: return mlp ? fused_f64<16, true>(a, g, f, grid, s) : fused_f64<16, false>(a, g, f, grid, s);
    default: return mlp ? fused_f64<8, true>(a, g, f, grid, s) : fused_f64<8, false>(a, g, f, grid, s);
    }
}

template <int TR, bool MLP>
static cudaError_t fused_ctas_f64(int* n) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(n, stage_fused_f64_kernel<TR, MLP>, update_threads<TR>(),
                                                         fused_smem_bytes<double, TR, MLP>());
}

cudaError_t fused_max_ctas_f64(bool mlp, int utr, int* n) {
    switch (fused_tr(utr)) {
    case 4: return mlp ? fused_ctas_f64<4, true>(n) : fused_ctas_f64<4, false>(n);
    case 16: return mlp ? fused_ctas_f64<16, true>(n) : fused_ctas_f64<16, false>(n);
    default: return mlp ? fused_ctas_f64<8, true>(n) : fused_ctas_f64<8, false>(n);
    }
}

template <int TR, bool MLP>
static cudaError_t configure_fused_f64() {
    return cudaFuncSetAttribute(stage_fused_f64_kernel<TR, MLP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)fused_smem_bytes<double, TR, MLP>());
}

template <int TR>
static cudaError_t configure_update_f64() {
    return cudaFuncSetAttribute(update_kernel<double, false, TR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)StageSmem<double, TR>::bytes);
}

cudaError_t configure_f64() {
    cudaError_t e = configure_update_f64<4>();
    if (e == cudaSuccess) e = configure_update_f64<8>();
    if (e == cudaSuccess) e = configure_update_f64<16>();
    if (e == cudaSuccess) e = configure_fused_f64<4, false>();
    if (e == cudaSuccess) e = configure_fused_f64<8, false>();
    if (e == cudaSuccess) e = configure_fused_f64<16, false>();
    if (e == cudaSuccess) e = configure_fused_f64<4, true>();
    if (e == cudaSuccess) e = configure_fused_f64<8, true>();
    if (e == cudaSuccess) e = configure_fused_f64<16, true>();
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(c2p_f64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(sizeof(MlpWeights) + 8 * MLP_ACT_ELEMS * sizeof(__nv_bfloat16)));
}

cudaError_t launch_ghost_f64(const GhostArgs& a, cudaStream_t s) {
    const int nq = a.nq[0] > a.nq[1] ? a.nq[0] : a.nq[1];
    dim3 grid((2 * nq + 127) / 128, 2);
    ghost_kernel<<<grid, 128, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_init_f64(const InitArgs& a, int ntiles, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    init_kernel<<<ntiles, TILE_THREADS, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_aos_to_soa(const double* aos, const double* scalar, double* soa, int64_t nr, int64_t nq,
                              cudaStream_t s) {
    const int64_t n = nr * nq;
    aos_to_soa_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(aos, scalar, soa, n);
    return cudaGetLastError();
}

cudaError_t launch_state_in(const DevBlock* blocks, const int4* tiles, int ntiles, int sel, const double* cons,
                            const double* scalar, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    state_in_kernel<<<ntiles, TILE_THREADS, 0, s>>>(blocks, tiles, sel, cons, scalar);
    return cudaGetLastError();
}

cudaError_t launch_state_out(const DevBlock* blocks, const int4* tiles, int ntiles, int sel, double* cons,
                             double* scalar, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    state_out_kernel<<<ntiles, TILE_THREADS, 0, s>>>(blocks, tiles, sel, cons, scalar);
    return cudaGetLastError();
}

// Two ghost rows of the five primitive fields, computed ahead into a compact
// [5][2][nq] array, into rows row0, row0 + 1 of a block's padded
// [5][nr + 4][nq] primitives; copied as 32-bit words (fields of 4 or 8 bytes).
__global__ void halo_rows_kernel(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int64_t words,
                                 int64_t dst_field_words, int64_t dst_off_words) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int f = blockIdx.y;
    if (k >= words) return;
    dst[f * dst_field_words + dst_off_words + k] = src[f * words + k];
}

cudaError_t launch_halo_rows(const void* src, void* dst, int nq, int nr, int row0, int elem_bytes, cudaStream_t s) {
    const int64_t wq = (int64_t)nq * elem_bytes / 4;   // words per row
    const int64_t words = 2 * wq;
    dim3 grid((unsigned)((words + 255) / 256), NFIELD);
    halo_rows_kernel<<<grid, 256, 0, s>>>(reinterpret_cast<const uint32_t*>(src), reinterpret_cast<uint32_t*>(dst),
                                          words, (int64_t)(nr + 4) * wq, (int64_t)row0 * wq);
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(const double* soa, double* aos, double* scalar, int64_t nr, int64_t nq,
                              cudaStream_t s) {
    const int64_t n = nr * nq;
    soa_to_aos_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(soa, aos, scalar, n);
    return cudaGetLastError();
}

}  // namespace knc
