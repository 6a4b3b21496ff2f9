// knc_mlp.cu — training data and training kernels of the learned c2p guess.
//
// Pairs are rows of 8 doubles (D, S_r, S_theta, tau, rho, u_r, u_theta, p) per
// unit volume. They come from the solver itself: sampled from a live state
// (knc_sample_pairs, recovered with the FP64 Newton of the stage) or produced
// by the solver's prim -> cons over a range of Lorentz factors and
// temperatures (knc_generate_pairs).
//
// Training: each step draws a batch and evaluates the loss gradient with one
// launch of mlp_train_tc_kernel: the forward pass rounds weights and
// activations to bf16 as inference does, and the back-propagation is FP32
// (straight-through for those roundings), with its three dense contractions on
// the fifth-generation tensor cores (tcgen05.mma, accumulators in tensor
// memory). Adam then updates the FP32 master weights.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "knc_internal.h"
#include "knc_mlp.cuh"
#include "knc_physics.cuh"
#include "knc_tc.cuh"
#include "knc_tma.cuh"

namespace knc {

// ---- training kernel: one CTA of 128 threads per SM, a tile of 128 batch
// rows at a time, thread t owning row t. The three 128 x 64 x K contractions
// run on the tensor cores (tcgen05.mma, bf16 operands in shared memory, FP32
// accumulators in tensor memory):
//   Z2  = A1 . W2^T                    (K = 64 hidden units)
//   dA1 = dZ2 . W2                     (K = 64)
//   dW2 += [dZ2_hi; dZ2_lo]^T . A1     (K = 128 rows, accumulated over tiles)
// A1 = bf16(silu(z1)) and W2 are bf16 already (the forward pass uses them so);
// dZ2 is FP32 and enters as the sum of two bf16 parts, hi = bf16(dZ2) and
// lo = bf16(dZ2 - hi), which carries 16 of its 24 significand bits. The
// per-unit sums (b1, W1, b2, W3, b3) are warp-shuffle reductions in FP32.
constexpr int TC_ROWS = 128;                       // batch rows per tile = MMA M
constexpr int TC_THREADS = 128;
constexpr uint32_t TC_TMEM_COLS = 256;             // Z2 at 0, dA1 at 64, dW2 at 128
constexpr uint32_t TC_KLBO = 128, TC_KSBO = 1024;  // [rows][64] tiles: 8 K-chunks of 128 B per 8-row group
constexpr uint32_t TC_TLBO = 144, TC_TSBO = 16 * 144;   // [n][128 rows] tiles: K-chunks 144 B apart
constexpr uint32_t TC_IDESC = tc_idesc_bf16(128, 64);
constexpr int TC_WAIT_POLLS = 1 << 22;

struct TcTrainSmem {
    unsigned char a1k[TC_ROWS * 64 * 2];      // A1 (M = row, K = unit)
    unsigned char dzk[2][TC_ROWS * 64 * 2];   // dZ2 hi, lo (M = row, K = unit)
    unsigned char w2k[64 * 64 * 2];           // W2 (N = output unit u, K = input unit v)
    unsigned char w2t[64 * 64 * 2];           // W2^T (N = v, K = u)
    unsigned char a1t[8 * TC_TSBO];           // A1^T (N = v, K = row)
    unsigned char dzt[16 * TC_TSBO];          // [dZ2 hi; dZ2 lo]^T (M = 128: u, then 64 + u; K = row)
    float w1[MLP_H * 3], b1[MLP_H], b2[MLP_H], w3[MLP_H];
    float b3, xm[3], xs[3];
    uint64_t bar[2];
    uint32_t tmem_slot;
};

// Byte offsets in the two operand layouts.
__device__ __forceinline__ uint32_t kbyte(int row, int k) {
    return (uint32_t)(row >> 3) * TC_KSBO + (uint32_t)(k >> 3) * TC_KLBO + (uint32_t)(row & 7) * 16u +
           (uint32_t)(k & 7) * 2u;
}
__device__ __forceinline__ uint32_t tbyte(int n, int row) {
    return (uint32_t)(n >> 3) * TC_TSBO + (uint32_t)(row >> 3) * TC_TLBO + (uint32_t)(n & 7) * 16u +
           (uint32_t)(row & 7) * 2u;
}

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + expf(-z)); }

__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, __nv_bfloat16 v) {
    *reinterpret_cast<__nv_bfloat16*>(base + off) = v;
}

// Sum over the warp's 32 rows of 32 per-row values: a butterfly that halves
// the set at each of 5 exchanges; lane l ends with the sum of column l.
__device__ __forceinline__ float warp_colsum32(float (&v)[32]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int m = 16, h = 16; m > 0; m >>= 1, h >>= 1) {
        const bool up = (lane & m) != 0;
#pragma unroll
        for (int k = 0; k < h; ++k) {
            const float send = up ? v[k] : v[k + h];
            const float keep = up ? v[k + h] : v[k];
            v[k] = keep + __shfl_xor_sync(0xffffffffu, send, m);
        }
    }
    return v[0];
}

// One launch = one gradient evaluation over `rows` rows. Row r reads data row
// (seed ? hash(seed, r) % n_data : r). Gradients (of the mean loss) are added
// into grad[]; the summed squared error into *loss_sum. A tensor-core wait
// that gives up sets *err.
__global__ void __launch_bounds__(TC_THREADS, 1) mlp_train_tc_kernel(const float* __restrict__ w,
                                                                    const float* __restrict__ x,
                                                                    const float* __restrict__ y, int64_t n_data,
                                                                    int64_t rows, uint64_t seed, float inv_batch,
                                                                    float* __restrict__ grad,
                                                                    float* __restrict__ loss_sum,
                                                                    float* __restrict__ pred, unsigned* err) {
    extern __shared__ unsigned char smem_raw[];
    TcTrainSmem& S =
        *reinterpret_cast<TcTrainSmem*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    for (int k = tid; k < MLP_H * MLP_H; k += TC_THREADS) {
        const int u = k >> 6, v = k & 63;
        const __nv_bfloat16 b = __float2bfloat16_rn(w[KNC_MLP_OFF_W2 + k]);
        st_bf16(S.w2k, kbyte(u, v), b);
        st_bf16(S.w2t, kbyte(v, u), b);
    }
    for (int k = tid; k < MLP_H * 3; k += TC_THREADS) S.w1[k] = bf16r(w[KNC_MLP_OFF_W1 + k]);
    for (int k = tid; k < MLP_H; k += TC_THREADS) {
        S.b1[k] = w[KNC_MLP_OFF_B1 + k];
        S.b2[k] = w[KNC_MLP_OFF_B2 + k];
        S.w3[k] = bf16r(w[KNC_MLP_OFF_W3 + k]);
    }
    if (tid == 0) {
        S.b3 = w[KNC_MLP_OFF_B3];
        for (int k = 0; k < 3; ++k) {
            S.xm[k] = w[KNC_MLP_OFF_XMEAN + k];
            S.xs[k] = w[KNC_MLP_OFF_XSCALE + k];
        }
        mbar_init(&S.bar[0], 1);
        mbar_init(&S.bar[1], 1);
        fence_barrier_init();
    }
    if (warp == 0) tc_alloc(smem_u32(&S.tmem_slot), TC_TMEM_COLS);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem_slot;
    const uint32_t a1k = smem_u32(S.a1k), w2k = smem_u32(S.w2k), w2t = smem_u32(S.w2t);
    const uint32_t dzk0 = smem_u32(S.dzk[0]), dzk1 = smem_u32(S.dzk[1]);
    const uint32_t a1t = smem_u32(S.a1t), dzt = smem_u32(S.dzt);

    // lane sums of columns lane and 32 + lane: W3, b2, b1, W1 (3)
    float g_w3[2] = {0.f, 0.f}, g_b2[2] = {0.f, 0.f}, g_b1[2] = {0.f, 0.f};
    float g_w1[3][2] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    float g_b3 = 0.f, l_sum = 0.f;
    uint32_t phase = 0;
    bool any_tile = false, failed = false;

    const int64_t ntiles = (rows + TC_ROWS - 1) / TC_ROWS;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t r = t * TC_ROWS + tid;
        const bool valid = r < rows;
        int64_t d = r;
        if (seed) d = (int64_t)(splitmix64(seed ^ splitmix64((uint64_t)r)) % (uint64_t)n_data);
        float xr0 = 0.f, xr1 = 0.f, xr2 = 0.f, yr = 0.f;
        if (valid) {
            xr0 = x[d * 3];
            xr1 = x[d * 3 + 1];
            xr2 = x[d * 3 + 2];
            yr = y[d];
        }
        const float xn0 = (xr0 - S.xm[0]) * S.xs[0];
        const float xn1 = (xr1 - S.xm[1]) * S.xs[1];
        const float xn2 = (xr2 - S.xm[2]) * S.xs[2];
        auto z1_of = [&](int v) {
            return __fmaf_rn(S.w1[v * 3 + 2], xn2, __fmaf_rn(S.w1[v * 3 + 1], xn1, __fmaf_rn(S.w1[v * 3], xn0, S.b1[v])));
        };
        // ---- layer 1: A1 row (K-major) and column (transposed tile)
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            uint32_t pk[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const int v = 8 * c + 2 * h;
                const float za = z1_of(v), zb = z1_of(v + 1);
                const __nv_bfloat16 ba = __float2bfloat16_rn(za / (1.0f + expf(-za)));
                const __nv_bfloat16 bb = __float2bfloat16_rn(zb / (1.0f + expf(-zb)));
                st_bf16(S.a1t, tbyte(v, tid), ba);
                st_bf16(S.a1t, tbyte(v + 1, tid), bb);
                __nv_bfloat162 p2;
                p2.x = ba;
                p2.y = bb;
                pk[h] = *reinterpret_cast<const uint32_t*>(&p2);
            }
            *reinterpret_cast<uint4*>(S.a1k + kbyte(tid, 8 * c)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
                tc_mma_bf16(tmem, tc_desc(a1k + 256u * ks, TC_KLBO, TC_KSBO), tc_desc(w2k + 256u * ks, TC_KLBO, TC_KSBO),
                            TC_IDESC, ks > 0);
            tc_commit(smem_u32(&S.bar[0]));
        }
        if (__syncthreads_or(!mbar_wait_bounded(&S.bar[0], phase, TC_WAIT_POLLS))) {
            failed = true;
            break;
        }
        tc_fence_after();
        // ---- layer 2 and the output
        float z2[64], s2[64];
        tc_ld64(tmem, 0, z2);
        float out = S.b3;
#pragma unroll
        for (int u = 0; u < 64; ++u) {
            z2[u] += S.b2[u];
            s2[u] = sigm(z2[u]);
            out = fmaf(z2[u] * s2[u], S.w3[u], out);
        }
        if (pred && valid && !seed) pred[r] = out;
        const float e = valid ? out - yr : 0.f;
        l_sum += e * e;
        const float dout = 2.0f * e * inv_batch;
        g_b3 += dout;
        // W3: dout h2 summed over rows
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            float q[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) q[k] = dout * (z2[32 * hh + k] * s2[32 * hh + k]);
            g_w3[hh] += warp_colsum32(q);
        }
        // dZ2 in place of z2
#pragma unroll
        for (int u = 0; u < 64; ++u) {
            const float s = s2[u];
            z2[u] = dout * S.w3[u] * s * (1.0f + z2[u] * (1.0f - s));
        }
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            float q[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) q[k] = z2[32 * hh + k];
            g_b2[hh] += warp_colsum32(q);
        }
        // dZ2 = hi + lo into the row tiles (dA1) and the stacked transposed tile (dW2)
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            uint32_t ph[4], pl[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const int u = 8 * c + 2 * h;
                const __nv_bfloat16 ha = __float2bfloat16_rn(z2[u]), hb = __float2bfloat16_rn(z2[u + 1]);
                const __nv_bfloat16 la = __float2bfloat16_rn(z2[u] - __bfloat162float(ha));
                const __nv_bfloat16 lb = __float2bfloat16_rn(z2[u + 1] - __bfloat162float(hb));
                st_bf16(S.dzt, tbyte(u, tid), ha);
                st_bf16(S.dzt, tbyte(u + 1, tid), hb);
                st_bf16(S.dzt, tbyte(64 + u, tid), la);
                st_bf16(S.dzt, tbyte(64 + u + 1, tid), lb);
                __nv_bfloat162 p2;
                p2.x = ha;
                p2.y = hb;
                ph[h] = *reinterpret_cast<const uint32_t*>(&p2);
                p2.x = la;
                p2.y = lb;
                pl[h] = *reinterpret_cast<const uint32_t*>(&p2);
            }
            *reinterpret_cast<uint4*>(S.dzk[0] + kbyte(tid, 8 * c)) = make_uint4(ph[0], ph[1], ph[2], ph[3]);
            *reinterpret_cast<uint4*>(S.dzk[1] + kbyte(tid, 8 * c)) = make_uint4(pl[0], pl[1], pl[2], pl[3]);
        }
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
                tc_mma_bf16(tmem + 64u, tc_desc(dzk0 + 256u * ks, TC_KLBO, TC_KSBO),
                            tc_desc(w2t + 256u * ks, TC_KLBO, TC_KSBO), TC_IDESC, ks > 0);
#pragma unroll
            for (int ks = 0; ks < 4; ++ks)
                tc_mma_bf16(tmem + 64u, tc_desc(dzk1 + 256u * ks, TC_KLBO, TC_KSBO),
                            tc_desc(w2t + 256u * ks, TC_KLBO, TC_KSBO), TC_IDESC, 1u);
#pragma unroll
            for (int ks = 0; ks < 8; ++ks)
                tc_mma_bf16(tmem + 128u, tc_desc(dzt + 2u * TC_TLBO * ks, TC_TLBO, TC_TSBO),
                            tc_desc(a1t + 2u * TC_TLBO * ks, TC_TLBO, TC_TSBO), TC_IDESC, (any_tile || ks > 0) ? 1u : 0u);
            tc_commit(smem_u32(&S.bar[1]));
        }
        any_tile = true;
        if (__syncthreads_or(!mbar_wait_bounded(&S.bar[1], phase, TC_WAIT_POLLS))) {
            failed = true;
            break;
        }
        tc_fence_after();
        phase ^= 1u;
        // ---- layer 1 backward: dz1 = dA1 silu'(z1), in place of dA1
        float da[64];
        tc_ld64(tmem, 64, da);
#pragma unroll
        for (int v = 0; v < 64; ++v) {
            const float z = z1_of(v);
            const float s = sigm(z);
            da[v] = da[v] * s * (1.0f + z * (1.0f - s));
        }
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            float q[32];
#pragma unroll
            for (int k = 0; k < 32; ++k) q[k] = da[32 * hh + k];
            g_b1[hh] += warp_colsum32(q);
#pragma unroll
            for (int k = 0; k < 32; ++k) q[k] = da[32 * hh + k] * xn0;
            g_w1[0][hh] += warp_colsum32(q);
#pragma unroll
            for (int k = 0; k < 32; ++k) q[k] = da[32 * hh + k] * xn1;
            g_w1[1][hh] += warp_colsum32(q);
#pragma unroll
            for (int k = 0; k < 32; ++k) q[k] = da[32 * hh + k] * xn2;
            g_w1[2][hh] += warp_colsum32(q);
        }
        tc_fence_before();
    }
    if (failed) {
        if (tid == 0) atomicExch(err, 1u);
        // the tensor core's work in flight, if any, gets one more bounded wait
        mbar_wait_bounded(&S.bar[0], phase, TC_WAIT_POLLS);
        mbar_wait_bounded(&S.bar[1], phase, TC_WAIT_POLLS);
    } else if (any_tile) {
        // ---- dW2: accumulator rows u (hi part) and 64 + u (lo part), summed
        float acc[64];
        tc_ld64(tmem, 128, acc);
        __syncthreads();   // every MMA has completed; the row tiles are free
        float* red = reinterpret_cast<float*>(S.a1k);   // [128][65] floats over a1k and dzk
#pragma unroll
        for (int v = 0; v < 64; ++v) red[tid * 65 + v] = acc[v];
        __syncthreads();
        for (int k = tid; k < MLP_H * MLP_H; k += TC_THREADS) {
            const int u = k >> 6, v = k & 63;
            atomicAdd(&grad[KNC_MLP_OFF_W2 + k], red[u * 65 + v] + red[(64 + u) * 65 + v]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            g_b3 += __shfl_xor_sync(0xffffffffu, g_b3, o);
            l_sum += __shfl_xor_sync(0xffffffffu, l_sum, o);
        }
        if (lane == 0) {
            atomicAdd(&grad[KNC_MLP_OFF_B3], g_b3);
            atomicAdd(loss_sum, l_sum);
        }
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            const int u = 32 * hh + lane;
            atomicAdd(&grad[KNC_MLP_OFF_W3 + u], g_w3[hh]);
            atomicAdd(&grad[KNC_MLP_OFF_B2 + u], g_b2[hh]);
            atomicAdd(&grad[KNC_MLP_OFF_B1 + u], g_b1[hh]);
            for (int k = 0; k < 3; ++k) atomicAdd(&grad[KNC_MLP_OFF_W1 + u * 3 + k], g_w1[k][hh]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tc_dealloc(tmem, TC_TMEM_COLS);
    }
}

__global__ void adam_kernel(float* w, float* m, float* v, float* g, int n, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float gk = g[k];
    g[k] = 0.f;
    if (k >= KNC_MLP_OFF_XMEAN) return;   // input normalisation is fixed
    const float mk = b1 * m[k] + (1.f - b1) * gk;
    const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    w[k] -= lr * (mk * c1) / (sqrtf(vk * c2) + eps);
}

// Features and target of each pair, in FP32 exactly as the c2p kernels form them.
__global__ void features_kernel(const double* __restrict__ pairs, int64_t n, float* __restrict__ x,
                                float* __restrict__ y) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double* r = pairs + k * 8;
    float f[3];
    mlp_features(r[0], r[1] * r[1] + r[2] * r[2], r[3], f);
    x[k * 3] = f[0];
    x[k * 3 + 1] = f[1];
    x[k * 3 + 2] = f[2];
    y[k] = (float)log(r[7] / r[0]);
}

__global__ void generate_pairs_kernel(double gm, double lw0, double lw1, double lt0, double lt1, uint64_t seed,
                                      int64_t n, double* __restrict__ out) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double u1 = uniform01(seed, 1, k, 0), u2 = uniform01(seed, 2, k, 0);
    const double u3 = uniform01(seed, 3, k, 0), u4 = uniform01(seed, 4, k, 0);
    const double W = exp(lw0 + u1 * (lw1 - lw0));
    const double T = exp(lt0 + u2 * (lt1 - lt0));
    const double rho = exp(log(1e-3) + u3 * log(1e6));
    const double ang = 2.0 * PI * u4;
    const double um = sqrt(fmax(W * W - 1.0, 0.0));
    double P[4] = {rho, um * cos(ang), um * sin(ang), T * rho};
    PhysT<double> ph;
    ph.srhd = 1;
    ph.hllc = 0;
    ph.gm = gm;
    ph.gm1 = gm - 1.0;
    ph.gh = gm / ph.gm1;
    ph.theta = 1.0;
    double U[4];
    prim_to_cons(ph, P, U);
    double* o = out + k * 8;
    for (int q = 0; q < 4; ++q) {
        o[q] = U[q];
        o[4 + q] = P[q];
    }
}

// Pairs from a live state: every `stride`-th zone (global zone order), its
// per-volume conserved state and the FP64 Newton recovery of it.
__global__ void __launch_bounds__(TILE_THREADS) sample_pairs_kernel(const DevBlock* blocks, const int4* tiles,
                                                                    int ntiles, int sel, int stride, double gm,
                                                                    double* out, int64_t capacity,
                                                                    unsigned long long* counter) {
    const int4 t = tiles[blockIdx.x];
    const DevBlock& B = blocks[t.x];
    const int i = t.y + threadIdx.x / TILE_Q;
    const int j = t.z + threadIdx.x % TILE_Q;
    if (i >= B.nr || j >= B.nq) return;
    const int64_t z = (int64_t)i * B.nq + j;
    if (((int64_t)t.w + z) % stride != 0) return;
    const int64_t n = (int64_t)B.nr * B.nq;
    const double* U = B.buf[sel];
    const double dV = B.dv[z];
    double u[4];
    for (int q = 0; q < 4; ++q) u[q] = U[q * n + z] / dV;
    double P[4];
    double bad;
    int it;
    const int kind = srhd_c2p_newton(gm, u, 0.0, P, it, bad);
    if (kind != HYDRO_NONE) return;
    const unsigned long long slot = atomicAdd(counter, 1ull);
    if ((int64_t)slot >= capacity) return;
    double* o = out + slot * 8;
    for (int q = 0; q < 4; ++q) {
        o[q] = u[q];
        o[4 + q] = P[q];
    }
}

cudaError_t launch_sample_pairs(const DevBlock* blocks, const int4* tiles, int ntiles, int sel, int stride, double gm,
                                double* out, int64_t capacity, unsigned long long* counter, cudaStream_t s) {
    if (ntiles <= 0) return cudaSuccess;
    sample_pairs_kernel<<<ntiles, TILE_THREADS, 0, s>>>(blocks, tiles, ntiles, sel, stride, gm, out, capacity,
                                                        counter);
    return cudaGetLastError();
}

namespace {

size_t train_smem_bytes() { return sizeof(TcTrainSmem) + 1024; }   // + alignment of the operand tiles

// The training kernel's shared memory, on the current device (every call:
// the library may serve several devices).
cudaError_t configure_train() {
    return cudaFuncSetAttribute(mlp_train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)train_smem_bytes());
}

// One CTA per 128-row tile up to one per SM (the kernel's shared memory
// admits one CTA per SM, so its tensor-memory allocation never waits).
int grid_for_rows(int64_t rows) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t tiles = (rows + TC_ROWS - 1) / TC_ROWS;
    return (int)std::max<int64_t>(1, std::min<int64_t>(sms, tiles));
}

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};

#define CKR(call)                                      \
    do {                                               \
        if ((call) != cudaSuccess) return KNC_ERR_CUDA; \
    } while (0)

}  // namespace
}  // namespace knc

using namespace knc;

extern "C" {

size_t knc_mlp_num_params(void) { return KNC_MLP_NUM_PARAMS; }

void knc_mlp_features(const double u[4], float out[3]) {
    const double d = u[0], ss = u[1] * u[1] + u[2] * u[2], tau = u[3];
    const double e = tau + d;
    const double a = tau * (tau + 2.0 * d) - ss;
    if (!(d > 0.0) || !(tau > 0.0) || !(a > 0.0)) {
        out[0] = out[1] = out[2] = 0.f;
        return;
    }
    const float df = (float)d, ef = (float)e;
    const float xs = std::sqrt((float)ss) / ef;
    out[0] = std::log((float)tau / df);
    out[1] = std::log(1.0f + xs) - std::log((float)(a + d * d) / (ef * ef));
    out[2] = std::log((float)a / (df * df));
}

int knc_generate_pairs(double gm, double w_lo, double w_hi, double t_lo, double t_hi, uint64_t seed, int64_t n,
                       double* out_host) {
    if (!out_host || n <= 0 || !(w_lo >= 1.0) || !(w_hi >= w_lo) || !(t_lo > 0.0) || !(t_hi >= t_lo) || !(gm > 1.0))
        return KNC_ERR_INVALID_ARGUMENT;
    DevBuf d;
    CKR(cudaMalloc(&d.p, (size_t)n * 8 * sizeof(double)));
    generate_pairs_kernel<<<(unsigned)((n + 255) / 256), 256>>>(gm, std::log(w_lo), std::log(w_hi), std::log(t_lo),
                                                                 std::log(t_hi), seed, n, (double*)d.p);
    CKR(cudaGetLastError());
    CKR(cudaMemcpy(out_host, d.p, (size_t)n * 8 * sizeof(double), cudaMemcpyDeviceToHost));
    return KNC_OK;
}

int knc_mlp_forward_backward(const float* weights, const float* x, const float* y, int32_t n, float* pred,
                             float* loss, float* grad) {
    if (!weights || !x || !y || n <= 0) return KNC_ERR_INVALID_ARGUMENT;
    CKR(configure_train());
    DevBuf dw, dx, dy, dg, dl, dp, de;
    CKR(cudaMalloc(&de.p, 4));
    CKR(cudaMemset(de.p, 0, 4));
    CKR(cudaMalloc(&dw.p, KNC_MLP_NUM_PARAMS * 4));
    CKR(cudaMalloc(&dx.p, (size_t)n * 12));
    CKR(cudaMalloc(&dy.p, (size_t)n * 4));
    CKR(cudaMalloc(&dg.p, KNC_MLP_NUM_PARAMS * 4));
    CKR(cudaMalloc(&dl.p, 4));
    CKR(cudaMalloc(&dp.p, (size_t)n * 4));
    CKR(cudaMemcpy(dw.p, weights, KNC_MLP_NUM_PARAMS * 4, cudaMemcpyHostToDevice));
    CKR(cudaMemcpy(dx.p, x, (size_t)n * 12, cudaMemcpyHostToDevice));
    CKR(cudaMemcpy(dy.p, y, (size_t)n * 4, cudaMemcpyHostToDevice));
    CKR(cudaMemset(dg.p, 0, KNC_MLP_NUM_PARAMS * 4));
    CKR(cudaMemset(dl.p, 0, 4));
    mlp_train_tc_kernel<<<grid_for_rows(n), TC_THREADS, train_smem_bytes()>>>(
        (const float*)dw.p, (const float*)dx.p, (const float*)dy.p, n, n, 0ull, 1.0f / (float)n, (float*)dg.p,
        (float*)dl.p, (float*)dp.p, (unsigned*)de.p);
    CKR(cudaGetLastError());
    unsigned err = 0;
    CKR(cudaMemcpy(&err, de.p, 4, cudaMemcpyDeviceToHost));
    if (err) return KNC_ERR_TIMEOUT;
    float lsum = 0.f;
    CKR(cudaMemcpy(&lsum, dl.p, 4, cudaMemcpyDeviceToHost));
    if (loss) *loss = lsum / (float)n;
    if (grad) CKR(cudaMemcpy(grad, dg.p, KNC_MLP_NUM_PARAMS * 4, cudaMemcpyDeviceToHost));
    if (pred) CKR(cudaMemcpy(pred, dp.p, (size_t)n * 4, cudaMemcpyDeviceToHost));
    return KNC_OK;
}

int knc_mlp_train(const double* pairs, int64_t n, float* weights, const knc_mlp_train_params* tp,
                  float* final_loss) {
    if (!pairs || n <= 0 || !weights || !tp || tp->batch <= 0 || tp->steps < 0) return KNC_ERR_INVALID_ARGUMENT;
    CKR(configure_train());
    DevBuf dpairs, dx, dy, dw, dm, dv, dg, dl, de;
    CKR(cudaMalloc(&de.p, 4));
    CKR(cudaMemset(de.p, 0, 4));
    CKR(cudaMalloc(&dpairs.p, (size_t)n * 8 * sizeof(double)));
    CKR(cudaMalloc(&dx.p, (size_t)n * 12));
    CKR(cudaMalloc(&dy.p, (size_t)n * 4));
    CKR(cudaMalloc(&dw.p, KNC_MLP_NUM_PARAMS * 4));
    CKR(cudaMalloc(&dm.p, KNC_MLP_NUM_PARAMS * 4));
    CKR(cudaMalloc(&dv.p, KNC_MLP_NUM_PARAMS * 4));
    CKR(cudaMalloc(&dg.p, KNC_MLP_NUM_PARAMS * 4));
    CKR(cudaMalloc(&dl.p, 4));
    CKR(cudaMemcpy(dpairs.p, pairs, (size_t)n * 8 * sizeof(double), cudaMemcpyHostToDevice));
    features_kernel<<<(unsigned)((n + 255) / 256), 256>>>((const double*)dpairs.p, n, (float*)dx.p, (float*)dy.p);
    CKR(cudaGetLastError());
    // fixed input normalisation from the data when the caller left it unset
    std::vector<float> w(weights, weights + KNC_MLP_NUM_PARAMS);
    if (w[KNC_MLP_OFF_XSCALE] == 0.f) {
        const int64_t m = std::min<int64_t>(n, 1 << 18);
        std::vector<float> xs((size_t)m * 3);
        CKR(cudaMemcpy(xs.data(), dx.p, (size_t)m * 12, cudaMemcpyDeviceToHost));
        for (int k = 0; k < 3; ++k) {
            double s = 0, s2 = 0;
            for (int64_t r = 0; r < m; ++r) {
                s += xs[r * 3 + k];
                s2 += (double)xs[r * 3 + k] * xs[r * 3 + k];
            }
            const double mean = s / m, var = std::max(s2 / m - mean * mean, 1e-12);
            w[KNC_MLP_OFF_XMEAN + k] = (float)mean;
            w[KNC_MLP_OFF_XSCALE + k] = (float)(1.0 / std::sqrt(var));
        }
    }
    CKR(cudaMemcpy(dw.p, w.data(), KNC_MLP_NUM_PARAMS * 4, cudaMemcpyHostToDevice));
    CKR(cudaMemset(dm.p, 0, KNC_MLP_NUM_PARAMS * 4));
    CKR(cudaMemset(dv.p, 0, KNC_MLP_NUM_PARAMS * 4));
    CKR(cudaMemset(dg.p, 0, KNC_MLP_NUM_PARAMS * 4));
    const int batch = tp->batch;
    const int grid = grid_for_rows(batch);
    const float b1 = tp->beta1 > 0.f ? tp->beta1 : 0.9f;
    const float b2 = tp->beta2 > 0.f ? tp->beta2 : 0.999f;
    const float eps = tp->eps > 0.f ? tp->eps : 1e-8f;
    double p1 = 1.0, p2 = 1.0;
    for (int64_t step = 0; step < tp->steps; ++step) {
        const uint64_t seed = splitmix64((tp->seed ? tp->seed : 1ull) + (uint64_t)step * 0x9E3779B97F4A7C15ull) | 1ull;
        mlp_train_tc_kernel<<<grid, TC_THREADS, train_smem_bytes()>>>(
            (const float*)dw.p, (const float*)dx.p, (const float*)dy.p, n, batch, seed, 1.0f / (float)batch,
            (float*)dg.p, (float*)dl.p, nullptr, (unsigned*)de.p);
        p1 *= b1;
        p2 *= b2;
        // learning-rate decay: cosine over the run to 5 % of the initial rate
        const double frac = tp->steps > 1 ? (double)step / (double)(tp->steps - 1) : 1.0;
        const float lr = (float)(tp->lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(3.14159265358979 * frac))));
        adam_kernel<<<(KNC_MLP_NUM_PARAMS + 255) / 256, 256>>>((float*)dw.p, (float*)dm.p, (float*)dv.p,
                                                               (float*)dg.p, KNC_MLP_NUM_PARAMS, lr, b1, b2, eps,
                                                               (float)(1.0 / (1.0 - p1)), (float)(1.0 / (1.0 - p2)));
    }
    CKR(cudaGetLastError());
    // final loss over (up to) the first 1M rows
    const int64_t ev = std::min<int64_t>(n, 1 << 20);
    CKR(cudaMemset(dl.p, 0, 4));
    mlp_train_tc_kernel<<<grid_for_rows(ev), TC_THREADS, train_smem_bytes()>>>(
        (const float*)dw.p, (const float*)dx.p, (const float*)dy.p, n, ev, 0ull, 1.0f / (float)ev, (float*)dg.p,
        (float*)dl.p, nullptr, (unsigned*)de.p);
    CKR(cudaGetLastError());
    unsigned err = 0;
    CKR(cudaMemcpy(&err, de.p, 4, cudaMemcpyDeviceToHost));
    if (err) return KNC_ERR_TIMEOUT;
    float lsum = 0.f;
    CKR(cudaMemcpy(&lsum, dl.p, 4, cudaMemcpyDeviceToHost));
    CKR(cudaMemcpy(weights, dw.p, KNC_MLP_NUM_PARAMS * 4, cudaMemcpyDeviceToHost));
    if (final_loss) *final_loss = lsum / (float)ev;
    return KNC_OK;
}

}  // extern "C"
