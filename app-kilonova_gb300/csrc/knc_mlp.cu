// knc_mlp.cu — training data and training kernels of the learned c2p guess.
//
// Pairs are rows of 8 doubles (D, S_r, S_theta, tau, rho, u_r, u_theta, p) per
// unit volume. They come from the solver itself: sampled from a live state
// (knc_sample_pairs, recovered with the FP64 Newton of the stage) or produced
// by the solver's prim -> cons over a range of Lorentz factors and
// temperatures (knc_generate_pairs).
//
// Training: each step draws a batch, runs the forward pass with the same
// tensor-core layer as inference (bf16 weights and activations, FP32
// accumulation), back-propagates in FP32 (straight-through for the bf16
// rounding of weights and activations) into per-warp private gradient tiles in
// shared memory, reduces them per CTA, and applies Adam.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "knc_internal.h"
#include "knc_mlp.cuh"
#include "knc_physics.cuh"

namespace knc {

constexpr int TRAIN_WARPS = 4;
constexpr int ZLD = 65;   // padded float rows of the per-warp z / dz tiles

struct TrainWarp {
    __nv_bfloat16 act[MLP_ACT_ELEMS];   // a1 = bf16(silu(z1)) rows
    float z[32 * ZLD];                  // z2, then dz2
    float dz1[32 * ZLD];
    float xn[32 * 3];
    float dout[32];
    float dw2[MLP_H * ZLD];             // private dW2 accumulator [u][v]
};

struct TrainSmem {
    MlpWeights W;
    TrainWarp warp[TRAIN_WARPS];
};

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + expf(-z)); }

// One launch = one gradient evaluation over `rows` rows. Row r reads data row
// (seed ? hash(seed, r) % n_data : r). Gradients (of the mean loss) are added
// into grad[]; the summed squared error into *loss_sum.
__global__ void __launch_bounds__(TRAIN_WARPS * 32) mlp_fwd_bwd_kernel(const float* __restrict__ w,
                                                                      const float* __restrict__ x,
                                                                      const float* __restrict__ y, int64_t n_data,
                                                                      int64_t rows, uint64_t seed, float inv_batch,
                                                                      float* __restrict__ grad,
                                                                      float* __restrict__ loss_sum,
                                                                      float* __restrict__ pred) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainSmem& S = *reinterpret_cast<TrainSmem*>(smem_raw);
    const int lane = threadIdx.x & 31;
    const int wid = threadIdx.x >> 5;
    TrainWarp& T = S.warp[wid];
    mlp_load(S.W, w);
    for (int k = lane; k < MLP_H * ZLD; k += 32) T.dw2[k] = 0.0f;
    __syncthreads();
    const MlpWeights& W = S.W;

    // register accumulators of the small parameter groups (lane owns units lane, lane+32)
    float g_w1[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    float g_b1[2] = {0.f, 0.f}, g_b2[2] = {0.f, 0.f}, g_w3[2] = {0.f, 0.f};
    float g_b3 = 0.f, l_sum = 0.f;

    const int64_t nchunks = (rows + 31) / 32;
    const int64_t gwarp = (int64_t)blockIdx.x * TRAIN_WARPS + wid;
    const int64_t nwarps = (int64_t)gridDim.x * TRAIN_WARPS;
    for (int64_t chunk = gwarp; chunk < nchunks; chunk += nwarps) {
        const int64_t r = chunk * 32 + lane;
        const bool valid = r < rows;
        int64_t d = r;
        if (seed) d = (int64_t)(splitmix64(seed ^ splitmix64((uint64_t)r)) % (uint64_t)n_data);
        float xr[3] = {0.f, 0.f, 0.f}, yr = 0.f;
        if (valid) {
            xr[0] = x[d * 3];
            xr[1] = x[d * 3 + 1];
            xr[2] = x[d * 3 + 2];
            yr = y[d];
        }
        // ---- forward
        mlp_layer1<false>(W, T.act, xr);
        T.xn[lane * 3 + 0] = (xr[0] - W.xm[0]) * W.xs[0];
        T.xn[lane * 3 + 1] = (xr[1] - W.xm[1]) * W.xs[1];
        T.xn[lane * 3 + 2] = (xr[2] - W.xm[2]) * W.xs[2];
        __syncwarp();
        float acc[2][8][4];
        mlp_layer2(W, T.act, acc);
        {
            const int g = lane >> 2, t = lane & 3;
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 8; ++nt) {
                    const int c = nt * 8 + 2 * t;
                    T.z[(mt * 16 + g) * ZLD + c] = acc[mt][nt][0];
                    T.z[(mt * 16 + g) * ZLD + c + 1] = acc[mt][nt][1];
                    T.z[(mt * 16 + g + 8) * ZLD + c] = acc[mt][nt][2];
                    T.z[(mt * 16 + g + 8) * ZLD + c + 1] = acc[mt][nt][3];
                }
        }
        __syncwarp();
        float out = W.b3;
        for (int u = 0; u < MLP_H; ++u) {
            const float z2 = T.z[lane * ZLD + u];
            out = fmaf(z2 * sigm(z2), W.w3[u], out);
        }
        if (pred && valid && !seed) pred[r] = out;
        const float e = valid ? out - yr : 0.f;
        l_sum += e * e;
        const float dout = 2.0f * e * inv_batch;
        T.dout[lane] = dout;
        g_b3 += dout;
        __syncwarp();
        // ---- backward, lane owns hidden units u = lane, lane + 32
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int u = lane + 32 * h;
            const float w3u = W.w3[u];
            float gw3 = 0.f, gb2 = 0.f;
            for (int row = 0; row < 32; ++row) {
                const float z2 = T.z[row * ZLD + u];
                const float s = sigm(z2);
                const float dr = T.dout[row];
                gw3 = fmaf(dr, z2 * s, gw3);
                const float dz2 = dr * w3u * s * (1.0f + z2 * (1.0f - s));
                T.z[row * ZLD + u] = dz2;
                gb2 += dz2;
            }
            g_w3[h] += gw3;
            g_b2[h] += gb2;
        }
        __syncwarp();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int u = lane + 32 * h;
            for (int v = 0; v < MLP_H; ++v) {
                float a = 0.f;
                for (int row = 0; row < 32; ++row)
                    a = fmaf(T.z[row * ZLD + u], __bfloat162float(T.act[row * MLP_LD + v]), a);
                T.dw2[u * ZLD + v] += a;
            }
        }
        // own row: da1 = dz2 W2, dz1 = da1 silu'(z1)
        {
            float z1[MLP_H];
            const float xn0 = T.xn[lane * 3], xn1 = T.xn[lane * 3 + 1], xn2 = T.xn[lane * 3 + 2];
            for (int v = 0; v < MLP_H; ++v)
                z1[v] = __fmaf_rn(W.w1[v * 3 + 2], xn2, __fmaf_rn(W.w1[v * 3 + 1], xn1, __fmaf_rn(W.w1[v * 3], xn0, W.b1[v])));
            for (int v = 0; v < MLP_H; ++v) {
                float da = 0.f;
                for (int u = 0; u < MLP_H; ++u)
                    da = fmaf(T.z[lane * ZLD + u], __bfloat162float(W.w2[u * MLP_LD + v]), da);
                const float s = sigm(z1[v]);
                T.dz1[lane * ZLD + v] = da * s * (1.0f + z1[v] * (1.0f - s));
            }
        }
        __syncwarp();
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int v = lane + 32 * h;
            float gb = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f;
            for (int row = 0; row < 32; ++row) {
                const float dz = T.dz1[row * ZLD + v];
                gb += dz;
                g0 = fmaf(dz, T.xn[row * 3], g0);
                g1 = fmaf(dz, T.xn[row * 3 + 1], g1);
                g2 = fmaf(dz, T.xn[row * 3 + 2], g2);
            }
            g_b1[h] += gb;
            g_w1[h][0] += g0;
            g_w1[h][1] += g1;
            g_w1[h][2] += g2;
        }
        __syncwarp();
    }
    // ---- reduce: warp-private tiles and registers -> global
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
    for (int h = 0; h < 2; ++h) {
        const int u = lane + 32 * h;
        atomicAdd(&grad[KNC_MLP_OFF_B1 + u], g_b1[h]);
        atomicAdd(&grad[KNC_MLP_OFF_B2 + u], g_b2[h]);
        atomicAdd(&grad[KNC_MLP_OFF_W3 + u], g_w3[h]);
        for (int k = 0; k < 3; ++k) atomicAdd(&grad[KNC_MLP_OFF_W1 + u * 3 + k], g_w1[h][k]);
    }
    __syncthreads();
    // sum the warps' dW2 tiles into warp 0's tile, then one atomic per entry
    for (int k = threadIdx.x; k < MLP_H * MLP_H; k += blockDim.x) {
        const int u = k / MLP_H, v = k - u * MLP_H;
        float s = 0.f;
        for (int q = 0; q < TRAIN_WARPS; ++q) s += S.warp[q].dw2[u * ZLD + v];
        if (s != 0.f) atomicAdd(&grad[KNC_MLP_OFF_W2 + k], s);
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

size_t train_smem_bytes() { return sizeof(TrainSmem); }

cudaError_t configure_train() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(mlp_fwd_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)train_smem_bytes());
    if (e == cudaSuccess) done = true;
    return e;
}

int grid_for_rows(int64_t rows) {
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t chunks = (rows + 31) / 32;
    // at least 4 chunks per warp so the per-CTA reduction amortises
    const int64_t ctas = std::max<int64_t>(1, std::min<int64_t>(sms, (chunks + 4 * TRAIN_WARPS - 1) / (4 * TRAIN_WARPS)));
    return (int)ctas;
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
    DevBuf dw, dx, dy, dg, dl, dp;
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
    mlp_fwd_bwd_kernel<<<grid_for_rows(n), TRAIN_WARPS * 32, train_smem_bytes()>>>(
        (const float*)dw.p, (const float*)dx.p, (const float*)dy.p, n, n, 0ull, 1.0f / (float)n, (float*)dg.p,
        (float*)dl.p, (float*)dp.p);
    CKR(cudaGetLastError());
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
    DevBuf dpairs, dx, dy, dw, dm, dv, dg, dl;
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
        mlp_fwd_bwd_kernel<<<grid, TRAIN_WARPS * 32, train_smem_bytes()>>>(
            (const float*)dw.p, (const float*)dx.p, (const float*)dy.p, n, batch, seed, 1.0f / (float)batch,
            (float*)dg.p, (float*)dl.p, nullptr);
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
    mlp_fwd_bwd_kernel<<<grid_for_rows(ev), TRAIN_WARPS * 32, train_smem_bytes()>>>(
        (const float*)dw.p, (const float*)dx.p, (const float*)dy.p, n, ev, 0ull, 1.0f / (float)ev, (float*)dg.p,
        (float*)dl.p, nullptr);
    CKR(cudaGetLastError());
    float lsum = 0.f;
    CKR(cudaMemcpy(&lsum, dl.p, 4, cudaMemcpyDeviceToHost));
    CKR(cudaMemcpy(weights, dw.p, KNC_MLP_NUM_PARAMS * 4, cudaMemcpyDeviceToHost));
    if (final_loss) *final_loss = lsum / (float)ev;
    return KNC_OK;
}

}  // extern "C"
