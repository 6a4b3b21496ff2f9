// knc_mlp.cuh — the learned pressure guess for cons -> prim recovery.
//
// MLP 3 -> 64 -> 64 -> 1 (SiLU), BF16 weights, FP32 accumulation. Inputs,
// all invariant under U -> k U (the recovery is scale-invariant, so log D
// carries no information):
//   x0 = log(tau / D)
//   x1 = -log(1 - |S| / (D + tau))      (the Lorentz-factor scale of |S|/(D+tau))
//   x2 = log((tau (tau + 2D) - S^2) / D^2)
// x2 is E^2 - S^2 - D^2 with E = tau + D; for cold gas it tends to
// 2 D W p / (gamma - 1), so it keeps the pressure visible where tau / D is
// dominated by kinetic energy (W >> 1, p / rho << 1). It is formed in FP64.
// The output is y = log(p / D), so the pressure guess is D exp(y), clamped to
// (0, (gamma - 1) tau]. The reference
// starts every Newton pressure recovery from the same guess
// (hydro-srhd's srhd_2d::Conserved::to_primitive, reached through
// src/physics/relativistic_hydro.rs:68-88); this guess replaces it and the
// plain guess stays as the fallback.
//
// Inference is warp-cooperative: a warp evaluates 32 zones at once, the
// 64x64 layer as 2 (rows) x 8 (columns) x 4 (k) tensor-core tiles
// mma.sync.m16n8k16 (bf16 in, f32 accumulate). All FP32 arithmetic is written
// with explicit fma intrinsics so the result does not depend on the FMA
// contraction flags of the translation unit that includes this header.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "../../include/knc.h"

namespace knc {

constexpr int MLP_H = KNC_MLP_HIDDEN;
constexpr int MLP_LD = 72;    // padded row of bf16 tiles: conflict-free fragment loads

struct MlpWeights {
    float w1[MLP_H * 3];
    float b1[MLP_H];
    float b2[MLP_H];
    float w3[MLP_H];
    float b3;
    float xm[3];
    float xs[3];
    float pad_;
    __nv_bfloat16 w2[MLP_H * MLP_LD];   // row = output unit
};

// Per-warp activation tile: 32 zones x 64 hidden units (bf16, padded rows).
constexpr int MLP_ACT_ELEMS = 32 * MLP_LD;

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Stage the packed weights into shared memory (W1, W3 rounded to bf16 as the
// forward pass uses them; W2 stored as bf16). Called by all threads of a CTA,
// followed by __syncthreads() in the caller.
__device__ __forceinline__ void mlp_load(MlpWeights& S, const float* __restrict__ w) {
    for (int k = threadIdx.x; k < MLP_H * 3; k += blockDim.x) S.w1[k] = bf16r(w[KNC_MLP_OFF_W1 + k]);
    for (int k = threadIdx.x; k < MLP_H; k += blockDim.x) {
        S.b1[k] = w[KNC_MLP_OFF_B1 + k];
        S.b2[k] = w[KNC_MLP_OFF_B2 + k];
        S.w3[k] = bf16r(w[KNC_MLP_OFF_W3 + k]);
    }
    for (int k = threadIdx.x; k < MLP_H * MLP_H; k += blockDim.x) {
        const int u = k / MLP_H, v = k - u * MLP_H;
        S.w2[u * MLP_LD + v] = __float2bfloat16_rn(w[KNC_MLP_OFF_W2 + k]);
    }
    if (threadIdx.x == 0) {
        S.b3 = w[KNC_MLP_OFF_B3];
        for (int k = 0; k < 3; ++k) {
            S.xm[k] = w[KNC_MLP_OFF_XMEAN + k];
            S.xs[k] = w[KNC_MLP_OFF_XSCALE + k];
        }
    }
}

// Features of a conserved state (any volume scaling): D, S^2 = S_r^2 + S_q^2, tau.
// Returns false when the state has no usable features (the plain guess applies).
__device__ __forceinline__ bool mlp_features(double d, double ss, double tau, float x[3]) {
    const double e = tau + d;
    const double a = tau * (tau + 2.0 * d) - ss;       // E^2 - S^2 - D^2
    if (!(d > 0.0) || !(tau > 0.0) || !(a > 0.0)) {
        x[0] = x[1] = x[2] = 0.f;
        return false;
    }
    const float df = (float)d, ef = (float)e;
    const float xs = sqrtf((float)ss) / ef;
    x[0] = __logf((float)tau / df);
    x[1] = __logf(1.0f + xs) - __logf((float)(a + d * d) / (ef * ef));
    x[2] = __logf((float)a / (df * df));
    return true;
}

__device__ __forceinline__ float tanh_approx(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// SiLU for inference: x sigmoid(x) with sigmoid(x) = (1 + tanh(x/2)) / 2.
__device__ __forceinline__ float silu_fast(float x) {
    return x * __fmaf_rn(0.5f, tanh_approx(0.5f * x), 0.5f);
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Layer 1 for this lane's zone into the warp's activation tile (row = lane).
template <bool FAST>
__device__ __forceinline__ void mlp_layer1(const MlpWeights& S, __nv_bfloat16* act, const float x[3],
                                           float* z1_out = nullptr) {
    const int lane = threadIdx.x & 31;
    const float xn0 = (x[0] - S.xm[0]) * S.xs[0];
    const float xn1 = (x[1] - S.xm[1]) * S.xs[1];
    const float xn2 = (x[2] - S.xm[2]) * S.xs[2];
    uint32_t* row = reinterpret_cast<uint32_t*>(act + lane * MLP_LD);
#pragma unroll 8
    for (int u = 0; u < MLP_H; u += 2) {
        const float za = __fmaf_rn(S.w1[u * 3 + 2], xn2, __fmaf_rn(S.w1[u * 3 + 1], xn1, __fmaf_rn(S.w1[u * 3], xn0, S.b1[u])));
        const float zb = __fmaf_rn(S.w1[u * 3 + 5], xn2, __fmaf_rn(S.w1[u * 3 + 4], xn1, __fmaf_rn(S.w1[u * 3 + 3], xn0, S.b1[u + 1])));
        float ha, hb;
        if (FAST) {
            ha = silu_fast(za);
            hb = silu_fast(zb);
        } else {
            ha = za / (1.0f + expf(-za));
            hb = zb / (1.0f + expf(-zb));
        }
        if (z1_out) {
            z1_out[u] = za;
            z1_out[u + 1] = zb;
        }
        row[u >> 1] = pack_bf16(ha, hb);
    }
}

// Layer 2 on tensor cores: acc[mt][nt][4] = b2 + A1 (32x64) W2^T (64x64).
__device__ __forceinline__ void mlp_layer2(const MlpWeights& S, const __nv_bfloat16* act, float acc[2][8][4]) {
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const float c0 = S.b2[nt * 8 + 2 * t], c1 = S.b2[nt * 8 + 2 * t + 1];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            acc[mt][nt][0] = c0;
            acc[mt][nt][1] = c1;
            acc[mt][nt][2] = c0;
            acc[mt][nt][3] = c1;
        }
    }
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
            const __nv_bfloat16* r0 = act + (mt * 16 + g) * MLP_LD + ks * 16 + 2 * t;
            const __nv_bfloat16* r1 = r0 + 8 * MLP_LD;
            a[mt][0] = *reinterpret_cast<const uint32_t*>(r0);
            a[mt][1] = *reinterpret_cast<const uint32_t*>(r1);
            a[mt][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
            a[mt][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const __nv_bfloat16* br = S.w2 + (nt * 8 + g) * MLP_LD + ks * 16 + 2 * t;
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(br);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(br + 8);
            mma_bf16_16816(acc[0][nt], a[0], b0, b1);
            mma_bf16_16816(acc[1][nt], a[1], b0, b1);
        }
    }
}

// Full inference for the 32 zones of a warp; every lane must call it (the
// tensor-core instructions are warp-wide). Returns y = log(p / D) for the
// calling lane's zone.
__device__ __forceinline__ float mlp_warp_infer(const MlpWeights& S, __nv_bfloat16* act, const float x[3]) {
    const int lane = threadIdx.x & 31;
    const int t = lane & 3;
    mlp_layer1<true>(S, act, x);
    __syncwarp();
    float acc[2][8][4];
    mlp_layer2(S, act, acc);
    float part[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const float wa = S.w3[nt * 8 + 2 * t], wb = S.w3[nt * 8 + 2 * t + 1];
            part[mt][0] = __fmaf_rn(silu_fast(acc[mt][nt][0]), wa, part[mt][0]);
            part[mt][0] = __fmaf_rn(silu_fast(acc[mt][nt][1]), wb, part[mt][0]);
            part[mt][1] = __fmaf_rn(silu_fast(acc[mt][nt][2]), wa, part[mt][1]);
            part[mt][1] = __fmaf_rn(silu_fast(acc[mt][nt][3]), wb, part[mt][1]);
        }
#pragma unroll
    for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            part[mt][h] += __shfl_xor_sync(0xffffffffu, part[mt][h], 1);
            part[mt][h] += __shfl_xor_sync(0xffffffffu, part[mt][h], 2);
        }
    // row z = 16 mt + 8 h + g is held by lane 4 g
    const int src = (lane & 7) * 4;
    const float v00 = __shfl_sync(0xffffffffu, part[0][0], src);
    const float v01 = __shfl_sync(0xffffffffu, part[0][1], src);
    const float v10 = __shfl_sync(0xffffffffu, part[1][0], src);
    const float v11 = __shfl_sync(0xffffffffu, part[1][1], src);
    const int mt = lane >> 4, h = (lane >> 3) & 1;
    const float y = mt ? (h ? v11 : v10) : (h ? v01 : v00);
    __syncwarp();
    return y + S.b3;
}

}  // namespace knc
