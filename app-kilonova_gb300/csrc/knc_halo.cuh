// knc_halo.cuh — halo rows that do not come from a same-shaped neighbour.
//
// ghost_zone: the two ghost blocks' rows next to the mesh ends, from the model
// at the stage time (src/scheme.rs:45-52 via BlockState::from_model and
// try_to_primitive): model primitive -> conserved x dV -> / dV -> primitive,
// the reference's round trip, then the scalar density.
// remap_zone: a halo row across a change of polar resolution (uneven blocks).
//
// Both are included by each stage translation unit, so a path's separate and
// fused kernels run the same instructions (the FP64 unit is compiled without
// FMA contraction, the mixed unit with it).
#pragma once

#include "knc_internal.h"
#include "knc_models.cuh"
#include "knc_physics.cuh"

namespace knc {

// The time of stage `sub` of step `step` of a fold that started at t0 with
// time step dt: the host's step arithmetic (the averages t1 (1 - b) + t0 b of
// godunov_core::runge_kutta, b = 1/2; 3/4 then 1/3), rounded operation by
// operation without contraction, so it equals the host's value bit for bit.
__device__ __forceinline__ double fold_stage_time(double t0, double dt, int order, int step, int sub) {
    auto avg = [](double t1, double tb, double bf) {
        return __dadd_rn(__dmul_rn(t1, __dadd_rn(-bf, 1.0)), __dmul_rn(tb, bf));
    };
    double t = t0;
    for (int k = 0;; ++k) {
        const double t1 = __dadd_rn(t, dt);
        double t2 = 0.0, end;
        if (order == 1) {
            end = t1;
        } else if (order == 2) {
            end = avg(__dadd_rn(t1, dt), t, 0.5);
        } else {
            t2 = avg(__dadd_rn(t1, dt), t, 0.75);
            end = avg(__dadd_rn(t2, dt), t, 1.0 / 3.0);
        }
        if (k >= step) return sub == 0 ? t : sub == 1 ? t1 : t2;
        t = end;
    }
}

// Zone k of the 2 x nq[end] ghost rows of end `end` (0: inner ghost block,
// min index - 1, whose last two rows feed the innermost block's rows 0, 1;
// 1: outer ghost block, whose first two rows feed rows nr+2, nr+3).
static __device__ __noinline__ void ghost_zone(const GhostArgs& a, int end, int k) {
    const int nq = a.nq[end];
    if (k >= 2 * nq || a.P[end] == nullptr) return;
    const int row = k / nq, j = k - row * nq;
    const double r = a.rc[end * 2 + row];
    const double q = a.qc[end][j];
    const double dV = a.dv[end][row * nq + j];
    double Pm[4];
    double scalar;
    if (a.host_prim[end]) {
        const double* hp = a.host_prim[end] + ((int64_t)row * nq + j) * 5;
        Pm[0] = hp[0];
        Pm[1] = hp[1];
        Pm[2] = hp[2];
        Pm[3] = hp[3];
        scalar = hp[4];
    } else {
        const double t = a.dt_bits ? fold_stage_time(a.t0, __dmul_rn(__longlong_as_double((long long)*a.dt_bits), a.cfl),
                                                     a.order, a.step, a.sub)
                                   : a.time;
        model_eval(a.model, r, q, t, false, a.ghost_index[end], 0, j, Pm, scalar);
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
    double Uv[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) Uv[c] = U[c] * dV;       // from_model: U dV
    const double smass = Uv[0] * scalar;                  // lab_frame_mass * scalar
    double u[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) u[c] = Uv[c] / dV;       // try_to_primitive: U / dV
    double P[4] = {0.0, 0.0, 0.0, 0.0};
    double bad = 0.0;
    int iters = 0, kind;
    if (a.srhd) kind = srhd_c2p_newton(a.gm, u, 0.0, P, iters, bad);
    else kind = newt_c2p(a.gm - 1.0, u, P, bad);
    if (kind != HYDRO_NONE && kind != HYDRO_NEGATIVE_PRESSURE) {
        atomicMin(&a.status->err_key, error_key(a.stage, 0x3ffeu + end, row, j, kind));
    }
    const double w = a.srhd ? sqrt(1.0 + P[1] * P[1] + P[2] * P[2]) : 1.0;
    const double v[NFIELD] = {P[0], P[1], P[2], P[3], smass / dV / w};
    const int nrt = a.nr_t[end];
    const int64_t pn = (int64_t)(nrt + 4) * nq;
    const int64_t off = (int64_t)(a.row0[end] + row) * nq + j;
    if (a.single_precision) {
        float* Pd = reinterpret_cast<float*>(a.P[end]);
#pragma unroll
        for (int c = 0; c < NFIELD; ++c) Pd[c * pn + off] = (float)v[c];
        // above the Lorentz-factor split: the FP64 row for zone_hp, and listed
        if (a.P64[end] && high_zone((float)v[1], (float)v[2], a.uu_high_f)) {
#pragma unroll
            for (int c = 0; c < NFIELD; ++c) a.P64[end][c * pn + off] = v[c];
            if (a.hp_list) note_high(a.hp_list, a.hp_count, a.hp_cap, a.edge_slot[end], a.row0[end] + row, nq, j);
        }
    } else {
        double* Pd = reinterpret_cast<double*>(a.P[end]);
#pragma unroll
        for (int c = 0; c < NFIELD; ++c) Pd[c * pn + off] = v[c];
    }
}

// ---- FP64 primitives of the mixed stage's zones above the Lorentz-factor split
// FP64 primitive (rho, u_r, u_theta, p, s) of the volume integrals U over the
// FP64 volume dv: Newton on the pressure to the reference's residual
// |f| < 1e-12 (D + tau) from the stored FP32 pressure pf[3] (a start one or
// two iterations from the root), the reference's iteration from the plain
// guess as the fallback, the stored FP32 primitive if both fail.
__device__ __forceinline__ void recover_hp(const double gm, const double (&U)[5], double dv, const float (&pf)[NFIELD],
                                           double (&v)[NFIELD]) {
#pragma unroll
    for (int q = 0; q < NFIELD; ++q) v[q] = (double)pf[q];
    const double m = U[0], s1 = U[1], s2 = U[2], tau = U[3];
    if (!(m > 0.0) || !(tau >= 0.0)) return;
    const double ss = s1 * s1 + s2 * s2;
    double p = 0.0, w = 1.0;
    int it = 0;
    if (newton_fast<double>(m, ss, tau, gm, (double)pf[3] * dv, NEWTON_TOLERANCE * (m + tau), 0.0, NEWTON_ITER_MAX,
                            p, w, it)) {
        const double inv_et = 1.0 / (tau + m + p);
        v[0] = m / w / dv;
        v[1] = w * s1 * inv_et;
        v[2] = w * s2 * inv_et;
        v[3] = p < 0.0 ? PRESSURE_FLOOR * v[0] : p / dv;
    } else {
        const double u[4] = {m, s1, s2, tau};
        double Pd[4];
        double bad;
        if (srhd_c2p_newton(gm, u, 0.0, Pd, it, bad) == HYDRO_ROOT_FINDER_FAILED) return;
        v[0] = Pd[0] / dv;
        v[1] = Pd[1];
        v[2] = Pd[2];
        v[3] = Pd[3] / dv;
    }
    v[4] = U[4] / dv / sqrt(1.0 + v[1] * v[1] + v[2] * v[2]);
}

template <class T>
__device__ __forceinline__ void store_row_zone(T* P, int nr, int nq, int prow, int j, const T (&v)[NFIELD]) {
    const int64_t pn = (int64_t)(nr + 4) * nq, off = (int64_t)prow * nq + j;
#pragma unroll
    for (int q = 0; q < NFIELD; ++q) P[q * pn + off] = v[q];
}

// A zone (i, j) of block `slot` just stored with FP32 primitive pf above the
// split: its FP64 primitive from this stage's state into P64, in every block
// view store_prim wrote it to (its own rows and the neighbours' halo rows),
// each listed for the update's FP64 faces.
__device__ __forceinline__ void hp_store(const StageArgs& a, int slot, const DevBlock& B, int i, int j,
                                         const float (&pf)[NFIELD]) {
    const int64_t n = (int64_t)B.nr * B.nq, z = (int64_t)i * B.nq + j;
    const double* Ub = B.buf[a.sel_in] + z;
    const double U[5] = {Ub[0], Ub[n], Ub[2 * n], Ub[3 * n], Ub[4 * n]};
    double v[NFIELD];
    recover_hp(a.gm, U, B.dv[z], pf, v);
    store_row_zone(B.P64, B.nr, B.nq, i + 2, j, v);
    if (a.hp_list) note_high(a.hp_list, a.hp_count, a.hp_cap, slot, i + 2, B.nq, j);
    if (i < 2 && B.P_in_nbr) {
        store_row_zone(a.blocks[B.slot_in].P64, B.nr_in_nbr, B.nq, B.nr_in_nbr + 2 + i, j, v);
        if (a.hp_list) note_high(a.hp_list, a.hp_count, a.hp_cap, B.slot_in, B.nr_in_nbr + 2 + i, B.nq, j);
    }
    if (i >= B.nr - 2 && B.P_out_nbr) {
        store_row_zone(a.blocks[B.slot_out].P64, B.nr_out_nbr, B.nq, i - (B.nr - 2), j, v);
        if (a.hp_list) note_high(a.hp_list, a.hp_count, a.hp_cap, B.slot_out, i - (B.nr - 2), B.nq, j);
    }
}

// Halo zone k of remap item it = {target slot, source slot, side}: target
// column j of halo row `row` from row `row` of the source's edge rows:
//  - a finer source (R = nq_s / nq_t): conserved volume integrals and volumes
//    of its R zones summed in column order, then the stage's recovery REC
//    — a conservative merge;
//  - a coarser source: its primitive at column j / R, copied.
// The recovery of a merged zone (volume integrals U, volume dv) into the
// primitive row v: the reference's Newton from the plain guess (the FP64
// stage, equal to the oracle). The mixed stage passes its own policy.
struct RemapRecoveryF64 {
    template <class R>
    __device__ static int recover(const StageArgs& a, const double (&U)[5], double dv, R (&v)[NFIELD]) {
        double u[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) u[q] = U[q] / dv;
        double P[4] = {0.0, 0.0, 0.0, 0.0};
        double bad = 0.0;
        int iters = 0, kind;
        if (a.srhd) kind = srhd_c2p_newton(a.gm, u, 0.0, P, iters, bad);
        else kind = newt_c2p(a.gm - 1.0, u, P, bad);
        const double w = a.srhd ? sqrt(1.0 + P[1] * P[1] + P[2] * P[2]) : 1.0;
        const double sv = U[4] / dv / w;
        v[0] = (R)P[0];
        v[1] = (R)P[1];
        v[2] = (R)P[2];
        v[3] = (R)P[3];
        v[4] = (R)sv;
        return kind;
    }
};

template <class R, class REC = RemapRecoveryF64>
static __device__ __noinline__ void remap_zone(const StageArgs& a, const int4 it, int k) {
    const DevBlock& T = a.blocks[it.x];
    const DevBlock& S = a.blocks[it.y];
    const int side = it.z;
    const int nq_t = T.nq, nq_s = S.nq;
    if (k >= 2 * nq_t) return;
    const int row = k / nq_t, j = k - row * nq_t;
    const int srow = side == 0 ? S.nr - 2 + row : row;          // source interior row
    const int trow = side == 0 ? row : T.nr + 2 + row;          // target padded row
    R v[NFIELD];
    double U[5] = {0.0, 0.0, 0.0, 0.0, 0.0}, dv = 0.0;   // a merged zone's volume integrals
    const int64_t soff = (int64_t)(srow + 2) * nq_s + j / (nq_t > nq_s ? nq_t / nq_s : 1);
    if (nq_s < nq_t) {
        const R* Ps = reinterpret_cast<const R*>(S.P);
        const int64_t pn = (int64_t)(S.nr + 4) * nq_s;
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) v[q] = Ps[q * pn + soff];
    } else {
        const int Rr = nq_s / nq_t;
        const double* Us = S.buf[a.sel_in];
        const int64_t n = (int64_t)S.nr * nq_s;
        for (int m = 0; m < Rr; ++m) {
            const int64_t z = (int64_t)srow * nq_s + j * Rr + m;
#pragma unroll
            for (int q = 0; q < 5; ++q) U[q] += Us[q * n + z];
            dv += S.dv[z];
        }
        const int kind = REC::recover(a, U, dv, v);
        if (kind != HYDRO_NONE && kind != HYDRO_NEGATIVE_PRESSURE)
            atomicMin(&a.status->err_key, error_key(a.stage, it.y, srow, j * Rr, kind));
    }
    R* Pt = reinterpret_cast<R*>(T.P);
    const int64_t pt = (int64_t)(T.nr + 4) * nq_t;
    const int64_t ot = (int64_t)trow * nq_t + j;
#pragma unroll
    for (int q = 0; q < NFIELD; ++q) Pt[q * pt + ot] = v[q];
    if constexpr (sizeof(R) == 4) {
        // the mixed stage: a halo zone above the split takes its FP64 primitive
        // too (the coarser source's, or the merged zone's recovered in FP64)
        // and is listed in the target's view
        if (T.P64 && high_zone((float)v[1], (float)v[2], a.uu_high_f)) {
            double v64[NFIELD];
            if (nq_s < nq_t) {
                const int64_t pn = (int64_t)(S.nr + 4) * nq_s;
#pragma unroll
                for (int q = 0; q < NFIELD; ++q) v64[q] = S.P64[q * pn + soff];
            } else {
                float pf[NFIELD];
#pragma unroll
                for (int q = 0; q < NFIELD; ++q) pf[q] = (float)v[q];
                recover_hp(a.gm, U, dv, pf, v64);
            }
            store_row_zone(T.P64, T.nr, nq_t, trow, j, v64);
            if (a.hp_list) note_high(a.hp_list, a.hp_count, a.hp_cap, it.x, trow, nq_t, j);
        }
    }
}

// Separate-launch forms: blockIdx.y = end / remap item. Internal linkage, so
// each translation unit keeps its own (differently compiled) kernels.
namespace {

__global__ void ghost_kernel(GhostArgs a) { ghost_zone(a, blockIdx.y, blockIdx.x * blockDim.x + threadIdx.x); }

template <class R, class REC = RemapRecoveryF64>
__global__ void remap_kernel(StageArgs a, const int4* __restrict__ items) {
    const unsigned long long ek = *(volatile unsigned long long*)&a.status->err_key;
    if (ek != NO_ERROR && (uint32_t)(ek >> 48) < (uint32_t)a.stage) return;
    remap_zone<R, REC>(a, items[blockIdx.y], blockIdx.x * blockDim.x + threadIdx.x);
}

}  // namespace

}  // namespace knc
