// knc_stage.cuh — the fused flux / source / update kernel of one RK stage.
//
// One CTA owns a TR x TILE_Q tile of one block (TR = 4, 8 or 16, chosen per
// context) and runs TR + 1 warps, so that the TR + 1 rows of radial faces and
// the TR rows of TILE_Q + 1 polar faces are each one pass over its threads
// (the Riemann solves are the costly part; no pass leaves most warps idle at
// the following barrier). It stages the tile's primitives plus a 2-zone halo
// (radial halo rows are already present in the padded P array; theta halo
// columns come from the same block) in shared memory, then:
//   1. PLM slopes in r for rows -1..TILE_R and in theta for columns -1..TILE_Q
//      (zero slope on the first and last column of the block,
//      src/scheme.rs:107-110 via ndarray_ops::extend_default_2d);
//   2. one Riemann solve per face of the tile, scaled by c (SRHD) and the face
//      area (src/scheme.rs:90-97, 121-128; zero flux through the poles);
//   3. per zone: geometric source x dV, dU = (S - dF_r - dF_q) dt,
//      U1 = U + dU (src/scheme.rs:130-157), and the RK average
//      (1 - b) U1 + b U0 fused in (src/state.rs:179-212).
// Every face flux is computed once per tile; a zone's state is read once and
// written once, so the output may alias the input or the RK base buffer.
#pragma once

#include "knc_bits.cuh"
#include "knc_internal.h"
#include "knc_physics.cuh"

namespace knc {

// a * b for double-float factors, as an unevaluated pair (hi, lo): the FP32
// rounding of the product stays data-dependent instead of freezing a fixed
// per-face error into every flux difference.
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float h = a.x * b.x;
    const float e = __fmaf_rn(a.x, b.x, -h);
    return make_float2(h, __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, e)));
}

// x * (hi + lo) in FP32
__device__ __forceinline__ float df_scale(float x, float2 a) { return __fmaf_rn(x, a.x, x * a.y); }

template <int TR>
constexpr int update_threads() {
    return (TR + 1) * TILE_Q;
}

template <class R, int TR_>
struct StageSmem {
    static constexpr int TR = TR_, TQ = TILE_Q;
    static constexpr int PR = TR + 4, PQ = TQ + 4;
    static constexpr int NP = NFIELD * PR * PQ;
    static constexpr int NGR = NFIELD * (TR + 2) * TQ;
    static constexpr int NGQ = NFIELD * TR * (TQ + 2);
    static constexpr int NFR = NFIELD * (TR + 1) * TQ;
    static constexpr int NFQ = NFIELD * TR * (TQ + 1);
    static constexpr size_t bytes = sizeof(R) * (size_t)(NP + NGR + NGQ + NFR + NFQ);
    static constexpr size_t work_bytes = sizeof(R) * (size_t)(NGR + NGQ + NFR + NFQ);   // without staged P
};

template <class R>
__device__ __forceinline__ PhysT<R> make_phys(const StageArgs& a) {
    PhysT<R> ph;
    ph.srhd = a.srhd;
    ph.hllc = a.hllc;
    if constexpr (sizeof(R) == 4) {
        ph.gm = a.gm_f;
        ph.gm1 = a.gm1_f;
        ph.gh = a.gh_f;
        ph.theta = a.theta_f;
    } else {
        ph.gm = a.gm;
        ph.gm1 = a.gm - 1.0;
        ph.gh = a.gh;
        ph.theta = a.plm_theta;
    }
    return ph;
}

// One update tile t = {slot, i0, j0, -} with update_threads<TR>() threads.
// BOX = false: the tile's primitives are staged here from the padded P array
// and the conserved state is read from global memory. BOX = true: both are
// already in shared memory as tensor-copy boxes: boxP [5][TR+4][TQ+8] from
// padded row i0 and column j0 - 4 (zero outside the block), boxU / boxU0
// [5][TR][TQ] from row i0, column j0 (boxU0 only with an RK average).
// The slope limiter of a stage: the reference's form in FP64, the
// branch-free form in the mixed stage.
template <class R, bool MIXED>
__device__ __forceinline__ R stage_plm(R theta, R a, R b, R c) {
    if constexpr (MIXED) return plm_gradient_f32(theta, a, b, c);
    else return plm_gradient(theta, a, b, c);
}

// The stage's time step: the host's dt, or (adaptive dt found on the device)
// the reduced dl / a_max times the CFL number, formed like the host would.
template <class R>
__device__ __forceinline__ R stage_dt(const StageArgs& a) {
    if (a.dt_bits) {
        const double d = __dmul_rn(__longlong_as_double((long long)*(volatile unsigned long long*)a.dt_bits), a.cfl);
        return (R)d;
    }
    return sizeof(R) == 4 ? (R)a.dt_f : (R)a.dt;
}

// ---- FP64 faces of the mixed stage at high Lorentz factor -----------------------
// FP32 face states of a flow with W well above 1 lose its thermal energy: the
// kinetic part of tau and of the energy flux is O(rho W^2) and rounds at
// 6e-8 of that, which for p / rho ~ 1e-3 is a 1e-4 error in the pressure and
// moves shocks by a fraction of a zone (the W = 100 jet). So the mixed stage
// keeps FP64 where the Lorentz factor is above the split, as it already does
// for the recovery: every face whose 4-zone stencil holds a zone with
// W > w_split (judged from the stored FP32 four-velocity, the same test in
// every update form) is solved in FP64 from FP64 primitives, and the zones
// such faces bound are updated in FP64 (zone_hp, after the strip helpers).

// The FP64 faces of zone (i, j) from the relativistic zones of its plus-shaped
// stencil: col bit k = zone (i - 2 + k, j), row bit k = zone (i, j - 2 + k),
// k = 0..4. Result: bit 0 radial face i, bit 1 radial face i + 1, bit 2 polar
// face j, bit 3 polar face j + 1 (zero: the zone takes the FP32 update).
__device__ __forceinline__ unsigned hp_faces(unsigned col, unsigned row) {
    return ((col & 0xfu) ? 1u : 0u) | ((col & 0x1eu) ? 2u : 0u) | ((row & 0xfu) ? 4u : 0u) |
           ((row & 0x1eu) ? 8u : 0u);
}

static __device__ __noinline__ void zone_hp(const StageArgs& a, const DevBlock& B, int i, int j);
__device__ __forceinline__ void drain_hp(const StageArgs& a);
__device__ __forceinline__ void clear_next_hp(const StageArgs& a);

// Whether this stage stored a primitive above the split (a uniform read of
// the list's length; a stage without a list is taken to have some).
__device__ __forceinline__ bool stage_has_high(const StageArgs& a) {
    return a.hp_count == nullptr || *(volatile const unsigned*)a.hp_count != 0u;
}

template <class R, bool MIXED, int TR_, bool BOX = false>
__device__ __forceinline__ void update_tile(const StageArgs& a, const int4 t, unsigned char* smem_raw,
                                            const R* boxP = nullptr, const double* boxU = nullptr,
                                            const double* boxU0 = nullptr) {
    using S = StageSmem<R, TR_>;
    constexpr int TR = S::TR, TQ = S::TQ, PR = S::PR, PQ = S::PQ;
    constexpr int PQS = BOX ? TQ + 8 : PQ;   // row stride of the staged primitives
    constexpr int COFF = BOX ? 2 : 0;        // column of j0 - 2 in a staged row
    constexpr int NT = update_threads<TR>();
    R* sP = BOX ? nullptr : reinterpret_cast<R*>(smem_raw);
    const R* sPc = BOX ? boxP + COFF : sP;
    R* sGr = reinterpret_cast<R*>(smem_raw) + (BOX ? 0 : S::NP);
    R* sGq = sGr + S::NGR;
    R* sFr = sGq + S::NGQ;
    R* sFq = sFr + S::NFR;

    const DevBlock& B = a.blocks[t.x];
    const int nr = B.nr, nq = B.nq, i0 = t.y, j0 = t.z;
    const int tid = threadIdx.x;
    const R* P = reinterpret_cast<const R*>(B.P);
    const int64_t pn = (int64_t)(nr + 4) * nq;
    const bool one_d = a.one_dimensional != 0;
    if (MIXED && !BOX && tid < TR * TQ) {
        // the state this thread updates at the end: start it towards L2 now
        const int i = i0 + tid / TQ, j = j0 + tid % TQ;
        if (i < nr && j < nq) {
            const int64_t n = (int64_t)nr * nq, z = (int64_t)i * nq + j;
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) {
                asm volatile("prefetch.global.L2 [%0];" ::"l"(B.buf[a.sel_in] + q * n + z));
                if (a.sel_base >= 0) asm volatile("prefetch.global.L2 [%0];" ::"l"(B.buf[a.sel_base] + q * n + z));
            }
        }
    }

    // ---- stage primitives (tile rows -2..TR+1 = padded rows i0..i0+TR+3)
    if (!BOX) {
        for (int k = tid; k < PR * PQ; k += NT) {
            const int rr = k / PQ, cc = k - rr * PQ;
            const int prow = i0 + rr;
            const int j = j0 - 2 + cc;
            const bool ok = prow < nr + 4 && j >= 0 && j < nq;
            const int64_t off = (int64_t)prow * nq + j;
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) sP[(q * PR + rr) * PQ + cc] = ok ? P[q * pn + off] : R(0);
        }
        __syncthreads();
    }

    const PhysT<R> ph = make_phys<R>(a);
    const R th = ph.theta;

    // ---- PLM slopes: radial for rows -1..TR, then polar for columns -1..TQ
    // (the radial count is a whole number of warps, so no warp mixes the two)
    {
        constexpr int NGRZ = (TR + 2) * TQ, NGQZ = TR * (TQ + 2);
        const int total = one_d ? NGRZ : NGRZ + NGQZ;
        for (int k = tid; k < total; k += NT) {
            if (k < NGRZ) {
                const int g = k / TQ, c = k - g * TQ;
#pragma unroll
                for (int q = 0; q < NFIELD; ++q) {
                    const R* col = sPc + (q * PR) * PQS + c + 2;
                    sGr[(q * (TR + 2) + g) * TQ + c] =
                        stage_plm<R, MIXED>(th, col[g * PQS], col[(g + 1) * PQS], col[(g + 2) * PQS]);
                }
            } else {
                const int kk = k - NGRZ;
                const int r = kk / (TQ + 2), c = kk - r * (TQ + 2);
                const int j = j0 - 1 + c;
                const bool edge = j <= 0 || j >= nq - 1;
#pragma unroll
                for (int q = 0; q < NFIELD; ++q) {
                    const R* row = sPc + (q * PR + r + 2) * PQS + c;
                    sGq[(q * TR + r) * (TQ + 2) + c] = edge ? R(0) : stage_plm<R, MIXED>(th, row[0], row[1], row[2]);
                }
            }
        }
    }
    __syncthreads();

    const R cflux = sizeof(R) == 4 ? (R)a.cflux_f : (R)a.cflux;

    // ---- radial faces i0..i0+TR (face i between zone rows i-1 and i): one
    // pass of all NT threads
    for (int k = tid; k < (TR + 1) * TQ; k += NT) {
        const int f = k / TQ, c = k - f * TQ;
        const int i = i0 + f, j = j0 + c;
        R out[NFIELD] = {R(0), R(0), R(0), R(0), R(0)};
        if (i <= nr && j < nq) {
            R pl[4], pr[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                pl[q] = sPc[(q * PR + f + 1) * PQS + c + 2] + sGr[(q * (TR + 2) + f) * TQ + c] * R(0.5);
                pr[q] = sPc[(q * PR + f + 2) * PQS + c + 2] - sGr[(q * (TR + 2) + f + 1) * TQ + c] * R(0.5);
            }
            const R sl = sPc[(4 * PR + f + 1) * PQS + c + 2] + sGr[(4 * (TR + 2) + f) * TQ + c] * R(0.5);
            const R sr = sPc[(4 * PR + f + 2) * PQS + c + 2] - sGr[(4 * (TR + 2) + f + 1) * TQ + c] * R(0.5);
            if constexpr (MIXED) riemann_srhd_f32<0>(ph, pl, pr, sl, sr, out);
            else riemann(ph, pl, pr, sl, sr, 0, out);
            if constexpr (MIXED) {
                const float2 A = df_mul(B.ar_r[i], B.ar_q[j]);   // c A_r
#pragma unroll
                for (int q = 0; q < NFIELD; ++q) out[q] = df_scale(out[q], A);
            } else {
                const R A = (R)B.ar[(int64_t)i * nq + j];
#pragma unroll
                for (int q = 0; q < NFIELD; ++q) out[q] = out[q] * cflux * A;
            }
        }
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) sFr[(q * (TR + 1) + f) * TQ + c] = out[q];
    }
    // ---- polar faces j0..j0+TQ (face j between zone columns j-1 and j): one
    // pass, TR rows of TQ + 1 faces on (TR + 1) TQ threads
    if (!one_d) {
        for (int k = tid; k < TR * (TQ + 1); k += NT) {
            const int r = k / (TQ + 1), c = k - r * (TQ + 1);
            const int i = i0 + r, j = j0 + c;
            R out[NFIELD] = {R(0), R(0), R(0), R(0), R(0)};
            if (i < nr && j > 0 && j < nq) {
                R pl[4], pr[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    pl[q] = sPc[(q * PR + r + 2) * PQS + c + 1] + sGq[(q * TR + r) * (TQ + 2) + c] * R(0.5);
                    pr[q] = sPc[(q * PR + r + 2) * PQS + c + 2] - sGq[(q * TR + r) * (TQ + 2) + c + 1] * R(0.5);
                }
                const R sl = sPc[(4 * PR + r + 2) * PQS + c + 1] + sGq[(4 * TR + r) * (TQ + 2) + c] * R(0.5);
                const R sr = sPc[(4 * PR + r + 2) * PQS + c + 2] - sGq[(4 * TR + r) * (TQ + 2) + c + 1] * R(0.5);
                if constexpr (MIXED) riemann_srhd_f32<1>(ph, pl, pr, sl, sr, out);
                else riemann(ph, pl, pr, sl, sr, 1, out);
                if constexpr (MIXED) {
                    const float2 A = df_mul(B.aq_r[i], B.aq_q[j]);   // c A_theta
#pragma unroll
                    for (int q = 0; q < NFIELD; ++q) out[q] = df_scale(out[q], A);
                } else {
                    const R A = (R)B.aq[(int64_t)i * (nq + 1) + j];
#pragma unroll
                    for (int q = 0; q < NFIELD; ++q) out[q] = out[q] * cflux * A;
                }
            }
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) sFq[(q * TR + r) * (TQ + 1) + c] = out[q];
        }
    }
    __syncthreads();

    // ---- sources, conserved update, RK average
    if (tid < TR * TQ) {
        const int r = tid / TQ, c = tid - r * TQ;
        const int i = i0 + r, j = j0 + c;
        unsigned hpf = 0u;
        if constexpr (MIXED) {
            // FP64 faces (a relativistic zone in the plus stencil): zone_hp
            if (i < nr && j < nq && stage_has_high(a)) {
                unsigned cm = 0u, rm = 0u;
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    const R* zc = sPc + (PR + r + k) * PQS + c + 2;   // u_r of zone (i - 2 + k, j)
                    const R* zr = sPc + (PR + r + 2) * PQS + c + k;   // u_r of zone (i, j - 2 + k)
                    cm |= high_zone(zc[0], zc[PR * PQS], a.uu_high_f) ? 1u << k : 0u;
                    rm |= high_zone(zr[0], zr[PR * PQS], a.uu_high_f) ? 1u << k : 0u;
                }
                hpf = hp_faces(cm, rm);
                // with a list the zone waits for drain_hp; without, it is updated here
                if (hpf && !a.hp_list) zone_hp(a, B, i, j);
            }
        }
        if (i < nr && j < nq && !(MIXED && hpf)) {
            const int64_t n = (int64_t)nr * nq;
            const int64_t z = (int64_t)i * nq + j;
            R Pc[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) Pc[q] = sPc[(q * PR + r + 2) * PQS + c + 2];
            R src[4];
            R dV = R(0);
            float2 cdV = make_float2(0.f, 0.f);
            if constexpr (MIXED) {
                sources_srhd_f32(ph, Pc, B.rc32[i], B.cot32[j], src);
                cdV = df_mul(B.dv_r[i], B.dv_q[j]);   // c dV
            } else {
                sources(ph, Pc, (R)B.rc[i], (R)B.cot[j], src);
                dV = (R)B.dv[z];
            }
            const R dt = stage_dt<R>(a);
            const double* Uin = B.buf[a.sel_in];
            double* Uout = B.buf[a.sel_out];
            const double* U0 = a.sel_base >= 0 ? B.buf[a.sel_base] : nullptr;
            double res[NFIELD];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                R sc;
                if constexpr (MIXED) sc = df_scale(src[q], cdV);
                else sc = src[q] * cflux * dV;
                const R fa = sFr[(q * (TR + 1) + r) * TQ + c];
                const R fb = sFr[(q * (TR + 1) + r + 1) * TQ + c];
                R du;
                if (one_d) {
                    du = (sc - (fb - fa)) * dt;
                } else {
                    const R fc = sFq[(q * TR + r) * (TQ + 1) + c];
                    const R fd = sFq[(q * TR + r) * (TQ + 1) + c + 1];
                    du = (sc - (fb - fa) - (fd - fc)) * dt;
                }
                const double uin = BOX ? boxU[(q * TR + r) * TQ + c] : Uin[q * n + z];
                res[q] = uin + (MIXED ? f2d_exp((float)du, a.lscale2) : (double)du);
            }
            {
                const R fa = sFr[(4 * (TR + 1) + r) * TQ + c];
                const R fb = sFr[(4 * (TR + 1) + r + 1) * TQ + c];
                R ds;
                if (one_d) {
                    ds = (fb - fa) * -dt;
                } else {
                    const R fc = sFq[(4 * TR + r) * (TQ + 1) + c];
                    const R fd = sFq[(4 * TR + r) * (TQ + 1) + c + 1];
                    ds = ((fb - fa) + (fd - fc)) * -dt;
                }
                const double uin = BOX ? boxU[(4 * TR + r) * TQ + c] : Uin[4 * n + z];
                res[4] = uin + (MIXED ? f2d_exp((float)ds, a.lscale2) : (double)ds);
            }
            if (U0) {
                if (MIXED && a.avg_half) {
                    // RK2 average (U1 + U0) / 2 with the halving on the integer pipe
#pragma unroll
                    for (int q = 0; q < NFIELD; ++q)
                        res[q] = half_exact(res[q] + (BOX ? boxU0[(q * TR + r) * TQ + c] : U0[q * n + z]));
                } else {
#pragma unroll
                    for (int q = 0; q < NFIELD; ++q)
                        res[q] = res[q] * a.w1 + (BOX ? boxU0[(q * TR + r) * TQ + c] : U0[q * n + z]) * a.bf;
                }
            }
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) Uout[q * n + z] = res[q];
        }
    }
}

// Update tiles (a.utiles) in a grid-stride loop: the launch is sized to the
// resident CTAs, so no CTA pays start-up per tile.
template <class R, bool MIXED, int TR>
__global__ void __launch_bounds__(update_threads<TR>(), MIXED ? (TR == 4 ? 6 : TR == 8 ? 3 : 2) : 1)
    update_kernel(StageArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // A failed c2p in this or an earlier stage stops the step: keep the
    // input state untouched so the failure can be reported from it.
    if (*(volatile unsigned long long*)&a.status->err_key != NO_ERROR) return;
    if constexpr (MIXED) clear_next_hp(a);
    for (int tile = blockIdx.x; tile < a.nutiles; tile += gridDim.x) {
        update_tile<R, MIXED, TR>(a, a.utiles[tile], smem_raw);
        __syncthreads();
    }
    if constexpr (MIXED) drain_hp(a);
}

// ---- warp strips ---------------------------------------------------------------
// The same update as update_tile, organised per warp without shared memory or
// CTA barriers: a warp owns a strip {slot, i0, j0, rows} of STRIP_OUT columns
// j0..j0+STRIP_OUT-1 (lanes 2..STRIP_OUT+1; lanes 0, 1 and the last two hold
// the polar halo) and marches down its rows. The radial window (rows i, i+1,
// i+2 and the slope of row i) and the lower radial face flux stay in
// registers; polar neighbours come through warp shuffles. Every face and
// zone expression is the one update_tile evaluates, on the same values, so
// the two forms give bit-identical states.

template <class R>
__device__ __forceinline__ void load_prim_row(const R* P, int64_t pn, int nq, int nr, int j, bool jin, int zrow,
                                              R v[NFIELD]) {
    const int prow = zrow + 2;   // padded row
    const bool ok = jin && prow < nr + 4;
    const int64_t off = ok ? (int64_t)prow * nq + j : 0;
#pragma unroll
    for (int q = 0; q < NFIELD; ++q) v[q] = ok ? P[q * pn + off] : R(0);
}

template <class R, bool MIXED>
__device__ __forceinline__ void strip_face(const PhysT<R>& ph, const StageArgs& a, const DevBlock& B, int axis,
                                           const R* pl, const R* pr, int i, int j, int nq, R cflux, R out[NFIELD]) {
    if constexpr (MIXED) {
        if (axis == 0) riemann_srhd_f32<0>(ph, pl, pr, pl[4], pr[4], out);
        else riemann_srhd_f32<1>(ph, pl, pr, pl[4], pr[4], out);
        const float2 A = axis == 0 ? df_mul(B.ar_r[i], B.ar_q[j]) : df_mul(B.aq_r[i], B.aq_q[j]);
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) out[q] = df_scale(out[q], A);
    } else {
        riemann(ph, pl, pr, pl[4], pr[4], axis, out);
        const R A = axis == 0 ? (R)B.ar[(int64_t)i * nq + j] : (R)B.aq[(int64_t)i * (nq + 1) + j];
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) out[q] = out[q] * cflux * A;
    }
}

// ---- FP64 faces of the mixed stage at high Lorentz factor (zone_hp) -----------
// FP64 primitive (rho, u_r, u_theta, p, s) of zone (r, c) of block B,
// r in [-2, nr + 1] (padded rows, halo included): a zone above the split
// takes the FP64 primitive its producer stored in P64 (the recovery from
// this stage's state, the ghost rows' model values, a remapped halo zone's);
// every other zone its stored FP32 primitive. P64 and P are read-only while
// the update runs, so every update form and every order of the FP64-face
// zones sees the same values (the middle RK3 stage updates in place).
__device__ __forceinline__ void prim_hp(const StageArgs& a, const DevBlock& B, int r, int c, double v[NFIELD]) {
    const float* P = reinterpret_cast<const float*>(B.P);
    const int64_t pn = (int64_t)(B.nr + 4) * B.nq;
    const int64_t off = (int64_t)(r + 2) * B.nq + c;
    if (high_zone(P[pn + off], P[2 * pn + off], a.uu_high_f)) {
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) v[q] = B.P64[q * pn + off];
    } else {
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) v[q] = (double)P[q * pn + off];
    }
}

// One face from its stencil s[0..3] (the face between s[1] and s[2]) with the
// stage's limiter; zl / zr: zero slope for s[1] / s[2] (the block's first and
// last column). FP64: the reference's face solve. FP32: the instructions the
// update forms run for the same face, so the value equals theirs.
template <class R>
__device__ __forceinline__ void face_states(R th, const R (*s)[NFIELD], bool zl, bool zr, R pl[NFIELD],
                                            R pr[NFIELD]) {
#pragma unroll
    for (int q = 0; q < NFIELD; ++q) {
        const R gl = zl ? R(0) : stage_plm<R, sizeof(R) == 4>(th, s[0][q], s[1][q], s[2][q]);
        const R gr = zr ? R(0) : stage_plm<R, sizeof(R) == 4>(th, s[1][q], s[2][q], s[3][q]);
        pl[q] = s[1][q] + gl * R(0.5);
        pr[q] = s[2][q] - gr * R(0.5);
    }
}

// Zone (i, j) of the mixed stage when its plus-shaped stencil holds a zone
// above the Lorentz-factor split (update forms: high_zone / hp_faces). Its
// faces whose 4-zone stencil holds such a zone are solved in FP64 from FP64
// primitives (prim_hp); its other faces are solved again in FP32 from the
// stored primitives with the update forms' own instructions, so a face
// shared with a zone of the FP32 update carries the same flux on both sides.
// Sources, update and RK average in FP64, written to U_out. Every zone
// bordering an FP64 face solves that face from the same inputs with the same
// instructions, so both of its zones see one flux.
static __device__ __noinline__ void zone_hp(const StageArgs& a, const DevBlock& B, int i, int j) {
    const int nq = B.nq, nr = B.nr;
    const float* P = reinterpret_cast<const float*>(B.P);
    const int64_t pn = (int64_t)(nr + 4) * nq;
    // FP32 primitives as the update forms see them: col32[k] zone (i - 2 + k, j),
    // row32[k] zone (i, j - 2 + k), zero outside the padded rows and the block's columns
    float col32[5][NFIELD], row32[5][NFIELD];
    unsigned cm = 0u, rm = 0u;
    for (int k = 0; k < 5; ++k) {
        const int c = j - 2 + k;
        load_prim_row(P, pn, nq, nr, j, true, i - 2 + k, col32[k]);
        load_prim_row(P, pn, nq, nr, c, c >= 0 && c < nq, i, row32[k]);
        cm |= high_zone(col32[k][1], col32[k][2], a.uu_high_f) ? 1u << k : 0u;
        rm |= high_zone(row32[k][1], row32[k][2], a.uu_high_f) ? 1u << k : 0u;
    }
    const unsigned faces = hp_faces(cm, rm);
    const PhysT<float> ph32 = make_phys<float>(a);
    const PhysT<double> ph = make_phys<double>(a);
    // col[k]: zone (i - 2 + k, j); row[k]: zone (i, j - 2 + k), FP64
    double col[5][NFIELD], row[5][NFIELD];
    prim_hp(a, B, i, j, col[2]);
#pragma unroll
    for (int q = 0; q < NFIELD; ++q) row[2][q] = col[2][q];
    if (faces & 3u)
        for (int k = 0; k < 5; ++k)
            if (k != 2) prim_hp(a, B, i - 2 + k, j, col[k]);
    if (faces & 12u)
        for (int k = 0; k < 5; ++k) {
            const int c = j - 2 + k;
            if (k == 2) continue;
            if (c >= 0 && c < nq) {
                prim_hp(a, B, i, c, row[k]);
            } else {
#pragma unroll
                for (int q = 0; q < NFIELD; ++q) row[k][q] = 0.0;
            }
        }
    const double l2 = ldexp(1.0, a.lscale2);   // FP32 fluxes carry areas in the stage's length units
    double F[4][NFIELD];
    for (int f = 0; f < 4; ++f) {
        // face f: radial i, radial i + 1, polar j, polar j + 1
        const bool radial = f < 2;
        const int k = radial ? i + f : j + (f - 2);   // between rows / columns k - 1 and k
        const bool exists = radial ? k <= nr : (k > 0 && k < nq && i < nr);
        const bool zl = !radial && (k - 1 == 0 || k - 1 == nq - 1);
        const bool zr = !radial && (k == 0 || k == nq - 1);
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) F[f][q] = 0.0;
        if (!exists) continue;
        if ((faces >> f) & 1u) {
            double pl[NFIELD], pr[NFIELD], out[NFIELD];
            face_states<double>(ph.theta, radial ? &col[f] : &row[f - 2], zl, zr, pl, pr);
            riemann(ph, pl, pr, pl[4], pr[4], radial ? 0 : 1, out);
            const double A = radial ? B.ar[(int64_t)k * nq + j] : B.aq[(int64_t)i * (nq + 1) + k];
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) F[f][q] = out[q] * a.cflux * A;
        } else {
            float pl[NFIELD], pr[NFIELD], out[NFIELD] = {0.f, 0.f, 0.f, 0.f, 0.f};
            face_states<float>(ph32.theta, radial ? &col32[f] : &row32[f - 2], zl, zr, pl, pr);
            strip_face<float, true>(ph32, a, B, radial ? 0 : 1, pl, pr, radial ? k : i, radial ? j : k, nq,
                                    a.cflux_f, out);
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) F[f][q] = (double)out[q] * l2;
        }
    }
    const int64_t n = (int64_t)nr * nq, z = (int64_t)i * nq + j;
    double src[4];
    sources(ph, col[2], B.rc[i], B.cot[j], src);
    const double dv = B.dv[z];
    const double dt = stage_dt<double>(a);
    const double* Uin = B.buf[a.sel_in];
    double* Uout = B.buf[a.sel_out];
    double res[NFIELD];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const double du = (src[q] * a.cflux * dv - (F[1][q] - F[0][q]) - (F[3][q] - F[2][q])) * dt;
        res[q] = Uin[q * n + z] + du;
    }
    res[4] = Uin[4 * n + z] + ((F[1][4] - F[0][4]) + (F[3][4] - F[2][4])) * -dt;
    if (a.sel_base >= 0) {
        const double* U0 = B.buf[a.sel_base];
        if (a.avg_half) {
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) res[q] = half_exact(res[q] + U0[q * n + z]);
        } else {
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) res[q] = res[q] * a.w1 + U0[q * n + z] * a.bf;
        }
    }
#pragma unroll
    for (int q = 0; q < NFIELD; ++q) Uout[q * n + z] = res[q];
}

// ---- the zones with FP64 faces, from the stage's list of zones above the split
// Work item c of listed zone h = (slot, padded row, column): the candidate
// zone at offset c of h's plus-shaped neighbourhood (c < 5: rows -2..2 of
// h's column; c >= 5: columns -2, -1, 1, 2 of h's row). A candidate inside
// its block is updated by zone_hp if h is the first zone above the split in
// the candidate's own plus stencil (column zones top to bottom, then row
// zones left to right): every zone with FP64 faces has exactly one such
// first zone, and every stored zone above the split is listed, so each is
// updated once.
__device__ __forceinline__ void hp_candidate(const StageArgs& a, unsigned item, unsigned c) {
    const int2 e = a.hp_list[item];
    const DevBlock& B = a.blocks[e.x];
    const int nq = B.nq, nr = B.nr;
    const int ih = e.y / nq - 2, jh = e.y - (e.y / nq) * nq;
    const int d = (int)c < 5 ? (int)c - 2 : ((int)c < 7 ? (int)c - 7 : (int)c - 6);
    const int ic = (int)c < 5 ? ih + d : ih;
    const int jc = (int)c < 5 ? jh : jh + d;
    if (ic < 0 || ic >= nr || jc < 0 || jc >= nq) return;
    const float* Pu = reinterpret_cast<const float*>(B.P) + (int64_t)(nr + 4) * nq;   // u_r; u_theta one field on
    const int64_t pn = (int64_t)(nr + 4) * nq;
    auto high = [&](int i, int j) {
        if (j < 0 || j >= nq) return false;
        const int64_t off = (int64_t)(i + 2) * nq + j;
        return high_zone(Pu[off], Pu[pn + off], a.uu_high_f);
    };
    int fi = 0, fj = -1;
    for (int k = 0; k < 5 && fj < 0; ++k)
        if (high(ic - 2 + k, jc)) {
            fi = ic - 2 + k;
            fj = jc;
        }
    for (int k = 0; k < 5 && fj < 0; ++k)
        if (k != 2 && high(ic, jc - 2 + k)) {
            fi = ic;
            fj = jc - 2 + k;
        }
    if (fi == ih && fj == jh) zone_hp(a, B, ic, jc);
}

// The update's second part: whole warps claim 32 work items at a time until
// the list's 9 items per listed zone are done. The list is complete before
// the update starts (the recovery, ghost and remap launches wrote it), and
// the zones it updates are the ones every update form left untouched.
__device__ __forceinline__ void drain_hp(const StageArgs& a) {
    if (!a.hp_list) return;
    const unsigned count = min(*(volatile const unsigned*)a.hp_count, a.hp_cap);
    if (count == 0u) return;
    const unsigned total = 9u * count;
    const unsigned lane = threadIdx.x & 31u;
    for (;;) {
        unsigned base = 0u;
        if (lane == 0u) base = atomicAdd(a.hp_claim, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= total) break;
        const unsigned w = base + lane;
        if (w < total) hp_candidate(a, w / 9u, w % 9u);
    }
}

// The next stage's list starts empty: cleared by the update of this stage
// (the previous stage's update, its last reader, finished before this one).
__device__ __forceinline__ void clear_next_hp(const StageArgs& a) {
    if (a.hp_count_next && blockIdx.x == 0 && threadIdx.x == 0) {
        *a.hp_count_next = 0u;
        *a.hp_claim_next = 0u;
    }
}

// HP (mixed stage only): the strip reaches a zone above the Lorentz-factor
// split; zones with FP64 faces are left untouched by the row loop.
template <class R, bool MIXED, bool HP = false>
__device__ __forceinline__ void update_strip(const StageArgs& a, const int4 it, const PhysT<R>& ph) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const DevBlock& B = a.blocks[it.x];
    const int nr = B.nr, nq = B.nq, i0 = it.y, j0 = it.z, rows = it.w;
    const int j = j0 - 2 + lane;
    const bool jin = j >= 0 && j < nq;
    const bool writes = lane >= 2 && lane < 2 + STRIP_OUT && jin;
    const R* P = reinterpret_cast<const R*>(B.P);
    const int64_t pn = (int64_t)(nr + 4) * nq;
    const int64_t n = (int64_t)nr * nq;
    const R th = ph.theta;
    const R cflux = sizeof(R) == 4 ? (R)a.cflux_f : (R)a.cflux;
    const R dt = stage_dt<R>(a);
    const double* Uin = B.buf[a.sel_in];
    double* Uout = B.buf[a.sel_out];
    const double* U0 = a.sel_base >= 0 ? B.buf[a.sel_base] : nullptr;
    const bool pedge = j <= 0 || j >= nq - 1;   // zero polar slope on the block's first and last column

    // rows i0-2 .. i0+1, slopes of rows i0-1 and i0, the flux through face i0
    R Pa[NFIELD], P0[NFIELD], P1[NFIELD], P2[NFIELD], g0[NFIELD], Flo[NFIELD];
    load_prim_row(P, pn, nq, nr, j, jin, i0 - 2, Pa);
    load_prim_row(P, pn, nq, nr, j, jin, i0 - 1, P2);   // P2 as scratch for row i0-1
    load_prim_row(P, pn, nq, nr, j, jin, i0, P0);
    load_prim_row(P, pn, nq, nr, j, jin, i0 + 1, P1);
    {
        R gm[NFIELD], pl[NFIELD], pr[NFIELD];
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) {
            gm[q] = stage_plm<R, MIXED>(th, Pa[q], P2[q], P0[q]);
            g0[q] = stage_plm<R, MIXED>(th, P2[q], P0[q], P1[q]);
            pl[q] = P2[q] + gm[q] * R(0.5);
            pr[q] = P0[q] - g0[q] * R(0.5);
        }
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) Flo[q] = R(0);
        if (i0 <= nr && j < nq && jin) strip_face<R, MIXED>(ph, a, B, 0, pl, pr, i0, j, nq, cflux, Flo);
    }
    // mixed: hk = the warp's relativistic zones of window row i - 2 + k (bit =
    // lane), warp-uniform; hp: some lane left zones to zone_hp
    unsigned h0 = 0u, h1 = 0u, h2 = 0u, h3 = 0u, h4 = 0u;
    bool hp = false;
    if constexpr (HP) {
        h0 = __ballot_sync(full, high_zone(Pa[1], Pa[2], a.uu_high_f));
        h1 = __ballot_sync(full, high_zone(P2[1], P2[2], a.uu_high_f));
        h2 = __ballot_sync(full, high_zone(P0[1], P0[2], a.uu_high_f));
        h3 = __ballot_sync(full, high_zone(P1[1], P1[2], a.uu_high_f));
    }
    load_prim_row(P, pn, nq, nr, j, jin, i0 + 2, P2);
    if constexpr (HP) h4 = __ballot_sync(full, high_zone(P2[1], P2[2], a.uu_high_f));

    // per-column factors
    const int jc = jin ? j : 0;
    for (int s = 0; s < rows; ++s) {
        const int i = i0 + s;
        // the next row, one step ahead
        R Pn[NFIELD];
        load_prim_row(P, pn, nq, nr, j, jin, i + 3, Pn);
        unsigned h5 = 0u;
        if constexpr (HP) h5 = __ballot_sync(full, high_zone(Pn[1], Pn[2], a.uu_high_f));
        // this row's state and RK base towards L1 (read at the end of the step)
        if (MIXED && writes) {
            const int64_t z = (int64_t)i * nq + j;
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) {
                asm volatile("prefetch.global.L1 [%0];" ::"l"(Uin + q * n + z));
                if (U0) asm volatile("prefetch.global.L1 [%0];" ::"l"(U0 + q * n + z));
            }
        }
        // ---- polar: slopes of row i, the face j - 1 | j, its right neighbour's
        R gq[NFIELD], plq[NFIELD], prq[NFIELD], Fq[NFIELD], Fq1[NFIELD];
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) {
            const R left = __shfl_up_sync(full, P0[q], 1);
            const R right = __shfl_down_sync(full, P0[q], 1);
            gq[q] = pedge ? R(0) : stage_plm<R, MIXED>(th, left, P0[q], right);
            plq[q] = __shfl_up_sync(full, P0[q] + gq[q] * R(0.5), 1);
            prq[q] = P0[q] - gq[q] * R(0.5);
            Fq[q] = R(0);
        }
        if (lane > 0 && i < nr && j > 0 && j < nq) strip_face<R, MIXED>(ph, a, B, 1, plq, prq, i, j, nq, cflux, Fq);
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) Fq1[q] = __shfl_down_sync(full, Fq[q], 1);
        // ---- radial: slope of row i+1, the face i+1
        R g1[NFIELD], plr[NFIELD], prr[NFIELD], Fhi[NFIELD];
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) {
            g1[q] = stage_plm<R, MIXED>(th, P0[q], P1[q], P2[q]);
            plr[q] = P0[q] + g0[q] * R(0.5);
            prr[q] = P1[q] - g1[q] * R(0.5);
            Fhi[q] = R(0);
        }
        if (i + 1 <= nr && jin) strip_face<R, MIXED>(ph, a, B, 0, plr, prr, i + 1, j, nq, cflux, Fhi);
        // ---- mixed: a relativistic zone in the plus stencil (FP64 faces) leaves
        // the zone to zone_hp after the row loop, its state untouched until then
        unsigned hpf = 0u;
        if constexpr (HP) {
            if ((h0 | h1 | h2 | h3 | h4) != 0u) {
                const unsigned col = ((h0 >> lane) & 1u) | ((h1 >> lane) & 1u) << 1 | ((h2 >> lane) & 1u) << 2 |
                                     ((h3 >> lane) & 1u) << 3 | ((h4 >> lane) & 1u) << 4;
                hpf = hp_faces(col, lane >= 2 ? (h2 >> (lane - 2)) & 0x1fu : 0u);   // lane = column + 2 - j0
                hp = hp || __any_sync(full, writes && hpf);
            }
        }
        if (writes && !(HP && hpf)) {
            // ---- sources, conserved update, RK average of zone (i, j)
            const int64_t z = (int64_t)i * nq + jc;
            R src[4];
            R dV = R(0);
            float2 cdV = make_float2(0.f, 0.f);
            if constexpr (MIXED) {
                sources_srhd_f32(ph, P0, B.rc32[i], B.cot32[jc], src);
                cdV = df_mul(B.dv_r[i], B.dv_q[jc]);
            } else {
                sources(ph, P0, (R)B.rc[i], (R)B.cot[jc], src);
                dV = (R)B.dv[z];
            }
            double res[NFIELD];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                R sc;
                if constexpr (MIXED) sc = df_scale(src[q], cdV);
                else sc = src[q] * cflux * dV;
                const R du = (sc - (Fhi[q] - Flo[q]) - (Fq1[q] - Fq[q])) * dt;
                res[q] = Uin[q * n + z] + (MIXED ? f2d_exp((float)du, a.lscale2) : (double)du);
            }
            {
                const R ds = ((Fhi[4] - Flo[4]) + (Fq1[4] - Fq[4])) * -dt;
                res[4] = Uin[4 * n + z] + (MIXED ? f2d_exp((float)ds, a.lscale2) : (double)ds);
            }
            if (U0) {
                if (MIXED && a.avg_half) {
#pragma unroll
                    for (int q = 0; q < NFIELD; ++q) res[q] = half_exact(res[q] + U0[q * n + z]);
                } else {
#pragma unroll
                    for (int q = 0; q < NFIELD; ++q) res[q] = res[q] * a.w1 + U0[q * n + z] * a.bf;
                }
            }
#pragma unroll
            for (int q = 0; q < NFIELD; ++q) Uout[q * n + z] = res[q];
        }
        // ---- advance the window
        if constexpr (HP) {
            h0 = h1;
            h1 = h2;
            h2 = h3;
            h3 = h4;
            h4 = h5;
        }
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) {
            Flo[q] = Fhi[q];
            g0[q] = g1[q];
            P0[q] = P1[q];
            P1[q] = P2[q];
            P2[q] = Pn[q];
        }
    }
    // a stage without a list: the zones with FP64 faces, once the row window
    // is dead (the strip's rows again, with the same relativistic-zone test
    // on the four-velocity rows); with a list, drain_hp updates them
    if constexpr (HP) {
        if (hp && !a.hp_list) {
            const float* Pu = reinterpret_cast<const float*>(B.P) + pn;   // u_r; u_theta one field further
            auto high_row = [&](int zrow) -> unsigned {
                const int prow = zrow + 2;
                if (!jin || prow >= nr + 4) return 0u;
                const int64_t off = (int64_t)prow * nq + j;
                return high_zone(Pu[off], Pu[pn + off], a.uu_high_f) ? 1u : 0u;
            };
            unsigned h = high_row(i0 - 2) | high_row(i0 - 1) << 1 | high_row(i0) << 2 | high_row(i0 + 1) << 3;
            for (int s = 0; s < rows; ++s) {
                h |= high_row(i0 + s + 2) << 4;
                const unsigned m = __ballot_sync(full, (h & 4u) != 0u);
                if (writes && hp_faces(h & 0x1fu, lane >= 2 ? (m >> (lane - 2)) & 0x1fu : 0u))
                    zone_hp(a, B, i0 + s, jc);
                h >>= 1;
            }
        }
    }
}

// Whether strip it = {slot, i0, j0, rows} reaches a zone above the Lorentz
// factor split: the stored four-velocity of every zone its output zones'
// stencils read (rows i0 - 2 .. i0 + rows + 1 of its 32 columns), warp-wide.
__device__ __forceinline__ bool strip_reaches_high(const StageArgs& a, const int4 it) {
    const DevBlock& B = a.blocks[it.x];
    const int nr = B.nr, nq = B.nq;
    const int j = it.z - 2 + (int)(threadIdx.x & 31);
    const float* Pu = reinterpret_cast<const float*>(B.P) + (int64_t)(nr + 4) * nq;   // u_r; u_theta one field on
    const int64_t pn = (int64_t)(nr + 4) * nq;
    bool any = false;
    if (j >= 0 && j < nq) {
        const int r1 = min(it.y + it.w + 4, nr + 4);   // padded rows i0 .. i0 + rows + 3
        for (int r = it.y; r < r1; ++r) {
            const int64_t off = (int64_t)r * nq + j;
            any |= high_zone(Pu[off], Pu[pn + off], a.uu_high_f);
        }
    }
    return __any_sync(0xffffffffu, any);
}

// A strip with FP64 faces, out of line: its detection and zone_hp calls stay
// out of the register allocation of the common strip.
static __device__ __noinline__ void update_strip_hp(const StageArgs& a, const int4 it) {
    update_strip<float, true, true>(a, it, make_phys<float>(a));
}

// The mixed stage's strips when the stage listed zones above the split:
// each strip checks whether it reaches one (then the out-of-line form leaves
// its zones with FP64 faces untouched), then the list's zones are updated.
// Out of line, so that the common strip loop keeps its own registers.
// first / step: this thread's warp's first strip and the warps of the grid.
static __device__ __noinline__ void update_strips_hp(const StageArgs& a, int first, int step) {
    const PhysT<float> ph = make_phys<float>(a);
    for (int k = first; k < a.nstrips; k += step) {
        const int4 it = a.strips[k];
        if (strip_reaches_high(a, it)) update_strip_hp(a, it);
        else update_strip<float, true>(a, it, ph);
    }
    drain_hp(a);
}

// The strips of a stage, warps first .. in steps of `step`: the mixed stage
// takes the form above when its list holds a zone.
template <class R, bool MIXED>
__device__ __forceinline__ void stage_strips(const StageArgs& a, int first, int step) {
    if constexpr (MIXED) {
        clear_next_hp(a);
        if (stage_has_high(a)) {
            update_strips_hp(a, first, step);
            return;
        }
    }
    const PhysT<R> ph = make_phys<R>(a);
    for (int k = first; k < a.nstrips; k += step) update_strip<R, MIXED>(a, a.strips[k], ph);
}

// Strips (a.strips) in a grid-stride loop over warps; MB = resident CTAs per
// SM the register allocation is sized for (a tuning choice: more warps
// against fewer registers).
template <class R, bool MIXED, int MB>
__global__ void __launch_bounds__(STRIP_WARPS * 32, MB) update_strip_kernel(const __grid_constant__ StageArgs a) {
    // launched chained to the recovery (programmatic dependent launch): wait
    // for it to complete, let the next stage's recovery be scheduled
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    if (*(volatile unsigned long long*)&a.status->err_key != NO_ERROR) return;
    stage_strips<R, MIXED>(a, blockIdx.x * STRIP_WARPS + (threadIdx.x >> 5), gridDim.x * STRIP_WARPS);
}

// Block-wide reduction helpers (warp shuffles, then one atomic per warp).
__device__ __forceinline__ void warp_reduce_stats(DevStatus* st, unsigned long long zones,
                                                  unsigned long long it64, unsigned long long it32,
                                                  unsigned long long fb, double dtz, bool want_dt) {
    const unsigned mask = 0xffffffffu;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        zones += __shfl_down_sync(mask, zones, o);
        it64 += __shfl_down_sync(mask, it64, o);
        it32 += __shfl_down_sync(mask, it32, o);
        fb += __shfl_down_sync(mask, fb, o);
        if (want_dt) dtz = fmin(dtz, __shfl_down_sync(mask, dtz, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (zones) atomicAdd(&st->c2p_zones, zones);
        if (it64) atomicAdd(&st->iters_fp64, it64);
        if (it32) atomicAdd(&st->iters_fp32, it32);
        if (fb) atomicAdd(&st->fallbacks, fb);
        if (want_dt) atomicMin(&st->dt_bits, (unsigned long long)__double_as_longlong(dtz));
    }
}

// Write one zone's primitive + scalar density into its padded row and, for
// the two rows next to a block edge, into the neighbour's halo rows.
template <class R>
__device__ __forceinline__ void store_prim(const DevBlock& B, int i, int j, const R v[NFIELD]) {
    const int nr = B.nr, nq = B.nq;
    R* Pd = reinterpret_cast<R*>(B.P);
    const int64_t pn = (int64_t)(nr + 4) * nq;
    const int64_t off = (int64_t)(i + 2) * nq + j;
#pragma unroll
    for (int q = 0; q < NFIELD; ++q) Pd[q * pn + off] = v[q];
    if (i < 2 && B.P_in_nbr) {
        R* Q = reinterpret_cast<R*>(B.P_in_nbr);
        const int nrn = B.nr_in_nbr;
        const int64_t qn = (int64_t)(nrn + 4) * nq;
        const int64_t qo = (int64_t)(nrn + 2 + i) * nq + j;
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) Q[q * qn + qo] = v[q];
    }
    if (i >= nr - 2 && B.P_out_nbr) {
        R* Q = reinterpret_cast<R*>(B.P_out_nbr);
        const int64_t qn = (int64_t)(B.nr_out_nbr + 4) * nq;
        const int64_t qo = (int64_t)(i - (nr - 2)) * nq + j;
#pragma unroll
        for (int q = 0; q < NFIELD; ++q) Q[q * qn + qo] = v[q];
    }
}

}  // namespace knc
