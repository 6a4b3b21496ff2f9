// knc_physics.cuh — per-zone physics of the finite-volume stage, on the device.
//
// Replaces the arithmetic the reference reaches through its Hydrodynamics
// trait (src/traits.rs:41-136): the adapters src/physics/relativistic_hydro.rs
// and src/physics/newtonian_hydro.rs and, behind them, the git crates
// hydro-srhd (srhd_2d: prim<->cons, riemann_hllc_scalar, sources, c2p),
// hydro-euler (euler_2d) and godunov-core (piecewise_linear::plm_gradient).
//
// Methods: SRHD prim/cons/flux and characteristic speeds after Marti & Mueller
// (Living Rev. Relativ. 2003), Newton pressure recovery after the same review
// (section 6), HLLE (Harten-Lax-van Leer with Einfeldt speeds), relativistic
// HLLC (Mignone & Bodo 2005), Newtonian HLLC (Toro ch. 10), generalised-minmod
// slopes (van Leer 1979), spherical-polar geometric sources.
//
// Templated on the arithmetic type. For `double` every expression keeps one
// fixed evaluation order; the FP64 translation unit is compiled without FMA
// contraction so these produce the same bits as the CPU oracle.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace knc {

constexpr double LIGHT_SPEED = 3e10;                   // src/physics/mod.rs:7
constexpr double PI = 3.14159265358979323846;
constexpr int NEWTON_ITER_MAX = 50;
constexpr double NEWTON_TOLERANCE = 1e-12;
constexpr double PRESSURE_FLOOR = 1e-3;                // relativistic_hydro.rs:79-81

enum : int {
    HYDRO_NONE = 0,
    HYDRO_NEGATIVE_DENSITY = 1,
    HYDRO_NEGATIVE_PRESSURE = 2,
    HYDRO_NEGATIVE_ENERGY_DENSITY = 3,
    HYDRO_ROOT_FINDER_FAILED = 4
};

template <class R>
struct PhysT {
    int srhd;      // 1 relativistic, 0 Newtonian
    int hllc;      // 1 HLLC, 0 HLLE
    R gm;          // gamma_law_index
    R gh;          // gm / (gm - 1)
    R gm1;         // gm - 1
    R theta;       // plm_theta
};

template <class R> __device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }
template <class R> __device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
__device__ __forceinline__ double rsqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ float rsqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ double rabs(double x) { return fabs(x); }
__device__ __forceinline__ float rabs(float x) { return fabsf(x); }

// godunov_core::piecewise_linear::plm_gradient: generalised minmod of
// theta (b - a), (c - a) / 2, theta (c - b).
template <class R>
__device__ __forceinline__ R plm_gradient(R theta, R a, R b, R c) {
    const R x = theta * (b - a);
    const R y = R(0.5) * (c - a);
    const R z = theta * (c - b);
    if (x > R(0) && y > R(0) && z > R(0)) return rmin(x, rmin(y, z));
    if (x < R(0) && y < R(0) && z < R(0)) return rmax(x, rmax(y, z));
    return R(0);
}

// FP32 generalised minmod without branches (the mixed stage): with
// x, y, z as in plm_gradient, y has the sign of x and z whenever those two
// agree (c - a = (c - b) + (b - a)), so the result is min(|x|, |y|, |z|) with
// the sign of x when x and z are non-zero and of one sign, else 0. The one
// difference from plm_gradient<float> is the sign of a zero result when
// 0.5 (c - a) underflows, which no sum with it can see.
__device__ __forceinline__ float plm_gradient_f32(float theta, float a, float b, float c) {
    const float x = theta * (b - a);
    const float y = 0.5f * (c - a);
    const float z = theta * (c - b);
    const float m = fminf(fabsf(x), fminf(fabsf(y), fabsf(z)));
    const bool agree = ((__float_as_uint(x) ^ __float_as_uint(z)) & 0x80000000u) == 0u && x != 0.0f && z != 0.0f;
    return agree ? copysignf(m, x) : 0.0f;
}

// One side of an interface: conserved state, normal flux, outer wave speeds,
// the passive scalar's conserved density (s W) and flux (s u_n).
template <class R>
struct Side {
    R U[4], F[4];
    R lm, lp, sU, sF, vn, pre;
};

template <class R>
__device__ __forceinline__ void srhd_side(const PhysT<R>& ph, R rho, R ur, R uq, R pre, R s, int axis,
                                          Side<R>& S) {
    const R uu = ur * ur + uq * uq;
    const R w2 = R(1) + uu;
    const R w = rsqrt_(w2);
    const R h = R(1) + pre / rho * ph.gh;
    const R d = rho * w;
    const R m = d * h;
    const R un = axis == 0 ? ur : uq;
    const R vn = un / w;
    S.U[0] = d;
    S.U[1] = m * ur;
    S.U[2] = m * uq;
    const R cs2 = ph.gm * pre / (rho * h);
    const R v2 = uu / w2;
    const R k = R(1) - cs2;
    const R a = vn * k;
    R b;
    if constexpr (sizeof(R) == 4) {
        // FP32: forms without cancellation, which the reference order has for
        // cold gas (tau = rho h W^2 - p - rho W) and for v -> 1 (1 - v^2,
        // 1 - v^2 cs^2 - v_n^2 (1 - cs^2)):
        //   tau = p (gh W^2 - 1) + D u^2 / (W + 1)
        //   1 - v^2 = 1 / W^2,   1 - v^2 cs^2 - v_n^2 (1 - cs^2) = 1/W^2 + v_t^2 (1 - cs^2)
        S.U[3] = pre * (ph.gh * w2 - R(1)) + d * uu / (w + R(1));
        const R ut = axis == 0 ? uq : ur;
        const R omv2 = R(1) / w2;
        b = rsqrt_(cs2 * omv2 * (omv2 + ut * ut * omv2 * k));
    } else {
        S.U[3] = m * w - pre - d;
        b = rsqrt_(cs2 * (R(1) - v2) * (R(1) - v2 * cs2 - vn * vn * k));
    }
    S.F[0] = S.U[0] * vn;
    S.F[1] = axis == 0 ? S.U[1] * vn + pre : S.U[1] * vn;
    S.F[2] = axis == 1 ? S.U[2] * vn + pre : S.U[2] * vn;
    S.F[3] = (S.U[3] + pre) * vn;
    const R inv = R(1) / (R(1) - v2 * cs2);
    S.lm = (a - b) * inv;
    S.lp = (a + b) * inv;
    S.sU = s * w;
    S.sF = s * un;
    S.vn = vn;
    S.pre = pre;
}

template <class R>
__device__ __forceinline__ void newt_side(const PhysT<R>& ph, R rho, R vr, R vq, R pre, R s, int axis,
                                          Side<R>& S) {
    const R vn = axis == 0 ? vr : vq;
    S.U[0] = rho;
    S.U[1] = rho * vr;
    S.U[2] = rho * vq;
    S.U[3] = pre / ph.gm1 + R(0.5) * rho * (vr * vr + vq * vq);
    S.F[0] = S.U[0] * vn;
    S.F[1] = axis == 0 ? S.U[1] * vn + pre : S.U[1] * vn;
    S.F[2] = axis == 1 ? S.U[2] * vn + pre : S.U[2] * vn;
    S.F[3] = (S.U[3] + pre) * vn;
    const R cs = rsqrt_(ph.gm * pre / rho);
    S.lm = vn - cs;
    S.lp = vn + cs;
    S.sU = s;
    S.sF = s * vn;
    S.vn = vn;
    S.pre = pre;
}

template <class R>
__device__ __forceinline__ void make_side(const PhysT<R>& ph, const R* P, R s, int axis, Side<R>& S) {
    if (ph.srhd) srhd_side(ph, P[0], P[1], P[2], P[3], s, axis, S);
    else newt_side(ph, P[0], P[1], P[2], P[3], s, axis, S);
}

template <class R>
__device__ __forceinline__ void hlle(const Side<R>& L, const Side<R>& Rr, R out[5]) {
    const R am = rmin(L.lm, Rr.lm);
    const R ap = rmax(L.lp, Rr.lp);
    if (am >= R(0)) {
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = L.F[q];
        out[4] = L.sF;
    } else if (ap <= R(0)) {
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = Rr.F[q];
        out[4] = Rr.sF;
    } else {
        const R inv = R(1) / (ap - am);
        const R apam = ap * am;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            out[q] = (ap * L.F[q] - am * Rr.F[q] + apam * (Rr.U[q] - L.U[q])) * inv;
        out[4] = (ap * L.sF - am * Rr.sF + apam * (Rr.sU - L.sU)) * inv;
    }
}

// Relativistic HLLC, Mignone & Bodo (2005): contact speed from the HLL state
// in the cancellation-free root form, star states with E = tau + D.
template <class R>
__device__ __forceinline__ void srhd_hllc(const Side<R>& L, const Side<R>& Rr, int axis, R out[5]) {
    const R am = rmin(L.lm, Rr.lm);
    const R ap = rmax(L.lp, Rr.lp);
    if (am >= R(0)) {
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = L.F[q];
        out[4] = L.sF;
        return;
    }
    if (ap <= R(0)) {
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = Rr.F[q];
        out[4] = Rr.sF;
        return;
    }
    const int n = axis == 0 ? 1 : 2;
    const int t = axis == 0 ? 2 : 1;
    const R inv = R(1) / (ap - am);
    const R apam = ap * am;
    R Uh[4], Fh[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        Uh[q] = (ap * Rr.U[q] - am * L.U[q] - (Rr.F[q] - L.F[q])) * inv;
        Fh[q] = (ap * L.F[q] - am * Rr.F[q] + apam * (Rr.U[q] - L.U[q])) * inv;
    }
    const R e_hll = Uh[3] + Uh[0];
    const R fe_hll = Fh[3] + Fh[0];
    const R m_hll = Uh[n];
    const R fm_hll = Fh[n];
    const R bq = e_hll + fm_hll;
    const R disc = rmax(bq * bq - R(4) * fe_hll * m_hll, R(0));
    const R lstar = R(2) * m_hll / (bq + rsqrt_(disc));
    const R pstar = fm_hll - fe_hll * lstar;
    const bool left = lstar >= R(0);
    const Side<R>& K = left ? L : Rr;
    const R lam = left ? am : ap;
    const R fac = R(1) / (lam - lstar);
    const R lv = lam - K.vn;
    const R e_k = K.U[3] + K.U[0];
    R Us[4];
    Us[0] = K.U[0] * lv * fac;
    Us[n] = (K.U[n] * lv + pstar - K.pre) * fac;
    Us[t] = K.U[t] * lv * fac;
    const R e_s = (e_k * lv + pstar * lstar - K.pre * K.vn) * fac;
    Us[3] = e_s - Us[0];
#pragma unroll
    for (int q = 0; q < 4; ++q) out[q] = K.F[q] + lam * (Us[q] - K.U[q]);
    const R s_star = K.sU * lv * fac;
    out[4] = K.sF + lam * (s_star - K.sU);
}

// Newtonian HLLC (Toro 3rd ed. section 10.4, contact speed eq. 10.37).
template <class R>
__device__ __forceinline__ void newt_hllc(const Side<R>& L, const Side<R>& Rr, int axis, R out[5]) {
    const R am = rmin(L.lm, Rr.lm);
    const R ap = rmax(L.lp, Rr.lp);
    if (am >= R(0)) {
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = L.F[q];
        out[4] = L.sF;
        return;
    }
    if (ap <= R(0)) {
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = Rr.F[q];
        out[4] = Rr.sF;
        return;
    }
    const int n = axis == 0 ? 1 : 2;
    const int t = axis == 0 ? 2 : 1;
    const R ql = L.U[0] * (am - L.vn);
    const R qr = Rr.U[0] * (ap - Rr.vn);
    const R sstar = (Rr.pre - L.pre + L.U[n] * (am - L.vn) - Rr.U[n] * (ap - Rr.vn)) / (ql - qr);
    const bool left = sstar >= R(0);
    const Side<R>& K = left ? L : Rr;
    const R lam = left ? am : ap;
    const R rho = K.U[0];
    const R lv = lam - K.vn;
    const R fac = rho * lv / (lam - sstar);
    R Us[4];
    Us[0] = fac;
    Us[n] = fac * sstar;
    Us[t] = fac * (K.U[t] / rho);
    Us[3] = fac * (K.U[3] / rho + (sstar - K.vn) * (sstar + K.pre / (rho * lv)));
#pragma unroll
    for (int q = 0; q < 4; ++q) out[q] = K.F[q] + lam * (Us[q] - K.U[q]);
    const R s_star = K.sU * lv / (lam - sstar);
    out[4] = K.sF + lam * (s_star - K.sU);
}

template <class R>
__device__ __forceinline__ void riemann(const PhysT<R>& ph, const R* pl, const R* pr, R sl, R sr,
                                        int axis, R out[5]) {
    Side<R> L, Rr;
    make_side(ph, pl, sl, axis, L);
    make_side(ph, pr, sr, axis, Rr);
    if (ph.hllc) {
        if (ph.srhd) srhd_hllc(L, Rr, axis, out);
        else newt_hllc(L, Rr, axis, out);
    } else {
        hlle(L, Rr, out);
    }
}

// ---- FP32 relativistic forms for the mixed stage ------------------------------
// The quantities of srhd_side<float> for a face normal fixed at compile time,
// with the reciprocals shared: 1/W from one rsqrt (W = W^2 / W, v_n = u_n / W,
// 1 - v^2 = 1/W^2), 1/rho and 1/h once each.
template <int AXIS>
__device__ __forceinline__ void srhd_side_f32(const PhysT<float>& ph, float rho, float ur, float uq, float pre,
                                              float s, Side<float>& S) {
    const float uu = ur * ur + uq * uq;
    const float w2 = 1.0f + uu;
    const float iw = rsqrtf(w2);
    const float w = w2 * iw;
    const float pr = pre * (1.0f / rho);     // p / rho
    const float h = 1.0f + pr * ph.gh;
    const float d = rho * w;
    const float m = d * h;
    const float un = AXIS == 0 ? ur : uq;
    const float ut = AXIS == 0 ? uq : ur;
    const float vn = un * iw;
    S.U[0] = d;
    S.U[1] = m * ur;
    S.U[2] = m * uq;
    const float cs2 = ph.gm * pr * (1.0f / h);
    const float omv2 = iw * iw;
    const float v2 = uu * omv2;
    const float k = 1.0f - cs2;
    const float a = vn * k;
    // tau without cancellation: p (gh W^2 - 1) + D u^2 / (W + 1)
    S.U[3] = pre * (ph.gh * w2 - 1.0f) + d * uu * (1.0f / (w + 1.0f));
    const float b = sqrtf(cs2 * omv2 * (omv2 + ut * ut * omv2 * k));
    S.F[0] = S.U[0] * vn;
    S.F[1] = AXIS == 0 ? S.U[1] * vn + pre : S.U[1] * vn;
    S.F[2] = AXIS == 1 ? S.U[2] * vn + pre : S.U[2] * vn;
    S.F[3] = (S.U[3] + pre) * vn;
    const float inv = 1.0f / (1.0f - v2 * cs2);
    S.lm = (a - b) * inv;
    S.lp = (a + b) * inv;
    S.sU = s * w;
    S.sF = s * un;
    S.vn = vn;
    S.pre = pre;
}

// Both sides of a face at once, on Blackwell's paired FP32 units: every
// product, sum and fused multiply-add of srhd_side_f32 runs on the (left,
// right) pair as one instruction (__fmul2_rn / __fadd2_rn / __ffma2_rn, each
// lane rounded like its scalar form); reciprocals and square roots stay
// per lane.
__device__ __forceinline__ float2 pair(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 bcast(float a) { return make_float2(a, a); }

template <int AXIS>
__device__ __forceinline__ void srhd_sides_f32x2(const PhysT<float>& ph, const float* pl, const float* pr, float sl,
                                                 float sr, Side<float>& L, Side<float>& R) {
    const float2 one = bcast(1.0f), mone = bcast(-1.0f);
    const float2 rho = pair(pl[0], pr[0]), ur = pair(pl[1], pr[1]), uq = pair(pl[2], pr[2]);
    const float2 pre = pair(pl[3], pr[3]), s = pair(sl, sr);
    const float2 uu = __ffma2_rn(ur, ur, __fmul2_rn(uq, uq));
    const float2 w2 = __fadd2_rn(one, uu);
    const float2 iw = pair(rsqrtf(w2.x), rsqrtf(w2.y));
    const float2 w = __fmul2_rn(w2, iw);
    const float2 prr = __fmul2_rn(pre, pair(1.0f / rho.x, 1.0f / rho.y));   // p / rho
    const float2 h = __ffma2_rn(prr, bcast(ph.gh), one);
    const float2 d = __fmul2_rn(rho, w);
    const float2 m = __fmul2_rn(d, h);
    const float2 un = AXIS == 0 ? ur : uq;
    const float2 ut = AXIS == 0 ? uq : ur;
    const float2 vn = __fmul2_rn(un, iw);
    const float2 U1 = __fmul2_rn(m, ur), U2 = __fmul2_rn(m, uq);
    const float2 cs2 = __fmul2_rn(__fmul2_rn(bcast(ph.gm), prr), pair(1.0f / h.x, 1.0f / h.y));
    const float2 omv2 = __fmul2_rn(iw, iw);                                  // 1 - v^2
    const float2 v2 = __fmul2_rn(uu, omv2);
    const float2 k = __ffma2_rn(cs2, mone, one);                            // 1 - cs^2
    const float2 a = __fmul2_rn(vn, k);
    const float2 wp1 = __fadd2_rn(w, one);
    const float2 t = __fmul2_rn(__fmul2_rn(rho, uu), pair(1.0f / wp1.x, 1.0f / wp1.y));   // rho u^2 / (W + 1)
    // tau without cancellation: p (gh W^2 - 1) + W rho u^2 / (W + 1)
    const float2 U3 = __ffma2_rn(pre, __ffma2_rn(bcast(ph.gh), w2, mone), __fmul2_rn(w, t));
    const float2 inner = __ffma2_rn(__fmul2_rn(__fmul2_rn(ut, ut), omv2), k, omv2);
    const float2 barg = __fmul2_rn(__fmul2_rn(cs2, omv2), inner);
    const float2 b = pair(sqrtf(barg.x), sqrtf(barg.y));
    // fluxes in the forms with the fewest roundings (all equal to U v_n + p e_n
    // in exact arithmetic): D v_n = rho u_n, S v_n = rho h u u_n,
    // (tau + p) v_n = u_n (rho u^2 / (W + 1) + gh p W); the density flux then
    // carries one rounding instead of three, which is what the density error
    // of a near-steady flow accumulates from
    const float2 rhoh = __ffma2_rn(bcast(ph.gh), pre, rho);
    const float2 rhohun = __fmul2_rn(rhoh, un);
    const float2 F0 = __fmul2_rn(rho, un);
    const float2 F1 = AXIS == 0 ? __ffma2_rn(rhohun, ur, pre) : __fmul2_rn(rhohun, ur);
    const float2 F2 = AXIS == 1 ? __ffma2_rn(rhohun, uq, pre) : __fmul2_rn(rhohun, uq);
    const float2 F3 = __fmul2_rn(un, __ffma2_rn(__fmul2_rn(bcast(ph.gh), pre), w, t));
    const float2 den = __ffma2_rn(__fmul2_rn(v2, cs2), mone, one);           // 1 - v^2 cs^2
    const float2 inv = pair(1.0f / den.x, 1.0f / den.y);
    const float2 lm = __fmul2_rn(__ffma2_rn(b, mone, a), inv);
    const float2 lp = __fmul2_rn(__fadd2_rn(a, b), inv);
    const float2 sU = __fmul2_rn(s, w), sF = __fmul2_rn(s, un);
    L.U[0] = d.x; R.U[0] = d.y;
    L.U[1] = U1.x; R.U[1] = U1.y;
    L.U[2] = U2.x; R.U[2] = U2.y;
    L.U[3] = U3.x; R.U[3] = U3.y;
    L.F[0] = F0.x; R.F[0] = F0.y;
    L.F[1] = F1.x; R.F[1] = F1.y;
    L.F[2] = F2.x; R.F[2] = F2.y;
    L.F[3] = F3.x; R.F[3] = F3.y;
    L.lm = lm.x; R.lm = lm.y;
    L.lp = lp.x; R.lp = lp.y;
    L.sU = sU.x; R.sU = sU.y;
    L.sF = sF.x; R.sF = sF.y;
    L.vn = vn.x; R.vn = vn.y;
    L.pre = pre.x; R.pre = pre.y;
}

// HLLE on paired fields (D, S_r), (S_theta, tau) and the scalar alone.
__device__ __forceinline__ void hlle_f32x2(const Side<float>& L, const Side<float>& R, float out[5]) {
    const float am = fminf(L.lm, R.lm);
    const float ap = fmaxf(L.lp, R.lp);
    if (am >= 0.0f) {
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = L.F[q];
        out[4] = L.sF;
    } else if (ap <= 0.0f) {
#pragma unroll
        for (int q = 0; q < 4; ++q) out[q] = R.F[q];
        out[4] = R.sF;
    } else {
        const float inv = 1.0f / (ap - am);
        const float apam = ap * am;
        const float2 AP = bcast(ap), MAM = bcast(-am), APAM = bcast(apam), INV = bcast(inv);
#pragma unroll
        for (int q = 0; q < 4; q += 2) {
            const float2 fl = pair(L.F[q], L.F[q + 1]), fr = pair(R.F[q], R.F[q + 1]);
            const float2 du = __fadd2_rn(pair(R.U[q], R.U[q + 1]), __fmul2_rn(pair(L.U[q], L.U[q + 1]), bcast(-1.0f)));
            const float2 o = __fmul2_rn(__ffma2_rn(APAM, du, __ffma2_rn(MAM, fr, __fmul2_rn(AP, fl))), INV);
            out[q] = o.x;
            out[q + 1] = o.y;
        }
        out[4] = (ap * L.sF - am * R.sF + apam * (R.sU - L.sU)) * inv;
    }
}

template <int AXIS>
__device__ __forceinline__ void riemann_srhd_f32(const PhysT<float>& ph, const float* pl, const float* pr,
                                                 float sl, float sr, float out[5]) {
    Side<float> L, Rr;
    srhd_sides_f32x2<AXIS>(ph, pl, pr, sl, sr, L, Rr);
    if (ph.hllc) srhd_hllc(L, Rr, AXIS, out);
    else hlle_f32x2(L, Rr, out);
}

// Geometric sources per unit volume for the FP32 relativistic stage: the
// enthalpy density rho h = rho + gh p without a division.
__device__ __forceinline__ void sources_srhd_f32(const PhysT<float>& ph, const float* P, float r, float cot,
                                                 float S[4]) {
    const float rho = P[0], ur = P[1], uq = P[2], pre = P[3];
    const float mass = rho + pre * ph.gh;
    const float ir = 1.0f / r;
    S[0] = 0.0f;
    S[1] = (2.0f * pre + mass * uq * uq) * ir;
    S[2] = (pre * cot - mass * ur * uq) * ir;
    S[3] = 0.0f;
}

// Geometric sources per unit volume (before LIGHT_SPEED and dV).
template <class R>
__device__ __forceinline__ void sources(const PhysT<R>& ph, const R* P, R r, R cot, R S[4]) {
    const R rho = P[0], ur = P[1], uq = P[2], pre = P[3];
    const R mass = ph.srhd ? rho * (R(1) + pre / rho * ph.gh) : rho;
    S[0] = R(0);
    S[1] = (R(2) * pre + mass * uq * uq) / r;
    S[2] = (pre * cot - mass * ur * uq) / r;
    S[3] = R(0);
}

template <class R>
__device__ __forceinline__ void prim_to_cons(const PhysT<R>& ph, const R* P, R* U) {
    if (ph.srhd) {
        const R rho = P[0], ur = P[1], uq = P[2], pre = P[3];
        const R uu = ur * ur + uq * uq;
        const R w = rsqrt_(R(1) + uu);
        const R h = R(1) + pre / rho * ph.gh;
        const R d = rho * w;
        const R m = d * h;
        U[0] = d;
        U[1] = m * ur;
        U[2] = m * uq;
        U[3] = m * w - pre - d;
    } else {
        const R rho = P[0], vr = P[1], vq = P[2], pre = P[3];
        U[0] = rho;
        U[1] = rho * vr;
        U[2] = rho * vq;
        U[3] = pre / ph.gm1 + R(0.5) * rho * (vr * vr + vq * vq);
    }
}

template <class R>
__device__ __forceinline__ R lorentz_factor(const PhysT<R>& ph, const R* P) {
    if (!ph.srhd) return R(1);
    return rsqrt_(R(1) + P[1] * P[1] + P[2] * P[2]);
}

// SRHD cons -> prim, FP64 (the plain path; the oracle runs the same
// expressions in the same order): Newton-Raphson on p (Marti & Mueller 2003
// section 6), |f| < 1e-12 (D + tau), at most 50 iterations, each with three
// divisions and a square root: with 1 - v^2 = 1/W^2, rho e = X / W^2 for
// X = tau + m (1 - W) + p (1 - W^2), rho h = m / W + rho e + p and
// f / f' = f rho h / (v^2 gamma p - rho h). Returns HYDRO_* and the
// iteration count.
__device__ __forceinline__ int srhd_c2p_newton(double gm, const double* U, double guess, double* P,
                                               int& iterations, double& bad) {
    const double m = U[0];
    const double tau = U[3];
    iterations = 0;
    if (m < 0.0) { bad = m; return HYDRO_NEGATIVE_DENSITY; }
    if (tau < 0.0) { bad = tau; return HYDRO_NEGATIVE_ENERGY_DENSITY; }
    const double ss = U[1] * U[1] + U[2] * U[2];
    const double tol = NEWTON_TOLERANCE * (m + tau);
    double p = guess;
    double w0 = 1.0;
    bool found = false;
    for (int n = 0; n < NEWTON_ITER_MAX; ++n) {
        const double et = tau + p + m;
        const double inv = 1.0 / et;
        const double b2 = fmin(ss * inv * inv, 1.0 - 1e-10);
        const double omb = 1.0 - b2;
        const double w2 = 1.0 / omb;
        const double w = sqrt(w2);
        const double de = (tau + m * (1.0 - w) + p * (1.0 - w2)) * omb;
        const double dh = m * omb * w + de + p;
        const double f = de * (gm - 1.0) - p;
        p -= f * dh / (b2 * gm * p - dh);
        iterations = n + 1;
        if (fabs(f) < tol) { w0 = w; found = true; break; }
    }
    if (!found) { bad = m; return HYDRO_ROOT_FINDER_FAILED; }
    const double et = tau + m + p;
    P[0] = m / w0;
    P[1] = w0 * U[1] / et;
    P[2] = w0 * U[2] / et;
    P[3] = p;
    if (p < 0.0) {
        P[3] = PRESSURE_FLOOR * P[0];
        return HYDRO_NEGATIVE_PRESSURE;
    }
    return HYDRO_NONE;
}

// Newton-Raphson on the pressure, the reference's iteration rewritten with two
// divisions: with X = tau + m (1 - W) + p (1 - W^2) and 1 - v^2 = 1/W^2,
// rho e = X / W^2, f = (gamma - 1) rho e - p, rho h = m / W + rho e + p and
// f / f' = f rho h / (v^2 gamma p - rho h). Converged when |f| < tol_abs or the
// step is below tol_rel |p| (FP32 only; tol_rel = 0 reproduces the reference's
// criterion). Returns the root and W at the last evaluated pressure.
template <class R>
__device__ __forceinline__ bool newton_fast(R m, R ss, R tau, R gm, R p, R tol_abs, R tol_rel, int maxit, R& p_out,
                                            R& w_out, int& iters) {
    const R bmax = sizeof(R) == 8 ? R(1.0 - 1e-10) : R(1.0f - 1e-6f);
    for (int n = 0; n < maxit; ++n) {
        const R et = tau + p + m;
        const R inv = R(1) / et;
        const R b2 = rmin(ss * inv * inv, bmax);
        const R omb = R(1) - b2;
        const R w = sizeof(R) == 8 ? (R)rsqrt((double)omb) : (R)rsqrtf((float)omb);
        const R w2 = w * w;
        const R X = tau + m * (R(1) - w) + p * (R(1) - w2);
        const R de = X * omb;
        const R f = (gm - R(1)) * de - p;
        const R dh = m * omb * w + de + p;
        const R den = b2 * gm * p - dh;
        const R step = f * dh / den;
        p = p - step;
        iters = n + 1;
        if (rabs(f) < tol_abs || rabs(step) <= tol_rel * rabs(p)) {
            p_out = p;
            w_out = w;
            return p == p;   // false for NaN
        }
    }
    return false;
}

template <class R>
__device__ __forceinline__ int newt_c2p(R gm1, const R* U, R* P, R& bad) {
    const R rho = U[0];
    if (rho < R(0)) { bad = rho; return HYDRO_NEGATIVE_DENSITY; }
    const R vr = U[1] / rho;
    const R vq = U[2] / rho;
    P[0] = rho;
    P[1] = vr;
    P[2] = vq;
    P[3] = (U[3] - R(0.5) * rho * (vr * vr + vq * vq)) * gm1;
    return HYDRO_NONE;
}

// The mixed stage's test for a zone above the Lorentz-factor split, on its
// stored FP32 four-velocity: u_r^2 + u_theta^2 = W^2 - 1 above thr. Every
// launch that stores primitives and every update form evaluates this one
// expression, so they agree zone by zone.
__device__ __forceinline__ bool high_zone(float ur, float uq, float thr) {
    return __fmaf_rn(ur, ur, __fmul_rn(uq, uq)) > thr;
}

// Append a stored zone above the split, {slot, padded row x nq + column}, to
// the stage's list (the capacity is every padded zone of the block set, so it
// is never exceeded).
__device__ __forceinline__ void note_high(int2* list, unsigned* count, unsigned cap, int slot, int prow, int nq,
                                          int j) {
    const unsigned k = atomicAdd(count, 1u);
    if (k < cap) list[k] = make_int2(slot, prow * nq + j);
}

// Max signal speed of a primitive state (time_step, state.rs:151-160).
template <class R>
__device__ __forceinline__ R max_signal_speed(const PhysT<R>& ph, const R* P) {
    if (ph.srhd) {
        Side<R> a, b;
        srhd_side(ph, P[0], P[1], P[2], P[3], R(0), 0, a);
        srhd_side(ph, P[0], P[1], P[2], P[3], R(0), 1, b);
        return rmax(rmax(rabs(a.lm), rabs(a.lp)), rmax(rabs(b.lm), rabs(b.lp)));
    }
    const R v = rsqrt_(P[1] * P[1] + P[2] * P[2]);
    return v + rsqrt_(ph.gm * P[3] / P[0]);
}

// Counter-based U[0,1): splitmix64 (Steele, Lea & Flood 2014) of (seed, block, i, j).
__device__ __host__ __forceinline__ uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __host__ __forceinline__ double uniform01(uint64_t seed, int32_t block, int64_t i, int64_t j) {
    uint64_t k = splitmix64(seed);
    k = splitmix64(k ^ (uint64_t)(uint32_t)block);
    k = splitmix64(k ^ (uint64_t)i);
    k = splitmix64(k ^ (uint64_t)j);
    return (double)(k >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace knc
