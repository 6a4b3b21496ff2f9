// knc_oracle.cpp — CPU FP64 oracle of the KNC finite-volume RK stage.
//
// TEST INFRASTRUCTURE ONLY (the checker; never part of the shipped library).
// PARITY UNPINNED: see knc_oracle.h for why no reference output exists.
//
// What follows restates, in order:
//   src/mesh.rs:119-407   geometry (vertices, face areas, volumes, centroids)
//   src/state.rs:55-244   from_model, c2p per block, time_step, weighted average
//   src/scheme.rs:16-240  try_advance_rk, add_remove_blocks, advance
//   src/physics/{mod,relativistic_hydro,newtonian_hydro}.rs  adapters: LIGHT_SPEED scaling, pressure floor, errors
// and writes the un-vendored crate physics from published methods:
//   SRHD prim<->cons, flux, Newton pressure recovery ......... Marti & Mueller,
//        Living Rev. Relativ. 6 (2003) 7, sections 2.1 and 6 (Newton-Raphson on p)
//   SRHD characteristic speeds ................................ Marti & Mueller (2003) eq. (29)
//   HLLE ...................................................... Einfeldt (1988); Harten, Lax & van Leer (1983)
//   relativistic HLLC ......................................... Mignone & Bodo, MNRAS 364 (2005) 126
//   Newtonian HLLE / HLLC ..................................... Toro, Riemann Solvers (3rd ed.) ch. 10
//   generalised-minmod PLM slope .............................. van Leer (1979); Kurganov & Tadmor (2000)
//   spherical-polar geometric sources ......................... divergence of the stress tensor
//                                                               in axisymmetric (r, theta)
//   SSP RK2 / RK3 ............................................. Shu & Osher, JCP 77 (1988) 439
//
// Every floating-point expression is written in one fixed evaluation order and
// compiled with -ffp-contract=off, so the same expression on the GPU (compiled
// without FMA contraction) produces the same bits.

#include "knc_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <tuple>
#include <mutex>
#include <thread>
#include <vector>

namespace {

constexpr double LIGHT_SPEED = 3e10;           // src/physics/mod.rs:7
constexpr double PI = 3.14159265358979323846;   // std::f64::consts::PI
constexpr int NEWTON_ITER_MAX = 50;
constexpr double NEWTON_TOLERANCE = 1e-12;
constexpr double PRESSURE_FLOOR = 1e-3;         // relativistic_hydro.rs:79-81

// ---------------------------------------------------------------- hashing --
// Counter-based uniform U[0,1) keyed on (seed, block, i, j): splitmix64 mixing
// (Steele, Lea & Flood, OOPSLA 2014) of a packed key; 53 high bits.
inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
inline double uniform01(uint64_t seed, int32_t block, int64_t i, int64_t j) {
    uint64_t k = splitmix64(seed);
    k = splitmix64(k ^ (uint64_t)(uint32_t)block);
    k = splitmix64(k ^ (uint64_t)i);
    k = splitmix64(k ^ (uint64_t)j);
    return (double)(k >> 11) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------- physics --
struct Phys {
    int system;
    int riemann;
    double gm;     // gamma_law_index
    double gh;     // gm / (gm - 1)
    double gm1;    // gm - 1
    double plm_theta;
};

Phys make_phys(const knc_hydro_params* h) {
    Phys p;
    p.system = h->system;
    p.riemann = h->riemann_solver;
    p.gm = h->gamma_law_index;
    p.gm1 = h->gamma_law_index - 1.0;
    p.gh = h->gamma_law_index / p.gm1;
    p.plm_theta = h->plm_theta;
    return p;
}

struct Prim { double v[4]; };   // SRHD (rho, u_r, u_q, p); Newtonian (rho, v_r, v_q, p)
struct Cons { double v[4]; };   // SRHD (D, S_r, S_q, tau); Newtonian (rho, m_r, m_q, E)

// godunov_core::piecewise_linear::plm_gradient — generalised minmod of the
// three one-sided / centred differences (van Leer; Kurganov & Tadmor).
inline double plm_gradient(double theta, double a, double b, double c) {
    const double x = theta * (b - a);
    const double y = 0.5 * (c - a);
    const double z = theta * (c - b);
    if (x > 0.0 && y > 0.0 && z > 0.0) return std::min(x, std::min(y, z));
    if (x < 0.0 && y < 0.0 && z < 0.0) return std::max(x, std::max(y, z));
    return 0.0;
}

// SRHD prim -> cons (Marti & Mueller 2003 eq. 3-5), h = 1 + gamma/(gamma-1) p/rho.
inline Cons srhd_p2c(const Phys& ph, const Prim& P) {
    const double rho = P.v[0], ur = P.v[1], uq = P.v[2], pre = P.v[3];
    const double uu = ur * ur + uq * uq;
    const double w = std::sqrt(1.0 + uu);
    const double h = 1.0 + pre / rho * ph.gh;
    const double d = rho * w;
    const double m = d * h;
    Cons U;
    U.v[0] = d;
    U.v[1] = m * ur;
    U.v[2] = m * uq;
    U.v[3] = m * w - pre - d;
    return U;
}

inline Cons newt_p2c(const Phys& ph, const Prim& P) {
    const double rho = P.v[0], vr = P.v[1], vq = P.v[2], pre = P.v[3];
    Cons U;
    U.v[0] = rho;
    U.v[1] = rho * vr;
    U.v[2] = rho * vq;
    U.v[3] = pre / ph.gm1 + 0.5 * rho * (vr * vr + vq * vq);
    return U;
}

inline Cons p2c(const Phys& ph, const Prim& P) {
    return ph.system == KNC_SYSTEM_RELATIVISTIC ? srhd_p2c(ph, P) : newt_p2c(ph, P);
}

inline double lorentz_factor(const Phys& ph, const Prim& P) {
    if (ph.system != KNC_SYSTEM_RELATIVISTIC) return 1.0;     // newtonian_hydro.rs:124-128
    return std::sqrt(1.0 + P.v[1] * P.v[1] + P.v[2] * P.v[2]); // relativistic_hydro.rs:162-164
}

// SRHD cons -> prim: Newton-Raphson on the pressure (Marti & Mueller 2003 §6),
// f(p) = rho e (gamma-1) - p with rho, e, W recovered at the trial p; df/dp
// approximated by v^2 c_s^2 - 1. Converged when |f| < 1e-12 (D + tau).
// Each step takes three divisions and a square root: with 1 - v^2 = 1/W^2,
// rho e = X / W^2 for X = tau + m (1 - W) + p (1 - W^2), rho h = m / W +
// rho e + p and f / f' = f rho h (v^2 gamma p - rho h)^-1 (the same iteration
// as the textbook form's seven divisions, rounded differently; which form the
// reference's un-vendored crate uses is not known).
// Plain guess p = 0 (the only guess the conserved state alone provides).
// Returns KNC_HYDRO_NONE, NEGATIVE_PRESSURE (floored), or an error kind.
int srhd_c2p(const Phys& ph, const Cons& U, double guess, Prim& P, int& iterations,
             double& bad_value) {
    const double m = U.v[0];
    const double tau = U.v[3];
    iterations = 0;
    if (m < 0.0) { bad_value = m; return KNC_HYDRO_NEGATIVE_DENSITY; }
    if (tau < 0.0) { bad_value = tau; return KNC_HYDRO_NEGATIVE_ENERGY_DENSITY; }
    const double gm = ph.gm;
    const double ss = U.v[1] * U.v[1] + U.v[2] * U.v[2];
    const double tol = NEWTON_TOLERANCE * (m + tau);
    double p = guess;
    double w0 = 1.0;
    bool found = false;
    for (int n = 0; n < NEWTON_ITER_MAX; ++n) {
        const double et = tau + p + m;
        const double inv = 1.0 / et;
        const double b2 = std::min(ss * inv * inv, 1.0 - 1e-10);
        const double omb = 1.0 - b2;
        const double w2 = 1.0 / omb;
        const double w = std::sqrt(w2);
        const double de = (tau + m * (1.0 - w) + p * (1.0 - w2)) * omb;
        const double dh = m * omb * w + de + p;
        const double f = de * (gm - 1.0) - p;
        p -= f * dh / (b2 * gm * p - dh);
        iterations = n + 1;
        if (std::fabs(f) < tol) { w0 = w; found = true; break; }
    }
    if (!found) { bad_value = m; return KNC_HYDRO_ROOT_FINDER_FAILED; }
    const double et = tau + m + p;
    P.v[0] = m / w0;
    P.v[1] = w0 * U.v[1] / et;
    P.v[2] = w0 * U.v[2] / et;
    P.v[3] = p;
    if (p < 0.0) {
        P.v[3] = PRESSURE_FLOOR * P.v[0];
        return KNC_HYDRO_NEGATIVE_PRESSURE;
    }
    return KNC_HYDRO_NONE;
}

int newt_c2p(const Phys& ph, const Cons& U, Prim& P, double& bad_value) {
    const double rho = U.v[0];
    if (rho < 0.0) { bad_value = rho; return KNC_HYDRO_NEGATIVE_DENSITY; }  // newtonian_hydro.rs:55-59
    const double vr = U.v[1] / rho;
    const double vq = U.v[2] / rho;
    P.v[0] = rho;
    P.v[1] = vr;
    P.v[2] = vq;
    P.v[3] = (U.v[3] - 0.5 * rho * (vr * vr + vq * vq)) * ph.gm1;
    return KNC_HYDRO_NONE;
}

// One side of an interface: conserved state, physical flux along `axis`,
// the two outer characteristic speeds, and the passive scalar's conserved
// density (s W) and flux (s u_n). The scalar is advected like the lab-frame
// density: the reference reconstructs s = scalar_mass / dV / W (scheme.rs:35).
struct Side {
    double U[4], F[4], lm, lp, sU, sF, vn, pre;
};

inline Side srhd_side(const Phys& ph, const Prim& P, double s, int axis) {
    const double rho = P.v[0], ur = P.v[1], uq = P.v[2], pre = P.v[3];
    const double uu = ur * ur + uq * uq;
    const double w2 = 1.0 + uu;
    const double w = std::sqrt(w2);
    const double h = 1.0 + pre / rho * ph.gh;
    const double d = rho * w;
    const double m = d * h;
    const double un = axis == 0 ? ur : uq;
    const double vn = un / w;
    Side S;
    S.U[0] = d;
    S.U[1] = m * ur;
    S.U[2] = m * uq;
    S.U[3] = m * w - pre - d;
    S.F[0] = S.U[0] * vn;
    S.F[1] = axis == 0 ? S.U[1] * vn + pre : S.U[1] * vn;
    S.F[2] = axis == 1 ? S.U[2] * vn + pre : S.U[2] * vn;
    S.F[3] = (S.U[3] + pre) * vn;
    // characteristic speeds along the normal (Marti & Mueller 2003 eq. 29)
    const double cs2 = ph.gm * pre / (rho * h);
    const double v2 = uu / w2;
    const double k = 1.0 - cs2;
    const double a = vn * k;
    const double b = std::sqrt(cs2 * (1.0 - v2) * (1.0 - v2 * cs2 - vn * vn * k));
    const double inv = 1.0 / (1.0 - v2 * cs2);
    S.lm = (a - b) * inv;
    S.lp = (a + b) * inv;
    S.sU = s * w;
    S.sF = s * un;
    S.vn = vn;
    S.pre = pre;
    return S;
}

inline Side newt_side(const Phys& ph, const Prim& P, double s, int axis) {
    const double rho = P.v[0], vr = P.v[1], vq = P.v[2], pre = P.v[3];
    const double vn = axis == 0 ? vr : vq;
    Side S;
    S.U[0] = rho;
    S.U[1] = rho * vr;
    S.U[2] = rho * vq;
    S.U[3] = pre / ph.gm1 + 0.5 * rho * (vr * vr + vq * vq);
    S.F[0] = S.U[0] * vn;
    S.F[1] = axis == 0 ? S.U[1] * vn + pre : S.U[1] * vn;
    S.F[2] = axis == 1 ? S.U[2] * vn + pre : S.U[2] * vn;
    S.F[3] = (S.U[3] + pre) * vn;
    const double cs = std::sqrt(ph.gm * pre / rho);
    S.lm = vn - cs;
    S.lp = vn + cs;
    S.sU = s;
    S.sF = s * vn;
    S.vn = vn;
    S.pre = pre;
    return S;
}

inline Side make_side(const Phys& ph, const Prim& P, double s, int axis) {
    return ph.system == KNC_SYSTEM_RELATIVISTIC ? srhd_side(ph, P, s, axis)
                                                : newt_side(ph, P, s, axis);
}

// HLLE (Harten, Lax & van Leer 1983 with Einfeldt's outer speeds).
inline void hlle(const Side& L, const Side& R, double out[5]) {
    const double am = std::min(L.lm, R.lm);
    const double ap = std::max(L.lp, R.lp);
    if (am >= 0.0) {
        for (int q = 0; q < 4; ++q) out[q] = L.F[q];
        out[4] = L.sF;
    } else if (ap <= 0.0) {
        for (int q = 0; q < 4; ++q) out[q] = R.F[q];
        out[4] = R.sF;
    } else {
        const double inv = 1.0 / (ap - am);
        const double apam = ap * am;
        for (int q = 0; q < 4; ++q)
            out[q] = (ap * L.F[q] - am * R.F[q] + apam * (R.U[q] - L.U[q])) * inv;
        out[4] = (ap * L.sF - am * R.sF + apam * (R.sU - L.sU)) * inv;
    }
}

// Relativistic HLLC (Mignone & Bodo 2005): contact speed from the quadratic
// F^E l^2 - (E + F^m) l + m = 0 of the HLL state (eq. 18), written in the
// cancellation-free form l* = 2m / ((E + F^m) + sqrt((E + F^m)^2 - 4 F^E m)),
// star states of eq. (16)-(17) with E = tau + D.
inline void srhd_hllc(const Side& L, const Side& R, int axis, double out[5]) {
    const double am = std::min(L.lm, R.lm);
    const double ap = std::max(L.lp, R.lp);
    if (am >= 0.0) {
        for (int q = 0; q < 4; ++q) out[q] = L.F[q];
        out[4] = L.sF;
        return;
    }
    if (ap <= 0.0) {
        for (int q = 0; q < 4; ++q) out[q] = R.F[q];
        out[4] = R.sF;
        return;
    }
    const int n = axis == 0 ? 1 : 2;
    const int t = axis == 0 ? 2 : 1;
    const double inv = 1.0 / (ap - am);
    const double apam = ap * am;
    double Uh[4], Fh[4];
    for (int q = 0; q < 4; ++q) {
        Uh[q] = (ap * R.U[q] - am * L.U[q] - (R.F[q] - L.F[q])) * inv;
        Fh[q] = (ap * L.F[q] - am * R.F[q] + apam * (R.U[q] - L.U[q])) * inv;
    }
    const double e_hll = Uh[3] + Uh[0];
    const double fe_hll = Fh[3] + Fh[0];
    const double m_hll = Uh[n];
    const double fm_hll = Fh[n];
    const double bq = e_hll + fm_hll;
    const double disc = std::max(bq * bq - 4.0 * fe_hll * m_hll, 0.0);
    const double lstar = 2.0 * m_hll / (bq + std::sqrt(disc));
    const double pstar = fm_hll - fe_hll * lstar;
    const Side& K = lstar >= 0.0 ? L : R;
    const double lam = lstar >= 0.0 ? am : ap;
    const double fac = 1.0 / (lam - lstar);
    const double lv = lam - K.vn;
    const double e_k = K.U[3] + K.U[0];
    double Us[4];
    Us[0] = K.U[0] * lv * fac;
    Us[n] = (K.U[n] * lv + pstar - K.pre) * fac;
    Us[t] = K.U[t] * lv * fac;
    const double e_s = (e_k * lv + pstar * lstar - K.pre * K.vn) * fac;
    Us[3] = e_s - Us[0];
    for (int q = 0; q < 4; ++q) out[q] = K.F[q] + lam * (Us[q] - K.U[q]);
    const double s_star = K.sU * lv * fac;
    out[4] = K.sF + lam * (s_star - K.sU);
}

// Newtonian HLLC (Toro 3rd ed. §10.4, contact speed eq. 10.37).
inline void newt_hllc(const Side& L, const Side& R, int axis, double out[5]) {
    const double am = std::min(L.lm, R.lm);
    const double ap = std::max(L.lp, R.lp);
    if (am >= 0.0) {
        for (int q = 0; q < 4; ++q) out[q] = L.F[q];
        out[4] = L.sF;
        return;
    }
    if (ap <= 0.0) {
        for (int q = 0; q < 4; ++q) out[q] = R.F[q];
        out[4] = R.sF;
        return;
    }
    const int n = axis == 0 ? 1 : 2;
    const int t = axis == 0 ? 2 : 1;
    const double ql = L.U[0] * (am - L.vn);
    const double qr = R.U[0] * (ap - R.vn);
    const double sstar = (R.pre - L.pre + L.U[n] * (am - L.vn) - R.U[n] * (ap - R.vn)) / (ql - qr);
    const Side& K = sstar >= 0.0 ? L : R;
    const double lam = sstar >= 0.0 ? am : ap;
    const double rho = K.U[0];
    const double lv = lam - K.vn;
    const double fac = rho * lv / (lam - sstar);
    double Us[4];
    Us[0] = fac;
    Us[n] = fac * sstar;
    Us[t] = fac * (K.U[t] / rho);
    Us[3] = fac * (K.U[3] / rho + (sstar - K.vn) * (sstar + K.pre / (rho * lv)));
    for (int q = 0; q < 4; ++q) out[q] = K.F[q] + lam * (Us[q] - K.U[q]);
    const double s_star = K.sU * lv / (lam - sstar);
    out[4] = K.sF + lam * (s_star - K.sU);
}

inline void riemann(const Phys& ph, const Prim& pl, const Prim& pr, double sl, double sr,
                    int axis, double out[5]) {
    const Side L = make_side(ph, pl, sl, axis);
    const Side R = make_side(ph, pr, sr, axis);
    if (ph.riemann == KNC_RIEMANN_HLLC) {
        if (ph.system == KNC_SYSTEM_RELATIVISTIC) srhd_hllc(L, R, axis, out);
        else newt_hllc(L, R, axis, out);
    } else {
        hlle(L, R, out);
    }
}

// Geometric source terms per unit volume in axisymmetric spherical polar
// coordinates (conservative form with face-area fluxes): the radial momentum
// gains (2p + T^{qq})/r and the polar momentum (p cot(theta) - T^{rq})/r,
// with T^{ij} = rho h u^i u^j (SRHD) or rho v^i v^j (Newtonian).
inline Cons sources(const Phys& ph, const Prim& P, double r, double cot) {
    const double rho = P.v[0], ur = P.v[1], uq = P.v[2], pre = P.v[3];
    const double mass = ph.system == KNC_SYSTEM_RELATIVISTIC ? rho * (1.0 + pre / rho * ph.gh) : rho;
    Cons S;
    S.v[0] = 0.0;
    S.v[1] = (2.0 * pre + mass * uq * uq) / r;
    S.v[2] = (pre * cot - mass * ur * uq) / r;
    S.v[3] = 0.0;
    return S;
}

inline double max_signal_speed(const Phys& ph, const Prim& P) {
    if (ph.system == KNC_SYSTEM_RELATIVISTIC) {
        const Side a = srhd_side(ph, P, 0.0, 0);
        const Side b = srhd_side(ph, P, 0.0, 1);
        return std::max(std::max(std::fabs(a.lm), std::fabs(a.lp)),
                        std::max(std::fabs(b.lm), std::fabs(b.lp)));
    }
    const double v = std::sqrt(P.v[1] * P.v[1] + P.v[2] * P.v[2]);
    return v + std::sqrt(ph.gm * P.v[3] / P.v[0]);
}

// ---------------------------------------------------------------- mesh ----
// src/mesh.rs restated. Rust's f64::log(self, base) is self.ln() / base.ln().
struct Extent { double r0, r1, q0, q1; };

struct MeshDef {
    knc_mesh_params p;
    double zone_dlogr() const {                       // mesh.rs:341-346
        return p.has_num_radial_zones ? 1.0 / (double)p.num_radial_zones
                                      : PI / (double)p.num_polar_zones;
    }
    double block_dlogr() const { return (double)p.block_size * zone_dlogr(); }
    Extent subgrid_extent(int32_t index) const {      // mesh.rs:358-372
        double q0 = 0.0, q1 = PI;
        if (p.num_polar_zones == 1) { q0 = PI * 0.5 - zone_dlogr(); q1 = PI * 0.5 + zone_dlogr(); }
        Extent e;
        e.r0 = p.reference_radius * std::pow(1.0 + block_dlogr(), (double)index);
        e.r1 = p.reference_radius * std::pow(1.0 + block_dlogr(), (double)index + 1.0);
        e.q0 = q0;
        e.q1 = q1;
        return e;
    }
    double t_start() const { return p.has_excision_delay ? p.excision_delay : 0.0; }
    double inner_excision_surface(double t) const {   // mesh.rs:322-325
        return p.inner_radius + std::max(t - t_start(), 0.0) * p.inner_excision_speed;
    }
    double outer_excision_surface(double t) const {   // mesh.rs:333-336
        return p.outer_radius + std::max(t - t_start(), 0.0) * p.outer_excision_speed;
    }
    bool moving() const { return p.inner_excision_speed > 0.0 || p.outer_excision_speed > 0.0; }
};

// SphericalPolarGrid::vertex_coordinate_signed, mesh.rs:202-210
inline double vertex_r(const Extent& e, int64_t nr, int64_t i) {
    const double y0 = std::log(e.r0) / std::log(10.0);
    const double y1 = std::log(e.r1) / std::log(10.0);
    const double dy = (y1 - y0) / (double)nr;
    return std::pow(10.0, y0 + dy * (double)i);
}
inline double vertex_q(const Extent& e, int64_t nq, int64_t j) {
    const double dq = (e.q1 - e.q0) / (double)nq;
    return e.q0 + dq * (double)j;
}
inline double cell_volume(double r0, double q0, double r1, double q1) {   // mesh.rs:119-123
    const double dcost = -(std::cos(q1) - std::cos(q0));
    return 2.0 * PI * (r1 * r1 * r1 - r0 * r0 * r0) / 3.0 * dcost;
}
inline double face_area(double r0, double q0, double r1, double q1) {     // mesh.rs:125-134
    const double s0 = r0 * std::sin(q0);
    const double s1 = r1 * std::sin(q1);
    const double z0 = r0 * std::cos(q0);
    const double z1 = r1 * std::cos(q1);
    const double ds = s1 - s0;
    const double dz = z1 - z0;
    return PI * (s0 + s1) * std::sqrt(ds * ds + dz * dz);
}

struct Geometry {             // GridGeometry, mesh.rs:22-29 (+ cot of centroid)
    int64_t nr = 0, nq = 0;
    std::vector<double> rv, qv, ar, aq, dv, rc, qc, cot;
};

Geometry make_geometry(const MeshDef& M, int32_t index, int64_t nr, int64_t nq) {   // mesh.rs:246-264
    Geometry G;
    const Extent e = M.subgrid_extent(index);
    G.nr = nr;
    G.nq = nq;
    G.rv.resize(nr + 1);
    G.qv.resize(nq + 1);
    for (int64_t i = 0; i <= nr; ++i) G.rv[i] = vertex_r(e, nr, i);
    for (int64_t j = 0; j <= nq; ++j) G.qv[j] = vertex_q(e, nq, j);
    G.ar.resize((nr + 1) * nq);
    G.aq.resize(nr * (nq + 1));
    G.dv.resize(nr * nq);
    G.rc.resize(nr * nq);
    G.qc.resize(nr * nq);
    G.cot.resize(nq);
    for (int64_t i = 0; i <= nr; ++i)
        for (int64_t j = 0; j < nq; ++j)
            G.ar[i * nq + j] = face_area(G.rv[i], G.qv[j], G.rv[i], G.qv[j + 1]);
    for (int64_t i = 0; i < nr; ++i)
        for (int64_t j = 0; j <= nq; ++j)
            G.aq[i * (nq + 1) + j] = face_area(G.rv[i], G.qv[j], G.rv[i + 1], G.qv[j]);
    for (int64_t i = 0; i < nr; ++i)
        for (int64_t j = 0; j < nq; ++j) {
            G.dv[i * nq + j] = cell_volume(G.rv[i], G.qv[j], G.rv[i + 1], G.qv[j + 1]);
            G.rc[i * nq + j] = std::sqrt(G.rv[i] * G.rv[i + 1]);       // centroid, mesh.rs:157-161
            G.qc[i * nq + j] = 0.5 * (G.qv[j] + G.qv[j + 1]);
        }
    for (int64_t j = 0; j < nq; ++j) {
        const double q = 0.5 * (G.qv[j] + G.qv[j + 1]);
        G.cot[j] = std::cos(q) / std::sin(q);
    }
    return G;
}

// ---------------------------------------------------------------- models --
struct ModelDef {
    knc_model_params p{};
    knc_primitive_at_fn host_fn = nullptr;
    void* host_user = nullptr;
};

// primitive_at / scalar_at (src/traits.rs:145-164) of the device models. The
// noise factor applies to initial data only (noise == true).
void model_eval(const Phys& ph, const ModelDef& Md, double r, double q, double t, bool noise,
                int32_t block, int64_t i, int64_t j, Prim& P, double& scalar) {
    const double* a = Md.p.p;
    scalar = 0.0;
    const double inv_r2 = 1.0 / (r * r);
    double amp = 0.0;
    switch (Md.p.kind) {
    case KNC_MODEL_WIND: {
        double rho = a[0] * inv_r2;
        amp = a[3];
        if (noise && amp != 0.0) rho = rho * (1.0 + amp * uniform01(Md.p.seed, block, i, j));
        P.v[0] = rho;
        P.v[1] = a[1];
        P.v[2] = 0.0;
        P.v[3] = a[2] * rho;
        break;
    }
    case KNC_MODEL_JET: {
        double rho = a[0] * inv_r2;
        amp = a[2];
        if (noise && amp != 0.0) rho = rho * (1.0 + amp * uniform01(Md.p.seed, block, i, j));
        P.v[0] = rho;
        P.v[1] = 0.0;
        P.v[2] = 0.0;
        P.v[3] = a[1] * rho;
        // nozzle inside the injection radius, both poles (jet_in_cloud.rs:172-174)
        const bool nozzle = (q < a[3] || q > PI - a[3]) && r < a[6];
        if (nozzle) {
            const double rj = a[0] * inv_r2 * a[5];
            P.v[0] = rj;
            P.v[1] = std::sqrt(a[4] * a[4] - 1.0);
            P.v[3] = a[1] * rj;
            scalar = 1.0;
        }
        break;
    }
    case KNC_MODEL_SPHERE: {
        double rho = r < a[2] ? a[0] : a[1];
        amp = a[4];
        if (noise && amp != 0.0) rho = rho * (1.0 + amp * uniform01(Md.p.seed, block, i, j));
        P.v[0] = rho;
        P.v[1] = 0.0;
        P.v[2] = 0.0;
        P.v[3] = a[3];
        scalar = r < a[2] ? 1.0 : 0.0;
        break;
    }
    case KNC_MODEL_JET_IN_CLOUD: {           // src/models/jet_in_cloud.rs:74-257
        const double cloud_mass = a[0], delay = a[1], duration = a[2], strength = a[3], theta_j = a[4];
        const double engine_u = a[5], m1 = a[6], slowest = a[7], fastest = a[8], psi = a[9];
        const double engine_beta = engine_u / std::sqrt(1.0 + engine_u * engine_u);
        const double r_interface = slowest * LIGHT_SPEED * t;
        const double v_jet = engine_beta * LIGHT_SPEED;
        const double r_head = v_jet * (t - delay);
        const double r_tail = v_jet * (t - delay - duration);
        const bool in_nozzle = q < theta_j || q > PI - theta_j;
        double u, f;
        if (in_nozzle && r < r_head && r > r_tail) {          // Zone::Jet
            u = engine_u;
            const double engine_gamma = std::sqrt(1.0 + engine_u * engine_u);
            f = strength * cloud_mass / (4.0 * PI * duration) / engine_gamma;
            scalar = 1e2;
        } else if (r > r_interface) {                         // Zone::Envelope
            const double b = std::min(r / t / LIGHT_SPEED, fastest);
            u = b / std::sqrt(1.0 - b * b);
            f = m1 / (4.0 * PI * psi * t) * (std::pow(b, -1.0 / psi) * std::pow(1.0 - b * b, 0.5 / psi - 1.0));
            scalar = 1e-2;
        } else {                                              // Zone::Cloud
            u = slowest / std::sqrt(1.0 - slowest * slowest);
            f = cloud_mass / (4.0 * PI * delay);
            scalar = 1.0;
        }
        const double d = f / (r * r * u) / LIGHT_SPEED;
        P.v[0] = d; P.v[1] = u; P.v[2] = 0.0; P.v[3] = d * 1e-3;
        break;
    }
    case KNC_MODEL_KINETIC_BOMB: {           // src/models/kinetic_bomb.rs:78-114
        const double v = std::sqrt(2.0 * a[3] / a[4]);
        const double dur = a[2] / v;
        if (a[1] + v * (t - dur) <= r && r < a[1] + v * t) {
            const double d = a[4] / dur / (4.0 * PI * r * r * v);
            P.v[0] = d; P.v[1] = v / LIGHT_SPEED; P.v[2] = 0.0; P.v[3] = d * 1e-3;
            scalar = 1.0;
        } else {
            const double x = r / a[1];
            const double d = a[0] * (x * x);
            P.v[0] = d; P.v[1] = 0.0; P.v[2] = 0.0; P.v[3] = d * 1e-3;
            scalar = 0.0;
        }
        break;
    }
    case KNC_MODEL_JET_IN_STAR: {            // src/models/jet_in_star.rs:87-236
        const double R0 = 7e10, M0 = 2e33;
        const double RHO_C = 3e7 * M0 / (1.33 * PI * R0 * R0 * R0);
        const double R1 = 0.0017 * R0, R2 = 0.0125 * R0, R3 = 0.65 * R0;
        const double RHO_WIND = 1e-9 * M0 / (1.33 * PI * R0 * R0 * R0);
        const double R_NOZZ = 0.01 * R0, R_ENV = 1.2 * R0;
        const double engine_u = a[4], theta_j = a[3], env_radius = a[5];
        const double rho_env = a[6] / (4.0 * PI * (env_radius * env_radius) * (env_radius - R3) * a[7]);
        const double r_head = engine_u / std::sqrt(1.0 + engine_u * engine_u) * LIGHT_SPEED * t;
        const bool in_nozzle = q < theta_j || q > PI - theta_j;
        double d, u = 0.0;
        if (in_nozzle && r < r_head) {
            const double r0 = R_NOZZ / R0;
            const double q2 = theta_j * theta_j;
            const double n0 = 4.0 * PI * r0 * r0 * r0 * (1.0 - std::exp(-2.0 / q2)) * q2;
            const double g = (r / R_NOZZ) * std::exp(-std::pow(r / R_NOZZ, 2.0) / 2.0) *
                             std::exp((std::pow(std::cos(q), 2.0) - 1.0) / q2);
            const double l = g / n0 * a[2] / (4.0 * PI * a[1]);
            const double rate = l / (std::sqrt(1.0 + engine_u * engine_u) * LIGHT_SPEED * LIGHT_SPEED);
            d = rate / (r * r * engine_u * LIGHT_SPEED);
            u = engine_u;
            scalar = 1e2;
        } else if (r < R3) {
            const double core = RHO_C * std::pow(1.0 - r / R3, 16.7) /
                                (1.0 + std::pow(r / R1, 3.24) / (1.0 + std::pow(r / R2, 2.57)));
            d = core + rho_env * std::pow(r / R3, -2.0);
            scalar = 1.0;
        } else if (R3 < r && r < env_radius) {
            d = rho_env * std::pow(r / R3, -2.5);
            scalar = 1e-2 * std::pow(r / R3, -2.0);
        } else {
            d = RHO_WIND * std::pow(r / R_ENV, -2.0);
            scalar = 1e-5 * std::pow(r / R_ENV, -2.0);
        }
        P.v[0] = d; P.v[1] = u; P.v[2] = 0.0; P.v[3] = d * 1e-10;
        break;
    }
    case KNC_MODEL_HOST: {
        double any[4];
        Md.host_fn(r, q, t, any, &scalar, Md.host_user);
        // Hydrodynamics::interpret: AnyPrimitive [u_r, u_q, rho, p] -> (rho, u_r, u_q, p)
        P.v[0] = any[2];
        P.v[1] = any[0];
        P.v[2] = any[1];
        P.v[3] = any[3];
        break;
    }
    default:
        P.v[0] = 1.0; P.v[1] = 0.0; P.v[2] = 0.0; P.v[3] = 1.0;
    }
    (void)ph;
}

// ---------------------------------------------------------------- state ---
struct Block {
    std::vector<double> U;   // [nr][nq][4] volume-integrated, reference AoS order
    std::vector<double> S;   // [nr][nq] scalar mass
};

struct ErrorRec {
    int kind = KNC_HYDRO_NONE;
    int32_t block = 0;
    int64_t i = 0, j = 0;
    double r = 0, q = 0, value = 0;
};

struct Rational {
    int64_t n = 0, d = 1;
    static int64_t gcd(int64_t a, int64_t b) { if (a < 0) a = -a; if (b < 0) b = -b; while (b) { int64_t t = a % b; a = b; b = t; } return a ? a : 1; }
    void norm() { int64_t g = gcd(n, d); n /= g; d /= g; if (d < 0) { n = -n; d = -d; } }
    Rational add(const Rational& o) const { Rational r; r.n = n * o.d + o.n * d; r.d = d * o.d; r.norm(); return r; }
    Rational mul(const Rational& o) const { Rational r; r.n = n * o.n; r.d = d * o.d; r.norm(); return r; }
};

// Prims of one block: [nr][nq] primitive + scalar density s = S / dV / W.
struct PrimBlock {
    std::vector<Prim> P;
    std::vector<double> s;
};

}  // namespace

struct oracle_ctx {
    knc_hydro_params hp{};
    Phys ph{};
    MeshDef mesh{};
    ModelDef model{};
    int threads = 1;
    double time = 0.0;
    Rational iteration;
    std::map<int32_t, Block> blocks;
    std::map<std::tuple<int32_t, int64_t, int64_t>, Geometry> geom;
    std::map<int32_t, std::pair<int64_t, int64_t>> shapes;   // uneven blocks: index -> (nr, nq)
    ErrorRec err;
    std::atomic<int64_t> c2p_zones{0}, c2p_iters{0};
};

namespace {

std::pair<int64_t, int64_t> shape_of(const oracle_ctx* c, int32_t index) {
    auto it = c->shapes.find(index);
    if (it != c->shapes.end()) return it->second;
    return {c->mesh.p.block_size, c->mesh.p.num_polar_zones};
}

const Geometry& geometry_of(oracle_ctx* c, int32_t index, int64_t nr, int64_t nq) {
    const auto key = std::make_tuple(index, nr, nq);
    auto it = c->geom.find(key);
    if (it == c->geom.end()) it = c->geom.emplace(key, make_geometry(c->mesh, index, nr, nq)).first;
    return it->second;
}

const Geometry& geometry_of(oracle_ctx* c, int32_t index) {
    const auto sh = shape_of(c, index);
    return geometry_of(c, index, sh.first, sh.second);
}

template <class F>
void parallel_for(int threads, int64_t n, F&& fn) {
    if (threads <= 1 || n <= 1) {
        for (int64_t k = 0; k < n; ++k) fn(k);
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> pool;
    const int nt = (int)std::min<int64_t>(threads, n);
    pool.reserve(nt);
    for (int t = 0; t < nt; ++t)
        pool.emplace_back([&]() {
            for (;;) {
                const int64_t k = next.fetch_add(1);
                if (k >= n) break;
                fn(k);
            }
        });
    for (auto& th : pool) th.join();
}

// BlockState::from_model, state.rs:55-69
Block block_from_model(oracle_ctx* c, int32_t index, const Geometry& G, double t, bool noise) {
    Block B;
    const int64_t nr = G.nr, nq = G.nq;
    B.U.resize(nr * nq * 4);
    B.S.resize(nr * nq);
    for (int64_t i = 0; i < nr; ++i)
        for (int64_t j = 0; j < nq; ++j) {
            const int64_t z = i * nq + j;
            Prim P;
            double scalar;
            model_eval(c->ph, c->model, G.rc[z], G.qc[z], t, noise, index, i, j, P, scalar);
            const Cons U = p2c(c->ph, P);
            for (int q = 0; q < 4; ++q) B.U[z * 4 + q] = U.v[q] * G.dv[z];
            B.S[z] = B.U[z * 4 + 0] * scalar;
        }
    return B;
}

// BlockState::try_to_primitive (state.rs:76-94) + scalar density (scheme.rs:35).
// Records the first error in (i, j) order; returns false on error.
bool block_to_primitive(oracle_ctx* c, int32_t index, const Block& B, const Geometry& G,
                        PrimBlock& out, ErrorRec& e) {
    const int64_t n = G.nr * G.nq;
    out.P.resize(n);
    out.s.resize(n);
    int64_t iters = 0;
    for (int64_t z = 0; z < n; ++z) {
        Cons u;
        for (int q = 0; q < 4; ++q) u.v[q] = B.U[z * 4 + q] / G.dv[z];
        int kind;
        double bad = 0.0;
        int it = 0;
        if (c->ph.system == KNC_SYSTEM_RELATIVISTIC) kind = srhd_c2p(c->ph, u, 0.0, out.P[z], it, bad);
        else kind = newt_c2p(c->ph, u, out.P[z], bad);
        iters += it;
        if (kind != KNC_HYDRO_NONE && kind != KNC_HYDRO_NEGATIVE_PRESSURE) {
            e.kind = kind;
            e.block = index;
            e.i = z / G.nq;
            e.j = z % G.nq;
            e.r = G.rc[z];
            e.q = G.qc[z];
            e.value = bad;
            return false;
        }
        out.s[z] = B.S[z] / G.dv[z] / lorentz_factor(c->ph, out.P[z]);
    }
    c->c2p_zones += n;
    c->c2p_iters += iters;
    return true;
}

// scheme.rs:68-158 for one block: halo assembly, PLM in r and theta, Godunov
// fluxes times face areas, sources times volume, conserved update.
// Halo value at column j of a block with nq columns, from row `row` of a
// neighbour with nq_n columns (a power-of-two ratio; the reference has one
// polar resolution everywhere, so this is the uneven-block extension):
//  - a finer neighbour: its R = nq_n / nq zones are merged conservatively
//    (volume integrals and volumes summed in column order) and recovered;
//  - a coarser neighbour: its zone j / R is copied (piecewise constant).
void halo_value(oracle_ctx* c, int64_t nq, int64_t j, const PrimBlock& pn, const Block* bn, const Geometry* gn,
                int64_t nq_n, int64_t row, Prim& P, double& s) {
    if (nq_n == nq) {
        P = pn.P[row * nq + j];
        s = pn.s[row * nq + j];
        return;
    }
    if (nq_n < nq) {
        const int64_t z = row * nq_n + j / (nq / nq_n);
        P = pn.P[z];
        s = pn.s[z];
        return;
    }
    const int64_t R = nq_n / nq;
    double U[5] = {0, 0, 0, 0, 0}, dv = 0.0;
    for (int64_t m = 0; m < R; ++m) {
        const int64_t z = row * nq_n + j * R + m;
        for (int q = 0; q < 4; ++q) U[q] += bn->U[z * 4 + q];
        U[4] += bn->S[z];
        dv += gn->dv[z];
    }
    Cons u;
    for (int q = 0; q < 4; ++q) u.v[q] = U[q] / dv;
    double bad;
    int it = 0;
    if (c->ph.system == KNC_SYSTEM_RELATIVISTIC) srhd_c2p(c->ph, u, 0.0, P, it, bad);
    else newt_c2p(c->ph, u, P, bad);
    s = U[4] / dv / lorentz_factor(c->ph, P);
}

struct Neighbour {
    const PrimBlock* prims;
    const Block* block;        // conserved state (null for a ghost block)
    const Geometry* geom;
    int64_t nr, nq;
};

void block_update(oracle_ctx* c, const Block& B, const Geometry& G, const Neighbour& L, const PrimBlock& p0,
                  const Neighbour& Rn, double dt, Block& out) {
    const Phys& ph = c->ph;
    const bool srhd = ph.system == KNC_SYSTEM_RELATIVISTIC;
    const double cflux = srhd ? LIGHT_SPEED : 1.0;
    const int64_t nr = G.nr, nq = G.nq;
    // pe: rows pl[-2..], p0, pr[..2]  (scheme.rs:76-77)
    const int64_t ne = nr + 4;
    std::vector<Prim> pe(ne * nq);
    std::vector<double> se(ne * nq);
    for (int64_t k = 0; k < ne; ++k)
        for (int64_t j = 0; j < nq; ++j) {
            if (k < 2) {
                halo_value(c, nq, j, *L.prims, L.block, L.geom, L.nq, L.nr - 2 + k, pe[k * nq + j], se[k * nq + j]);
            } else if (k < nr + 2) {
                const int64_t z = (k - 2) * nq + j;
                pe[k * nq + j] = p0.P[z];
                se[k * nq + j] = p0.s[z];
            } else {
                halo_value(c, nq, j, *Rn.prims, Rn.block, Rn.geom, Rn.nq, k - nr - 2, pe[k * nq + j], se[k * nq + j]);
            }
        }
    const double th = ph.plm_theta;
    // radial gradients gx: rows 0..nr+2 centred on pe rows 1..nr+2 (scheme.rs:79-80)
    std::vector<Prim> gx((nr + 2) * nq);
    std::vector<double> hx((nr + 2) * nq);
    for (int64_t k = 0; k < nr + 2; ++k)
        for (int64_t j = 0; j < nq; ++j) {
            const int64_t a = k * nq + j, b = (k + 1) * nq + j, cc = (k + 2) * nq + j;
            for (int q = 0; q < 4; ++q)
                gx[k * nq + j].v[q] = plm_gradient(th, pe[a].v[q], pe[b].v[q], pe[cc].v[q]);
            hx[k * nq + j] = plm_gradient(th, se[a], se[b], se[cc]);
        }
    // radial Godunov fluxes times face areas (scheme.rs:81-97), nr+1 faces
    std::vector<double> fx((nr + 1) * nq * 5);
    for (int64_t f = 0; f <= nr; ++f)
        for (int64_t j = 0; j < nq; ++j) {
            const int64_t zl = (f + 1) * nq + j, zr = (f + 2) * nq + j;
            Prim PL, PR;
            for (int q = 0; q < 4; ++q) {
                PL.v[q] = pe[zl].v[q] + gx[f * nq + j].v[q] * 0.5;
                PR.v[q] = pe[zr].v[q] - gx[(f + 1) * nq + j].v[q] * 0.5;
            }
            const double SL = se[zl] + hx[f * nq + j] * 0.5;
            const double SR = se[zr] - hx[(f + 1) * nq + j] * 0.5;
            double flux[5];
            riemann(ph, PL, PR, SL, SR, 0, flux);
            const double A = G.ar[f * nq + j];
            for (int q = 0; q < 5; ++q) fx[(f * nq + j) * 5 + q] = flux[q] * cflux * A;
        }
    const bool one_dimensional = nq == 1;   // scheme.rs:45
    std::vector<double> fy;
    if (!one_dimensional) {
        // polar gradients: zero on the first and last column (extend_default_2d)
        std::vector<Prim> gy(nr * nq);
        std::vector<double> hy(nr * nq);
        for (int64_t i = 0; i < nr; ++i)
            for (int64_t j = 0; j < nq; ++j) {
                const int64_t k = i + 2;
                if (j == 0 || j == nq - 1) {
                    for (int q = 0; q < 4; ++q) gy[i * nq + j].v[q] = 0.0;
                    hy[i * nq + j] = 0.0;
                    continue;
                }
                const int64_t a = k * nq + j - 1, b = k * nq + j, cc = k * nq + j + 1;
                for (int q = 0; q < 4; ++q)
                    gy[i * nq + j].v[q] = plm_gradient(th, pe[a].v[q], pe[b].v[q], pe[cc].v[q]);
                hy[i * nq + j] = plm_gradient(th, se[a], se[b], se[cc]);
            }
        // polar fluxes on interior faces; zero flux at both poles (scheme.rs:112-128)
        fy.assign(nr * (nq + 1) * 5, 0.0);
        for (int64_t i = 0; i < nr; ++i)
            for (int64_t f = 1; f < nq; ++f) {
                const int64_t k = i + 2;
                const int64_t zl = k * nq + f - 1, zr = k * nq + f;
                Prim PL, PR;
                for (int q = 0; q < 4; ++q) {
                    PL.v[q] = pe[zl].v[q] + gy[i * nq + f - 1].v[q] * 0.5;
                    PR.v[q] = pe[zr].v[q] - gy[i * nq + f].v[q] * 0.5;
                }
                const double SL = se[zl] + hy[i * nq + f - 1] * 0.5;
                const double SR = se[zr] - hy[i * nq + f] * 0.5;
                double flux[5];
                riemann(ph, PL, PR, SL, SR, 1, flux);
                const double A = G.aq[i * (nq + 1) + f];
                for (int q = 0; q < 5; ++q) fy[(i * (nq + 1) + f) * 5 + q] = flux[q] * cflux * A;
            }
    }
    // sources, update (scheme.rs:130-157)
    out.U.resize(B.U.size());
    out.S.resize(B.S.size());
    for (int64_t i = 0; i < nr; ++i)
        for (int64_t j = 0; j < nq; ++j) {
            const int64_t z = i * nq + j;
            const Cons src = sources(ph, p0.P[z], G.rc[z], G.cot[j]);
            const double* a = &fx[(i * nq + j) * 5];
            const double* b = &fx[((i + 1) * nq + j) * 5];
            for (int q = 0; q < 4; ++q) {
                const double sc = src.v[q] * cflux * G.dv[z];
                double du;
                if (one_dimensional) du = (sc - (b[q] - a[q])) * dt;
                else {
                    const double* cc = &fy[(i * (nq + 1) + j) * 5];
                    const double* d = &fy[(i * (nq + 1) + j + 1) * 5];
                    du = (sc - (b[q] - a[q]) - (d[q] - cc[q])) * dt;
                }
                out.U[z * 4 + q] = B.U[z * 4 + q] + du;
            }
            double ds;
            if (one_dimensional) ds = (b[4] - a[4]) * -dt;
            else {
                const double* cc = &fy[(i * (nq + 1) + j) * 5];
                const double* d = &fy[(i * (nq + 1) + j + 1) * 5];
                ds = ((b[4] - a[4]) + (d[4] - cc[4])) * -dt;
            }
            out.S[z] = B.S[z] + ds;
        }
}

struct StateView {
    double time;
    Rational iteration;
    std::map<int32_t, Block> blocks;
};

// try_advance_rk, scheme.rs:16-173. Returns false with c->err set on failure.
bool stage(oracle_ctx* c, const StateView& s, double dt, StateView& out) {
    std::vector<int32_t> idx;
    for (auto& kv : s.blocks) idx.push_back(kv.first);
    const int32_t lo = idx.front() - 1, hi = idx.back() + 1;   // state.rs:128-130
    // ghost blocks take their own radial shape and the adjacent live block's
    // polar resolution; geometry must exist before threads read the map
    std::map<int32_t, const Geometry*> gmap;
    for (int32_t k = idx.front(); k <= idx.back(); ++k) gmap[k] = &geometry_of(c, k);
    gmap[lo] = &geometry_of(c, lo, shape_of(c, lo).first, gmap[idx.front()]->nq);
    gmap[hi] = &geometry_of(c, hi, shape_of(c, hi).first, gmap[idx.back()]->nq);
    std::map<int32_t, PrimBlock> prims;
    for (int32_t k = lo; k <= hi; ++k) prims[k];
    std::vector<ErrorRec> errs(idx.size() + 2);
    std::vector<char> ok(idx.size() + 2, 1);
    // c2p of live blocks and of the two ghost blocks built from the model at the stage time
    parallel_for(c->threads, (int64_t)idx.size() + 2, [&](int64_t k) {
        int32_t bi;
        Block ghost;
        const Block* B;
        if (k < (int64_t)idx.size()) { bi = idx[k]; B = &s.blocks.at(bi); }
        else {
            bi = k == (int64_t)idx.size() ? lo : hi;
            ghost = block_from_model(c, bi, *gmap.at(bi), s.time, false);
            B = &ghost;
        }
        ok[k] = block_to_primitive(c, bi, *B, *gmap.at(bi), prims.at(bi), errs[k]);
    });
    for (size_t k = 0; k < ok.size(); ++k)
        if (!ok[k]) {
            // report the error of the lowest block index (deterministic order)
            ErrorRec best;
            bool have = false;
            for (size_t m = 0; m < ok.size(); ++m)
                if (!ok[m] && (!have || errs[m].block < best.block)) { best = errs[m]; have = true; }
            c->err = best;
            return false;
        }
    out.blocks.clear();
    for (int32_t b : idx) out.blocks[b];
    parallel_for(c->threads, (int64_t)idx.size(), [&](int64_t k) {
        const int32_t b = idx[k];
        auto nb = [&](int32_t n) {
            const Geometry* g = gmap.at(n);
            auto it = s.blocks.find(n);
            return Neighbour{&prims.at(n), it == s.blocks.end() ? nullptr : &it->second, g, g->nr, g->nq};
        };
        block_update(c, s.blocks.at(b), *gmap.at(b), nb(b - 1), prims.at(b), nb(b + 1), dt, out.blocks.at(b));
    });
    out.time = s.time + dt;
    Rational one;
    one.n = 1;
    out.iteration = s.iteration.add(one);
    return true;
}

// WeightedAverage(Async), state.rs:179-244: (1 - b) s1 + b s0 on conserved,
// scalar mass, time and iteration.
void weighted_average(oracle_ctx* c, StateView& s1, Rational br, const StateView& s0) {
    const double bf = (double)br.n / (double)br.d;
    const double w1 = -bf + 1.0;
    std::vector<int32_t> idx;
    for (auto& kv : s1.blocks) idx.push_back(kv.first);
    parallel_for(c->threads, (int64_t)idx.size(), [&](int64_t k) {
        Block& a = s1.blocks.at(idx[k]);
        const Block& b = s0.blocks.at(idx[k]);
        for (size_t z = 0; z < a.U.size(); ++z) a.U[z] = a.U[z] * w1 + b.U[z] * bf;
        for (size_t z = 0; z < a.S.size(); ++z) a.S[z] = a.S[z] * w1 + b.S[z] * bf;
    });
    s1.time = s1.time * w1 + s0.time * bf;
    Rational one;
    one.n = 1;
    Rational mbr = br;
    mbr.n = -mbr.n;
    s1.iteration = s1.iteration.mul(mbr.add(one)).add(s0.iteration.mul(br));
}

// godunov_core::runge_kutta::RungeKuttaOrder::try_advance_async (scheme.rs:237):
// Shu-Osher SSP forms RK1, RK2 (b = 1/2), RK3 (b = 3/4, then 1/3).
bool rk_step(oracle_ctx* c, double dt) {
    StateView s0;
    s0.time = c->time;
    s0.iteration = c->iteration;
    s0.blocks = c->blocks;
    StateView s1, s2;
    const int order = c->hp.runge_kutta_order;
    Rational half; half.n = 1; half.d = 2;
    Rational q34; q34.n = 3; q34.d = 4;
    Rational q13; q13.n = 1; q13.d = 3;
    if (!stage(c, s0, dt, s1)) return false;
    if (order == 1) {
        c->blocks.swap(s1.blocks);
        c->time = s1.time;
        c->iteration = s1.iteration;
        return true;
    }
    if (!stage(c, s1, dt, s2)) return false;
    if (order == 2) {
        weighted_average(c, s2, half, s0);
        c->blocks.swap(s2.blocks);
        c->time = s2.time;
        c->iteration = s2.iteration;
        return true;
    }
    weighted_average(c, s2, q34, s0);
    StateView s3;
    if (!stage(c, s2, dt, s3)) return false;
    weighted_average(c, s3, q13, s0);
    c->blocks.swap(s3.blocks);
    c->time = s3.time;
    c->iteration = s3.iteration;
    return true;
}

// add_remove_blocks, scheme.rs:179-206
void add_remove_blocks(oracle_ctx* c) {
    if (c->blocks.empty()) return;
    const int32_t inner = c->blocks.begin()->first;
    const int32_t outer = c->blocks.rbegin()->first;
    if (c->mesh.subgrid_extent(inner).r1 < c->mesh.inner_excision_surface(c->time)) {
        c->blocks.erase(inner);
    }
    if (c->mesh.subgrid_extent(outer).r1 < c->mesh.outer_excision_surface(c->time)) {
        const int32_t nb = outer + 1;
        c->blocks[nb] = block_from_model(c, nb, geometry_of(c, nb), c->time, false);
    }
}

int validate(const knc_hydro_params* h, const knc_mesh_params* m) {
    if (h->plm_theta < 1.0 || h->plm_theta > 2.0) return KNC_ERR_CONFIG;
    if (h->cfl_number < 0.0 || h->cfl_number > 0.7) return KNC_ERR_CONFIG;
    if (h->runge_kutta_order < 1 || h->runge_kutta_order > 3) return KNC_ERR_CONFIG;
    if (m->reference_radius <= 0.0 || m->inner_radius < 0.0 || m->outer_radius < 0.0) return KNC_ERR_CONFIG;
    if (m->block_size < 2) return KNC_ERR_CONFIG;
    if (m->num_polar_zones != 1 && m->num_polar_zones < 16) return KNC_ERR_CONFIG;
    if (m->num_polar_zones == 1 && !m->has_num_radial_zones) return KNC_ERR_CONFIG;
    if (m->inner_excision_speed < 0.0 || m->outer_excision_speed < 0.0) return KNC_ERR_CONFIG;
    if (m->outer_excision_speed < m->inner_excision_speed) return KNC_ERR_CONFIG;
    return KNC_OK;
}

}  // namespace

// ====================================================================== API
extern "C" {

int oracle_create(const knc_hydro_params* hydro, const knc_mesh_params* mesh, int32_t threads,
                  oracle_ctx** out) {
    if (!hydro || !mesh || !out) return KNC_ERR_INVALID_ARGUMENT;
    const int v = validate(hydro, mesh);
    if (v != KNC_OK) return v;
    oracle_ctx* c = new oracle_ctx();
    c->hp = *hydro;
    c->ph = make_phys(hydro);
    c->mesh.p = *mesh;
    c->threads = threads > 0 ? threads : 1;
    c->iteration.n = 0;
    c->iteration.d = 1;
    *out = c;
    return KNC_OK;
}

void oracle_destroy(oracle_ctx* c) { delete c; }

int oracle_set_model(oracle_ctx* c, const knc_model_params* m) {
    if (!c || !m) return KNC_ERR_INVALID_ARGUMENT;
    c->model.p = *m;
    return KNC_OK;
}

int oracle_init_from_model(oracle_ctx* c, double time) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    if (c->mesh.p.reference_radius > c->mesh.outer_excision_surface(time)) return KNC_ERR_CONFIG;
    c->blocks.clear();
    std::vector<int32_t> idx;
    for (int32_t i = 0;; ++i) {                     // Mesh::grid_blocks, mesh.rs:384-397
        if (c->mesh.subgrid_extent(i).r0 >= c->mesh.outer_excision_surface(time)) break;
        idx.push_back(i);
        if (i > 1000000) return KNC_ERR_CONFIG;
    }
    std::vector<const Geometry*> gs;
    for (int32_t i : idx) { gs.push_back(&geometry_of(c, i)); c->blocks[i]; }
    parallel_for(c->threads, (int64_t)idx.size(), [&](int64_t k) {
        c->blocks.at(idx[k]) = block_from_model(c, idx[k], *gs[k], time, true);
    });
    c->time = time;
    c->iteration.n = 0;
    c->iteration.d = 1;
    return KNC_OK;
}

int oracle_add_block(oracle_ctx* c, int32_t index, const double* cons, const double* scalar) {
    if (!c || !cons || !scalar) return KNC_ERR_INVALID_ARGUMENT;
    const auto sh = shape_of(c, index);
    const int64_t n = sh.first * sh.second;
    Block B;
    B.U.assign(cons, cons + n * 4);
    B.S.assign(scalar, scalar + n);
    geometry_of(c, index);
    c->blocks[index] = std::move(B);
    return KNC_OK;
}

int oracle_set_block_shapes(oracle_ctx* c, int32_t first, int32_t count, const int32_t* nr, const int32_t* nq) {
    if (!c || count < 0 || (count && (!nr || !nq))) return KNC_ERR_INVALID_ARGUMENT;
    const int64_t nq0 = c->mesh.p.num_polar_zones;
    for (int32_t k = 0; k < count; ++k) {
        // nq = nq0 * 2^m, so the polar grids of any two blocks nest
        int64_t a = nq0, b = nq[k];
        while (a > 0 && b > 0 && a != b && ((a < b && b % 2 == 0) || (a > b && a % 2 == 0))) {
            if (a < b) b /= 2;
            else a /= 2;
        }
        if (nr[k] < 2 || a != b || (nq0 != 1 && nq[k] < 16) || (nq0 == 1 && nq[k] != 1)) return KNC_ERR_CONFIG;
    }
    for (int32_t k = 0; k < count; ++k) c->shapes[first + k] = {nr[k], nq[k]};
    return KNC_OK;
}

int oracle_block_shape_of(const oracle_ctx* c, int32_t index, int64_t* nr, int64_t* nq) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    const auto sh = shape_of(c, index);
    if (nr) *nr = sh.first;
    if (nq) *nq = sh.second;
    return KNC_OK;
}

int oracle_remove_block(oracle_ctx* c, int32_t index) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    return c->blocks.erase(index) ? KNC_OK : KNC_ERR_NO_BLOCK;
}

int oracle_get_block(oracle_ctx* c, int32_t index, double* cons, double* scalar) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    auto it = c->blocks.find(index);
    if (it == c->blocks.end()) return KNC_ERR_NO_BLOCK;
    if (cons) std::memcpy(cons, it->second.U.data(), it->second.U.size() * sizeof(double));
    if (scalar) std::memcpy(scalar, it->second.S.data(), it->second.S.size() * sizeof(double));
    return KNC_OK;
}

// The primitive export of one block (Products::try_from_state,
// src/products.rs:43-66, via BlockState::try_to_primitive, state.rs:76-94):
// [nr][nq][5] = (rho, u_r, u_theta, p, scalar concentration s / rho).
int oracle_get_primitives(oracle_ctx* c, int32_t index, double* prim) {
    if (!c || !prim) return KNC_ERR_INVALID_ARGUMENT;
    auto it = c->blocks.find(index);
    if (it == c->blocks.end()) return KNC_ERR_NO_BLOCK;
    const Geometry& G = geometry_of(c, index);
    PrimBlock pb;
    ErrorRec e;
    if (!block_to_primitive(c, index, it->second, G, pb, e)) {
        c->err = e;
        return KNC_ERR_HYDRO;
    }
    const int64_t n = G.nr * G.nq;
    for (int64_t z = 0; z < n; ++z) {
        for (int q = 0; q < 4; ++q) prim[z * 5 + q] = pb.P[z].v[q];
        prim[z * 5 + 4] = pb.s[z] / pb.P[z].v[0];
    }
    return KNC_OK;
}

// BlockProducts::try_from_block_state (src/products.rs:43-66) of one block:
// the block's vertices, its primitives in AnyPrimitive order (velocity_r,
// velocity_q, mass_density, gas_pressure) and scalar_mass / lab_frame_mass of
// the volume-integrated state.
int oracle_get_products(oracle_ctx* c, int32_t index, double* rv, double* qv, double* prim, double* scalar) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    auto it = c->blocks.find(index);
    if (it == c->blocks.end()) return KNC_ERR_NO_BLOCK;
    const Geometry& G = geometry_of(c, index);
    if (rv) std::memcpy(rv, G.rv.data(), G.rv.size() * sizeof(double));
    if (qv) std::memcpy(qv, G.qv.data(), G.qv.size() * sizeof(double));
    if (!prim && !scalar) return KNC_OK;
    PrimBlock pb;
    ErrorRec e;
    if (!block_to_primitive(c, index, it->second, G, pb, e)) {
        c->err = e;
        return KNC_ERR_HYDRO;
    }
    const Block& B = it->second;
    const int64_t n = G.nr * G.nq;
    for (int64_t z = 0; z < n; ++z) {
        if (prim) {
            prim[z * 4 + 0] = pb.P[z].v[1];
            prim[z * 4 + 1] = pb.P[z].v[2];
            prim[z * 4 + 2] = pb.P[z].v[0];
            prim[z * 4 + 3] = pb.P[z].v[3];
        }
        if (scalar) scalar[z] = B.S[z] / B.U[z * 4 + 0];
    }
    return KNC_OK;
}

int oracle_num_blocks(const oracle_ctx* c, int32_t* n) {
    if (!c || !n) return KNC_ERR_INVALID_ARGUMENT;
    *n = (int32_t)c->blocks.size();
    return KNC_OK;
}

int oracle_block_indexes(const oracle_ctx* c, int32_t* out, int32_t capacity) {
    if (!c || !out) return KNC_ERR_INVALID_ARGUMENT;
    int32_t k = 0;
    for (auto& kv : c->blocks) {
        if (k >= capacity) return KNC_ERR_INVALID_ARGUMENT;
        out[k++] = kv.first;
    }
    return KNC_OK;
}

int oracle_set_time(oracle_ctx* c, double time, int64_t num, int64_t den) {
    if (!c || den == 0) return KNC_ERR_INVALID_ARGUMENT;
    c->time = time;
    c->iteration.n = num;
    c->iteration.d = den;
    c->iteration.norm();
    return KNC_OK;
}

int oracle_get_time(const oracle_ctx* c, double* time, int64_t* num, int64_t* den) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    if (time) *time = c->time;
    if (num) *num = c->iteration.n;
    if (den) *den = c->iteration.d;
    return KNC_OK;
}

// State::time_step, state.rs:143-162
int oracle_time_step(oracle_ctx* c, double* dt) {
    if (!c || !dt || c->blocks.empty()) return KNC_ERR_INVALID_ARGUMENT;
    const bool global = c->ph.system == KNC_SYSTEM_RELATIVISTIC && !c->hp.adaptive_time_step;
    if (global) {
        // smallest_spacing of the innermost block (mesh.rs:304-307); with
        // uneven blocks the minimum over all blocks, which for equal shapes is
        // always the innermost block's
        double spacing = std::numeric_limits<double>::max();
        for (auto& kv : c->blocks) {
            const Extent e = c->mesh.subgrid_extent(kv.first);
            const int64_t nr = shape_of(c, kv.first).first;
            spacing = std::min(spacing, vertex_r(e, nr, 1) - vertex_r(e, nr, 0));
        }
        *dt = c->hp.cfl_number * spacing / LIGHT_SPEED;
        return KNC_OK;
    }
    double dtmin = std::numeric_limits<double>::max();
    for (auto& kv : c->blocks) {
        const Geometry& G = geometry_of(c, kv.first);
        PrimBlock pb;
        ErrorRec e;
        if (!block_to_primitive(c, kv.first, kv.second, G, pb, e)) { c->err = e; return KNC_ERR_HYDRO; }
        const double cmax = c->ph.system == KNC_SYSTEM_RELATIVISTIC ? LIGHT_SPEED : 1.0;
        for (int64_t i = 0; i < G.nr; ++i)
            for (int64_t j = 0; j < G.nq; ++j) {
                const double dr = G.rv[i + 1] - G.rv[i];
                const double dq = G.qv[j + 1] - G.qv[j];
                const double dl = std::min(dr, dq * G.rv[i]);                  // mesh.rs:40-46
                const double a = max_signal_speed(c->ph, pb.P[i * G.nq + j]) * cmax;
                dtmin = std::min(dtmin, dl / a);
            }
    }
    *dt = dtmin * c->hp.cfl_number;
    return KNC_OK;
}

// scheme::advance, scheme.rs:212-240
int oracle_advance(oracle_ctx* c, int32_t fold) {
    if (!c || fold < 0 || c->blocks.empty()) return KNC_ERR_INVALID_ARGUMENT;
    double dt;
    const int r = oracle_time_step(c, &dt);
    if (r != KNC_OK) return r;
    return oracle_advance_dt(c, fold, dt);
}

// scheme::advance with the time step given by the caller (a multi-domain
// driver passes the minimum of every domain's time_step).
int oracle_advance_dt(oracle_ctx* c, int32_t fold, double dt) {
    if (!c || fold < 0 || c->blocks.empty() || !(dt > 0.0)) return KNC_ERR_INVALID_ARGUMENT;
    for (int32_t k = 0; k < fold; ++k) {
        if (c->mesh.moving()) add_remove_blocks(c);
        if (!rk_step(c, dt)) return KNC_ERR_HYDRO;
    }
    return KNC_OK;
}

int oracle_last_error(const oracle_ctx* c, knc_error* out) {
    if (!c || !out) return KNC_ERR_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->kind = c->err.kind;
    out->block = c->err.block;
    out->i = (int32_t)c->err.i;
    out->j = (int32_t)c->err.j;
    out->r = c->err.r;
    out->theta = c->err.q;
    out->value = c->err.value;
    std::snprintf(out->message, sizeof(out->message), "hydro error %d at position (r, theta) = (%.4e, %.4f)",
                  c->err.kind, c->err.r, c->err.q);
    return KNC_OK;
}

int oracle_c2p_stats(const oracle_ctx* c, int64_t* zones, int64_t* iters) {
    if (!c) return KNC_ERR_INVALID_ARGUMENT;
    if (zones) *zones = c->c2p_zones.load();
    if (iters) *iters = c->c2p_iters.load();
    return KNC_OK;
}

void oracle_prim_to_cons(const knc_hydro_params* h, const double p[4], double u[4]) {
    const Phys ph = make_phys(h);
    Prim P;
    for (int q = 0; q < 4; ++q) P.v[q] = p[q];
    const Cons U = p2c(ph, P);
    for (int q = 0; q < 4; ++q) u[q] = U.v[q];
}

int oracle_cons_to_prim(const knc_hydro_params* h, const double u[4], double guess, double p[4],
                        int32_t* iterations) {
    const Phys ph = make_phys(h);
    Cons U;
    for (int q = 0; q < 4; ++q) U.v[q] = u[q];
    Prim P{};
    double bad = 0.0;
    int it = 0, kind;
    if (ph.system == KNC_SYSTEM_RELATIVISTIC) kind = srhd_c2p(ph, U, guess < 0.0 ? 0.0 : guess, P, it, bad);
    else kind = newt_c2p(ph, U, P, bad);
    for (int q = 0; q < 4; ++q) p[q] = P.v[q];
    if (iterations) *iterations = it;
    return kind;
}

void oracle_flux(const knc_hydro_params* h, const double p[4], int32_t axis, double f[4],
                 double* lm, double* lp) {
    const Phys ph = make_phys(h);
    Prim P;
    for (int q = 0; q < 4; ++q) P.v[q] = p[q];
    const Side S = make_side(ph, P, 0.0, axis);
    for (int q = 0; q < 4; ++q) f[q] = S.F[q];
    if (lm) *lm = S.lm;
    if (lp) *lp = S.lp;
}

void oracle_riemann(const knc_hydro_params* h, const double pl[4], const double pr[4], double sl,
                    double sr, int32_t axis, double out[5]) {
    const Phys ph = make_phys(h);
    Prim L, R;
    for (int q = 0; q < 4; ++q) { L.v[q] = pl[q]; R.v[q] = pr[q]; }
    riemann(ph, L, R, sl, sr, axis, out);
}

double oracle_plm_gradient(double theta, double a, double b, double c) {
    return plm_gradient(theta, a, b, c);
}

void oracle_sources(const knc_hydro_params* h, const double p[4], double r, double theta, double s[4]) {
    const Phys ph = make_phys(h);
    Prim P;
    for (int q = 0; q < 4; ++q) P.v[q] = p[q];
    const Cons S = sources(ph, P, r, std::cos(theta) / std::sin(theta));
    for (int q = 0; q < 4; ++q) s[q] = S.v[q];
}

double oracle_max_signal_speed(const knc_hydro_params* h, const double p[4]) {
    const Phys ph = make_phys(h);
    Prim P;
    for (int q = 0; q < 4; ++q) P.v[q] = p[q];
    return max_signal_speed(ph, P);
}

int oracle_block_geometry(const knc_mesh_params* m, int32_t index, double* rv, double* qv, double* ar,
                          double* aq, double* dv, double* rc, double* qc) {
    if (!m) return KNC_ERR_INVALID_ARGUMENT;
    MeshDef M;
    M.p = *m;
    const Geometry G = make_geometry(M, index, m->block_size, m->num_polar_zones);
    if (rv) std::memcpy(rv, G.rv.data(), G.rv.size() * sizeof(double));
    if (qv) std::memcpy(qv, G.qv.data(), G.qv.size() * sizeof(double));
    if (ar) std::memcpy(ar, G.ar.data(), G.ar.size() * sizeof(double));
    if (aq) std::memcpy(aq, G.aq.data(), G.aq.size() * sizeof(double));
    if (dv) std::memcpy(dv, G.dv.data(), G.dv.size() * sizeof(double));
    if (rc) std::memcpy(rc, G.rc.data(), G.rc.size() * sizeof(double));
    if (qc) std::memcpy(qc, G.qc.data(), G.qc.size() * sizeof(double));
    return KNC_OK;
}

}  // extern "C"

// ------------------------------------------------------------ MLP (CPU) ---
namespace {
inline float bf16_round(float x) {                 // round to nearest even
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) return x;  // inf / nan unchanged
    const uint32_t lsb = (u >> 16) & 1u;
    u = (u + 0x7fffu + lsb) & 0xffff0000u;
    float y;
    std::memcpy(&y, &u, 4);
    return y;
}
inline double sigmoid(double z) { return 1.0 / (1.0 + std::exp(-z)); }
}  // namespace

extern "C" void oracle_mlp_forward_backward(const float* w, const float* x, const float* y, int32_t n,
                                            int32_t round_bf16, double* pred, double* loss, double* grad) {
    auto rnd = [round_bf16](float v) { return round_bf16 ? bf16_round(v) : v; };
    constexpr int H = KNC_MLP_HIDDEN;
    std::vector<double> g(KNC_MLP_NUM_PARAMS, 0.0);
    double W1[H][3], W2[H][H], W3[H];
    for (int u = 0; u < H; ++u) {
        for (int k = 0; k < 3; ++k) W1[u][k] = rnd(w[KNC_MLP_OFF_W1 + u * 3 + k]);
        for (int v = 0; v < H; ++v) W2[u][v] = rnd(w[KNC_MLP_OFF_W2 + u * H + v]);
        W3[u] = rnd(w[KNC_MLP_OFF_W3 + u]);
    }
    double L = 0.0;
    for (int32_t r = 0; r < n; ++r) {
        double xn[3], z1[H], s1[H], a1[H], z2[H], s2[H], h2[H];
        for (int k = 0; k < 3; ++k)
            xn[k] = ((double)x[r * 3 + k] - w[KNC_MLP_OFF_XMEAN + k]) * w[KNC_MLP_OFF_XSCALE + k];
        for (int u = 0; u < H; ++u) {
            double z = w[KNC_MLP_OFF_B1 + u];
            for (int k = 0; k < 3; ++k) z += W1[u][k] * xn[k];
            z1[u] = z;
            s1[u] = sigmoid(z);
            a1[u] = round_bf16 ? (double)bf16_round((float)(z * s1[u])) : z * s1[u];
        }
        double out = w[KNC_MLP_OFF_B3];
        for (int u = 0; u < H; ++u) {
            double z = w[KNC_MLP_OFF_B2 + u];
            for (int v = 0; v < H; ++v) z += W2[u][v] * a1[v];
            z2[u] = z;
            s2[u] = sigmoid(z);
            h2[u] = z * s2[u];
            out += W3[u] * h2[u];
        }
        if (pred) pred[r] = out;
        const double e = out - (double)y[r];
        L += e * e;
        const double dout = 2.0 * e / (double)n;
        g[KNC_MLP_OFF_B3] += dout;
        double dz2[H];
        for (int u = 0; u < H; ++u) {
            g[KNC_MLP_OFF_W3 + u] += dout * h2[u];
            const double dh2 = dout * W3[u];
            dz2[u] = dh2 * s2[u] * (1.0 + z2[u] * (1.0 - s2[u]));
            g[KNC_MLP_OFF_B2 + u] += dz2[u];
            for (int v = 0; v < H; ++v) g[KNC_MLP_OFF_W2 + u * H + v] += dz2[u] * a1[v];
        }
        for (int v = 0; v < H; ++v) {
            double da = 0.0;
            for (int u = 0; u < H; ++u) da += dz2[u] * W2[u][v];
            const double dz1 = da * s1[v] * (1.0 + z1[v] * (1.0 - s1[v]));
            g[KNC_MLP_OFF_B1 + v] += dz1;
            for (int k = 0; k < 3; ++k) g[KNC_MLP_OFF_W1 + v * 3 + k] += dz1 * xn[k];
        }
    }
    if (loss) *loss = L / (double)n;
    if (grad) for (int k = 0; k < KNC_MLP_NUM_PARAMS; ++k) grad[k] = g[k];
}
