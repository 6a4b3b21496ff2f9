// knc_models.cuh — device-side initial / boundary models.
//
// The reference evaluates `InitialModel::primitive_at` and `scalar_at`
// (src/traits.rs:145-164) on the host for the initial data and, at every RK
// stage, for the two ghost blocks (src/scheme.rs:45-52). Keeping these
// functors on the device lets a whole stage run without host work, so a fold
// of steps can be captured in a CUDA graph. Geometry follows the nozzle
// convention of src/models/jet_in_cloud.rs:172-174 (both poles).
#pragma once

#include "knc_physics.cuh"
#include "../../include/knc.h"

namespace knc {

// ---- the reference's setups (cgs units, LIGHT_SPEED = 3e10) -----------------
// Each writes the primitive in this library's order (rho, u_r, u_theta, p),
// i.e. `Hydrodynamics::interpret` of the model's AnyPrimitive.

// JetInCloud, src/models/jet_in_cloud.rs:74-257. a = (cloud_mass, engine_delay,
// engine_duration, engine_strength, engine_theta, engine_u, envelop_m1,
// envelop_slowest_beta, envelop_fastest_beta, envelop_psi).
__device__ __forceinline__ void jet_in_cloud(const double* a, double r, double q, double t, double P[4],
                                             double& scalar) {
    const double cloud_mass = a[0], delay = a[1], duration = a[2], strength = a[3], theta_j = a[4];
    const double engine_u = a[5], m1 = a[6], slowest = a[7], fastest = a[8], psi = a[9];
    const double engine_beta = engine_u / sqrt(1.0 + engine_u * engine_u);
    const double v_min = slowest * LIGHT_SPEED;
    const double v_jet = engine_beta * LIGHT_SPEED;
    const double r_interface = v_min * t;
    const double r_head = v_jet * (t - delay);
    const double r_tail = v_jet * (t - delay - duration);
    const bool nozzle = q < theta_j || q > PI - theta_j;
    int zone;   // 0 cloud, 1 envelope, 2 jet
    if (nozzle && r < r_head && r > r_tail) zone = 2;
    else if (r > r_interface) zone = 1;
    else zone = 0;
    double u, f;
    if (zone == 0) {
        u = slowest / sqrt(1.0 - slowest * slowest);
        f = cloud_mass / (4.0 * PI * delay);
        scalar = 1.0;
    } else if (zone == 1) {
        const double b = fmin(r / t / LIGHT_SPEED, fastest);
        u = b / sqrt(1.0 - b * b);
        const double ff = pow(b, -1.0 / psi) * pow(1.0 - b * b, 0.5 / psi - 1.0);
        f = m1 / (4.0 * PI * psi * t) * ff;
        scalar = 1e-2;
    } else {
        u = engine_u;
        const double engine_gamma = sqrt(1.0 + engine_u * engine_u);
        const double e = strength * cloud_mass;
        const double l = e / (4.0 * PI * duration);
        f = l / engine_gamma;
        scalar = 1e2;
    }
    const double d = f / (r * r * u) / LIGHT_SPEED;
    P[0] = d;
    P[1] = u;
    P[2] = 0.0;
    P[3] = d * 1e-3;
}

// KineticBomb, src/models/kinetic_bomb.rs:78-114. a = (external_medium_density,
// launch_radius, shell_thickness, kinetic_energy, shell_mass).
__device__ __forceinline__ void kinetic_bomb(const double* a, double r, double t, double P[4], double& scalar) {
    const double rho_ext = a[0], launch = a[1], thickness = a[2], energy = a[3], mass = a[4];
    const double v = sqrt(2.0 * energy / mass);
    const double shell_duration = thickness / v;
    const double r_outer = launch + v * t;
    const double r_inner = launch + v * (t - shell_duration);
    if (r_inner <= r && r < r_outer) {
        const double mdot = mass / shell_duration;
        const double d = mdot / (4.0 * PI * r * r * v);
        P[0] = d;
        P[1] = v / LIGHT_SPEED;
        P[2] = 0.0;
        P[3] = d * 1e-3;
        scalar = 1.0;
    } else {
        const double x = r / launch;
        const double d = rho_ext * (x * x);
        P[0] = d;
        P[1] = 0.0;
        P[2] = 0.0;
        P[3] = d * 1e-3;
        scalar = 0.0;
    }
}

// JetInStar, src/models/jet_in_star.rs:87-236, with the progenitor constants of
// Duffell & MacFadyen (2015) as that file states them. a = (star_mass,
// engine_duration, engine_energy, engine_theta, engine_u, envelope_radius,
// envelope_mass, volume_factor).
__device__ __forceinline__ void jet_in_star(const double* a, double r, double q, double t, double P[4],
                                            double& scalar) {
    const double R0 = 7e10, M0 = 2e33;
    const double RHO_C = 3e7 * M0 / (1.33 * PI * R0 * R0 * R0);
    const double R1 = 0.0017 * R0, R2 = 0.0125 * R0, R3 = 0.65 * R0;
    const double K1 = 3.24, K2 = 2.57, NN = 16.7, ALPHA = 2.5;
    const double RHO_WIND = 1e-9 * M0 / (1.33 * PI * R0 * R0 * R0);
    const double R_NOZZ = 0.01 * R0, R_ENV = 1.2 * R0;
    const double duration = a[1], energy = a[2], theta_j = a[3], engine_u = a[4];
    const double env_radius = a[5], env_mass = a[6], fill = a[7];
    const double engine_beta = engine_u / sqrt(1.0 + engine_u * engine_u);
    const double r_head = engine_beta * LIGHT_SPEED * t;
    const bool nozzle = q < theta_j || q > PI - theta_j;
    int zone;   // 0 core, 1 envelope, 2 wind, 3 jet
    if (nozzle && r < r_head) zone = 3;
    else if (r < R3) zone = 0;
    else if (R3 < r && r < env_radius) zone = 1;
    else zone = 2;
    double d, u = 0.0;
    const double rho_env = env_mass / (4.0 * PI * (env_radius * env_radius) * (env_radius - R3) * fill);
    if (zone == 0) {
        const double num = RHO_C * pow(1.0 - r / R3, NN);
        const double den = 1.0 + pow(r / R1, K1) / (1.0 + pow(r / R2, K2));
        d = num / den + rho_env * pow(r / R3, -2.0);
        scalar = 1.0;
    } else if (zone == 1) {
        d = rho_env * pow(r / R3, -ALPHA);
        scalar = 1e-2 * pow(r / R3, -2.0);
    } else if (zone == 3) {
        const double r0 = R_NOZZ / R0;
        const double q2 = theta_j * theta_j;
        const double n0 = 4.0 * PI * r0 * r0 * r0 * (1.0 - exp(-2.0 / q2)) * q2;
        const double cq = cos(q);
        const double g = (r / R_NOZZ) * exp(-pow(r / R_NOZZ, 2.0) / 2.0) * exp((pow(cq, 2.0) - 1.0) / q2);
        const double nozzle_fn = g / n0;
        const double engine_gamma = sqrt(1.0 + engine_u * engine_u);
        const double l = nozzle_fn * energy / (4.0 * PI * duration);
        const double rate = l / (engine_gamma * LIGHT_SPEED * LIGHT_SPEED);
        d = rate / (r * r * engine_u * LIGHT_SPEED);
        u = engine_u;
        scalar = 1e2;
    } else {
        d = RHO_WIND * pow(r / R_ENV, -2.0);
        scalar = 1e-5 * pow(r / R_ENV, -2.0);
    }
    P[0] = d;
    P[1] = u;
    P[2] = 0.0;
    P[3] = d * 1e-10;
}

// Primitive (rho, u_r, u_theta, p) and scalar concentration of model M at the
// centroid (r, q) and time t. `noise` multiplies the density of initial data
// by (1 + amp U[0,1)) keyed on (seed, block, i, j); ghost blocks never see it.
__device__ __forceinline__ void model_eval(const knc_model_params& M, double r, double q, double t,
                                           bool noise, int32_t block, int64_t i, int64_t j, double P[4],
                                           double& scalar) {
    const double* a = M.p;
    scalar = 0.0;
    const double inv_r2 = 1.0 / (r * r);
    switch (M.kind) {
    case KNC_MODEL_WIND: {
        double rho = a[0] * inv_r2;
        const double amp = a[3];
        if (noise && amp != 0.0) rho = rho * (1.0 + amp * uniform01(M.seed, block, i, j));
        P[0] = rho;
        P[1] = a[1];
        P[2] = 0.0;
        P[3] = a[2] * rho;
        break;
    }
    case KNC_MODEL_JET: {
        double rho = a[0] * inv_r2;
        const double amp = a[2];
        if (noise && amp != 0.0) rho = rho * (1.0 + amp * uniform01(M.seed, block, i, j));
        P[0] = rho;
        P[1] = 0.0;
        P[2] = 0.0;
        P[3] = a[1] * rho;
        const bool nozzle = (q < a[3] || q > PI - a[3]) && r < a[6];
        if (nozzle) {
            const double rj = a[0] * inv_r2 * a[5];
            P[0] = rj;
            P[1] = sqrt(a[4] * a[4] - 1.0);
            P[3] = a[1] * rj;
            scalar = 1.0;
        }
        break;
    }
    case KNC_MODEL_SPHERE: {
        double rho = r < a[2] ? a[0] : a[1];
        const double amp = a[4];
        if (noise && amp != 0.0) rho = rho * (1.0 + amp * uniform01(M.seed, block, i, j));
        P[0] = rho;
        P[1] = 0.0;
        P[2] = 0.0;
        P[3] = a[3];
        scalar = r < a[2] ? 1.0 : 0.0;
        break;
    }
    case KNC_MODEL_JET_IN_CLOUD:
        jet_in_cloud(a, r, q, t, P, scalar);
        break;
    case KNC_MODEL_KINETIC_BOMB:
        kinetic_bomb(a, r, t, P, scalar);
        break;
    case KNC_MODEL_JET_IN_STAR:
        jet_in_star(a, r, q, t, P, scalar);
        break;
    default:
        P[0] = 1.0;
        P[1] = 0.0;
        P[2] = 0.0;
        P[3] = 1.0;
    }
}

}  // namespace knc
