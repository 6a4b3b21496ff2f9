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
    default:
        P[0] = 1.0;
        P[1] = 0.0;
        P[2] = 0.0;
        P[3] = 1.0;
    }
    (void)t;
}

}  // namespace knc
