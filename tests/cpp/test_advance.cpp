// Tests of the C++ host surface (include/knc.hpp) against the CPU oracle,
// written as a host program of the library would be: knc::advance moves a
// knc::State through the GPU, and the oracle advances the same State.
//
//   advance_matches_oracle        the 4 x 64 x 128 relativistic wind (gamma 4/3,
//                                 PLM 1.5, HLLE, RK2, CFL 0.4) from its model,
//                                 100 steps through knc::advance in folds of
//                                 25: every block, the time and the iteration
//                                 bit for bit equal to the oracle's
//   hydro_error_at_position       a negative density in one zone: advance
//                                 throws knc::HydroError with the oracle's
//                                 kind, block, zone, centroid and value
//   mixed_precision_within_gate   the mixed-precision stage, 100 steps: lab-frame
//                                 density L1 against the oracle at most 1e-6
//   newtonian_sphere_matches_oracle  NewtonianHydro, HLLC, adaptive time step,
//                                 the over-dense sphere: 40 steps bit for bit
//   state_round_trip              load then state() returns the same blocks
//
// Exit status 0 when every test passes; one line per test on stdout.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/knc.hpp"
#include "../../oracle/knc_oracle.h"

namespace {

knc::RelativisticHydro wind_hydro() {
    knc::RelativisticHydro h;
    h.gamma_law_index = 4.0 / 3.0;
    h.plm_theta = 1.5;
    h.cfl_number = 0.4;
    h.runge_kutta_order = knc::RungeKuttaOrder::RK2;
    h.riemann_solver = knc::RiemannSolver::HLLE;
    return h;
}

knc::Mesh wind_mesh() {
    knc::Mesh m;
    m.reference_radius = 1.0;
    m.inner_radius = 1.0;
    m.outer_radius = 10.0;
    m.num_polar_zones = 128;
    m.block_size = 64;
    m.num_radial_zones = {true, 82};
    return m;
}

knc_model_params wind_model() {
    knc_model_params p{};
    p.kind = KNC_MODEL_WIND;
    p.seed = 1;
    p.p[0] = 1.0;    // rho at r = 1
    p.p[1] = 1.0;    // u^r
    p.p[2] = 1e-4;   // p / rho
    p.p[3] = 0.01;   // noise amplitude
    return p;
}

// The oracle behind the same surface: a State in, a State out.
struct Oracle {
    oracle_ctx* ctx = nullptr;
    template <class Hydro>
    Oracle(const Hydro& h, const knc::Mesh& m) {
        const knc_hydro_params hp = h.to_c();
        const knc_mesh_params mp = m.to_c();
        if (oracle_create(&hp, &mp, 8, &ctx) != KNC_OK) throw std::runtime_error("oracle_create");
    }
    ~Oracle() { oracle_destroy(ctx); }
    void load(const knc::State& s) {
        for (const auto& kv : s.solution)
            if (oracle_add_block(ctx, kv.first, kv.second.conserved.data(), kv.second.scalar_mass.data()) != KNC_OK)
                throw std::runtime_error("oracle_add_block");
        oracle_set_time(ctx, s.time, s.iteration.num, s.iteration.den);
    }
    knc::State state() const {
        knc::State s;
        oracle_get_time(ctx, &s.time, &s.iteration.num, &s.iteration.den);
        int32_t n = 0;
        oracle_num_blocks(ctx, &n);
        std::vector<int32_t> idx(n);
        oracle_block_indexes(ctx, idx.data(), n);
        for (int32_t i : idx) {
            knc::BlockState b;
            oracle_block_shape_of(ctx, i, &b.nr, &b.nq);
            b.conserved.resize((size_t)(b.nr * b.nq * 4));
            b.scalar_mass.resize((size_t)(b.nr * b.nq));
            oracle_get_block(ctx, i, b.conserved.data(), b.scalar_mass.data());
            s.solution.emplace(i, std::move(b));
        }
        return s;
    }
};

bool same_state(const knc::State& a, const knc::State& b, std::string& why) {
    if (a.time != b.time) return why = "time differs", false;
    if (a.iteration.num != b.iteration.num || a.iteration.den != b.iteration.den) return why = "iteration differs", false;
    if (a.solution.size() != b.solution.size()) return why = "block sets differ", false;
    for (const auto& kv : a.solution) {
        auto it = b.solution.find(kv.first);
        if (it == b.solution.end()) return why = "block " + std::to_string(kv.first) + " missing", false;
        const knc::BlockState& x = kv.second;
        const knc::BlockState& y = it->second;
        if (x.conserved.size() != y.conserved.size() ||
            std::memcmp(x.conserved.data(), y.conserved.data(), x.conserved.size() * sizeof(double)) != 0)
            return why = "conserved state of block " + std::to_string(kv.first) + " differs", false;
        if (std::memcmp(x.scalar_mass.data(), y.scalar_mass.data(), x.scalar_mass.size() * sizeof(double)) != 0)
            return why = "scalar mass of block " + std::to_string(kv.first) + " differs", false;
    }
    return true;
}

bool advance_matches_oracle(std::string& why) {
    const auto hydro = wind_hydro();
    const auto mesh = wind_mesh();
    knc::Engine engine(hydro, mesh);
    engine.set_model(wind_model());
    knc::State state = engine.from_model(0.0);
    Oracle oracle(hydro, mesh);
    const knc_model_params model = wind_model();
    oracle_set_model(oracle.ctx, &model);
    oracle.load(state);
    for (int k = 0; k < 4; ++k) {
        state = knc::advance(std::move(state), engine, 25);
        oracle_advance(oracle.ctx, 25);
    }
    return same_state(state, oracle.state(), why);
}

bool hydro_error_at_position(std::string& why) {
    const auto hydro = wind_hydro();
    const auto mesh = wind_mesh();
    knc::Engine engine(hydro, mesh);
    engine.set_model(wind_model());
    knc::State state = engine.from_model(0.0);
    // a negative lab-frame density in zone (10, 37) of block 2
    knc::BlockState& b = state.solution.at(2);
    b.conserved[(size_t)((10 * b.nq + 37) * 4)] *= -1.0;
    Oracle oracle(hydro, mesh);
    const knc_model_params model = wind_model();
    oracle_set_model(oracle.ctx, &model);
    oracle.load(state);
    knc_error ref{};
    if (oracle_advance(oracle.ctx, 1) != KNC_ERR_HYDRO) return why = "the oracle did not fail", false;
    oracle_last_error(oracle.ctx, &ref);
    try {
        knc::advance(state, engine, 1);
    } catch (const knc::HydroError& e) {
        if (e.kind != ref.kind || e.block != ref.block || e.i != ref.i || e.j != ref.j)
            return why = "failing zone differs: " + std::to_string(e.block) + " (" + std::to_string(e.i) + ", " +
                         std::to_string(e.j) + ")", false;
        if (e.r != ref.r || e.theta != ref.theta || e.value != ref.value)
            return why = "position or value differs", false;
        if (e.kind != KNC_HYDRO_NEGATIVE_DENSITY) return why = "not a negative density", false;
        return true;
    }
    return why = "no HydroError thrown", false;
}

bool mixed_precision_within_gate(std::string& why) {
    // the mixed-precision stage (FP32 fluxes, FP64 state and recovery above
    // the Lorentz-factor split) through the same surface: lab-frame density L1
    // against the FP64 oracle at most 1e-6 after 100 steps
    const auto hydro = wind_hydro();
    const auto mesh = wind_mesh();
    knc::Engine engine(hydro, mesh);
    engine.set_model(wind_model());
    engine.set_precision(KNC_PRECISION_MIXED);
    knc::State state = engine.from_model(0.0);
    Oracle oracle(hydro, mesh);
    const knc_model_params model = wind_model();
    oracle_set_model(oracle.ctx, &model);
    oracle.load(state);
    state = knc::advance(std::move(state), engine, 100);
    oracle_advance(oracle.ctx, 100);
    const knc::State ref = oracle.state();
    if (state.time != ref.time) return why = "time differs", false;
    double num = 0.0, den = 0.0;
    for (const auto& kv : ref.solution) {
        const knc::BlockState& b = kv.second;
        const knc::BlockState& g = state.solution.at(kv.first);
        for (size_t z = 0; z < b.conserved.size(); z += 4) {
            num += std::fabs(g.conserved[z] - b.conserved[z]);
            den += std::fabs(b.conserved[z]);
        }
    }
    const double l1 = num / den;
    if (!(l1 <= 1e-6)) return why = "density L1 " + std::to_string(l1), false;
    return true;
}

bool newtonian_sphere_matches_oracle(std::string& why) {
    // NewtonianHydro (gamma 5/3, HLLC, RK2, always an adaptive time step) on
    // the seeded over-dense sphere at rest: 40 steps in folds of 10, bit for bit
    knc::NewtonianHydro hydro;
    hydro.gamma_law_index = 5.0 / 3.0;
    hydro.riemann_solver = knc::RiemannSolver::HLLC;
    const auto mesh = wind_mesh();
    knc_model_params sphere{};
    sphere.kind = KNC_MODEL_SPHERE;
    sphere.seed = 1;
    sphere.p[0] = 10.0;   // rho inside
    sphere.p[1] = 1.0;    // rho outside
    sphere.p[2] = 2.0;    // sphere radius
    sphere.p[3] = 1e-2;   // pressure
    sphere.p[4] = 0.01;   // noise amplitude
    knc::Engine engine(hydro, mesh);
    engine.set_model(sphere);
    knc::State state = engine.from_model(0.0);
    Oracle oracle(hydro, mesh);
    oracle_set_model(oracle.ctx, &sphere);
    oracle.load(state);
    for (int k = 0; k < 4; ++k) {
        state = knc::advance(std::move(state), engine, 10);
        oracle_advance(oracle.ctx, 10);
    }
    return same_state(state, oracle.state(), why);
}

bool state_round_trip(std::string& why) {
    const auto hydro = wind_hydro();
    const auto mesh = wind_mesh();
    knc::Engine engine(hydro, mesh);
    engine.set_model(wind_model());
    const knc::State a = engine.from_model(0.0);
    knc::Engine other(hydro, mesh);
    other.set_model(wind_model());
    other.load(a);
    return same_state(a, other.state(), why);
}

}  // namespace

int main() {
    struct Case {
        const char* name;
        bool (*run)(std::string&);
    };
    const Case cases[] = {{"advance_matches_oracle", advance_matches_oracle},
                          {"hydro_error_at_position", hydro_error_at_position},
                          {"mixed_precision_within_gate", mixed_precision_within_gate},
                          {"newtonian_sphere_matches_oracle", newtonian_sphere_matches_oracle},
                          {"state_round_trip", state_round_trip}};
    int failed = 0;
    for (const Case& c : cases) {
        std::string why;
        bool ok = false;
        try {
            ok = c.run(why);
        } catch (const std::exception& e) {
            why = std::string("exception: ") + e.what();
        }
        std::printf("%s %s%s%s\n", ok ? "ok  " : "FAIL", c.name, ok ? "" : ": ", ok ? "" : why.c_str());
        failed += ok ? 0 : 1;
    }
    return failed ? 1 : 0;
}
