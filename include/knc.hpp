/*
 * knc.hpp — the C++ host surface over the C ABI of knc.h, shaped like the
 * reference's Rust API of the path it replaces:
 *   scheme::advance(state, hydro, model, mesh, geometry, runtime, fold)
 *       -> Result<State, HydroError>                      (src/scheme.rs:212-240)
 *   State { time, iteration, solution: HashMap<BlockIndex, BlockState> },
 *   BlockState { conserved, scalar_mass }                  (src/state.rs:27-43)
 *   HydroError { source, position (r, theta) }            (src/physics/mod.rs:83-130)
 *   RelativisticHydro / NewtonianHydro, Mesh   (src/physics/{relativistic,newtonian}_hydro.rs,
 *                                                src/mesh.rs:84-113)
 * Header only, C++17. The device state lives in an Engine (one knc_ctx on
 * the current device); `advance` moves a State through it the way the
 * reference moves its State through scheme::advance. A zone's failed
 * recovery throws HydroError (the reference returns it as a value and never
 * panics); any other failed call throws knc::Error.
 */
#pragma once

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "knc.h"

namespace knc {

enum class RungeKuttaOrder { RK1 = 1, RK2 = 2, RK3 = 3 };
enum class RiemannSolver { HLLE = KNC_RIEMANN_HLLE, HLLC = KNC_RIEMANN_HLLC };

// src/physics/relativistic_hydro.rs:15-36
struct RelativisticHydro {
    double gamma_law_index = 4.0 / 3.0;
    double plm_theta = 1.5;
    double cfl_number = 0.4;
    RungeKuttaOrder runge_kutta_order = RungeKuttaOrder::RK2;
    RiemannSolver riemann_solver = RiemannSolver::HLLE;
    bool adaptive_time_step = false;

    knc_hydro_params to_c() const {
        knc_hydro_params p{};
        p.system = KNC_SYSTEM_RELATIVISTIC;
        p.runge_kutta_order = static_cast<int32_t>(runge_kutta_order);
        p.riemann_solver = static_cast<int32_t>(riemann_solver);
        p.adaptive_time_step = adaptive_time_step ? 1 : 0;
        p.gamma_law_index = gamma_law_index;
        p.plm_theta = plm_theta;
        p.cfl_number = cfl_number;
        return p;
    }
};

// src/physics/newtonian_hydro.rs:15-28 (always an adaptive time step)
struct NewtonianHydro {
    double gamma_law_index = 5.0 / 3.0;
    double plm_theta = 1.5;
    double cfl_number = 0.4;
    RungeKuttaOrder runge_kutta_order = RungeKuttaOrder::RK2;
    RiemannSolver riemann_solver = RiemannSolver::HLLE;

    knc_hydro_params to_c() const {
        knc_hydro_params p{};
        p.system = KNC_SYSTEM_NEWTONIAN;
        p.runge_kutta_order = static_cast<int32_t>(runge_kutta_order);
        p.riemann_solver = static_cast<int32_t>(riemann_solver);
        p.adaptive_time_step = 1;
        p.gamma_law_index = gamma_law_index;
        p.plm_theta = plm_theta;
        p.cfl_number = cfl_number;
        return p;
    }
};

// src/mesh.rs:84-113; the Option<> fields are std::pair<bool, T>
struct Mesh {
    double reference_radius = 1.0;
    double inner_radius = 1.0;
    double outer_radius = 10.0;
    double inner_excision_speed = 0.0;
    double outer_excision_speed = 0.0;
    std::pair<bool, double> excision_delay{false, 0.0};
    std::pair<bool, int64_t> num_radial_zones{false, 0};
    int64_t num_polar_zones = 128;
    int64_t block_size = 64;

    knc_mesh_params to_c() const {
        knc_mesh_params p{};
        p.reference_radius = reference_radius;
        p.inner_radius = inner_radius;
        p.outer_radius = outer_radius;
        p.inner_excision_speed = inner_excision_speed;
        p.outer_excision_speed = outer_excision_speed;
        p.excision_delay = excision_delay.second;
        p.has_excision_delay = excision_delay.first ? 1 : 0;
        p.num_radial_zones = num_radial_zones.second;
        p.has_num_radial_zones = num_radial_zones.first ? 1 : 0;
        p.num_polar_zones = num_polar_zones;
        p.block_size = block_size;
        return p;
    }
};

using BlockIndex = int32_t;   // BlockIndex (i, 0): the radial block number

struct BlockState {
    int64_t nr = 0, nq = 0;
    std::vector<double> conserved;     // [nr][nq][4]: D, S_r, S_theta, tau, volume integrated
    std::vector<double> scalar_mass;   // [nr][nq]
};

struct Rational {   // the reference's Rational64 iteration
    int64_t num = 0, den = 1;
};

struct State {
    double time = 0.0;
    Rational iteration;
    std::map<BlockIndex, BlockState> solution;
};

// A library call that failed for another reason than a zone's recovery.
class Error : public std::runtime_error {
public:
    Error(int status, const std::string& what) : std::runtime_error(what), status(status) {}
    int status;
};

// HydroError::at_position: the failing zone, its centroid and value.
class HydroError : public Error {
public:
    HydroError(int status, const knc_error& e)
        : Error(status, e.message), kind(e.kind), block(e.block), i(e.i), j(e.j), r(e.r), theta(e.theta),
          value(e.value) {}
    int kind;        // KNC_HYDRO_*
    BlockIndex block;
    int i, j;
    double r, theta;
    double value;
};

// The device state of one simulation (a knc_ctx on the current device).
class Engine {
public:
    template <class Hydro>
    Engine(const Hydro& hydro, const Mesh& mesh) {
        const knc_hydro_params h = hydro.to_c();
        const knc_mesh_params m = mesh.to_c();
        const int st = knc_create(&h, &m, &ctx_);
        if (st != KNC_OK) throw Error(st, std::string("knc_create: ") + knc_status_string(st));
    }
    ~Engine() {
        if (ctx_) knc_destroy(ctx_);
    }
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;
    Engine(Engine&& o) noexcept : ctx_(o.ctx_) { o.ctx_ = nullptr; }
    Engine& operator=(Engine&& o) noexcept {
        std::swap(ctx_, o.ctx_);
        return *this;
    }

    knc_ctx* handle() const { return ctx_; }

    void set_model(const knc_model_params& model) { check(knc_set_model(ctx_, &model), "knc_set_model"); }
    void set_precision(int32_t precision) { check(knc_set_precision(ctx_, precision), "knc_set_precision"); }
    void set_batched(bool graph) { check(knc_set_batched(ctx_, graph ? 1 : 0), "knc_set_batched"); }
    // KNC_GUESS_PLAIN (weights unused) or KNC_GUESS_MLP with a packed weight
    // vector of knc_mlp_num_params() floats
    void set_c2p_guess(int32_t guess, const std::vector<float>& weights = {}) {
        check(knc_set_c2p_guess(ctx_, guess, weights.empty() ? nullptr : weights.data(), weights.size()),
              "knc_set_c2p_guess");
    }
    // uneven blocks: (nr, nq) of block indexes first .. first + nr.size() - 1
    void set_block_shapes(int32_t first, const std::vector<int32_t>& nr, const std::vector<int32_t>& nq) {
        if (nr.size() != nq.size()) throw Error(KNC_ERR_INVALID_ARGUMENT, "set_block_shapes: nr and nq differ in length");
        check(knc_set_block_shapes(ctx_, first, (int32_t)nr.size(), nr.data(), nq.data()), "knc_set_block_shapes");
    }
    void set_tuning(const knc_tuning& t) { check(knc_set_tuning(ctx_, &t), "knc_set_tuning"); }
    knc_tuning autotune(int32_t reps = 3) {
        knc_tuning t{};
        check(knc_autotune(ctx_, reps, &t, nullptr), "knc_autotune");
        return t;
    }

    // State::from_model at time t (src/state.rs:55-69, 128-130)
    State from_model(double time) {
        check(knc_init_from_model(ctx_, time), "knc_init_from_model");
        return state();
    }

    // State::time_step (src/state.rs:143-162)
    double time_step() {
        double dt = 0.0;
        check(knc_time_step(ctx_, &dt), "knc_time_step");
        return dt;
    }

    // The blocks, time and iteration of `s` replace the device's.
    void load(const State& s) {
        std::vector<int32_t> have(count());
        if (!have.empty()) check(knc_block_indexes(ctx_, have.data(), (int32_t)have.size()), "knc_block_indexes");
        for (int32_t i : have)
            if (!s.solution.count(i)) check(knc_remove_block(ctx_, i), "knc_remove_block");
        for (const auto& kv : s.solution)
            check(knc_add_block(ctx_, kv.first, kv.second.conserved.data(), kv.second.scalar_mass.data()),
                  "knc_add_block");
        check(knc_set_time(ctx_, s.time, s.iteration.num, s.iteration.den), "knc_set_time");
    }

    // The device's blocks, time and iteration.
    State state() const {
        State s;
        check(knc_get_time(ctx_, &s.time, &s.iteration.num, &s.iteration.den), "knc_get_time");
        std::vector<int32_t> idx(count());
        if (!idx.empty()) check(knc_block_indexes(ctx_, idx.data(), (int32_t)idx.size()), "knc_block_indexes");
        for (int32_t i : idx) {
            BlockState b;
            check(knc_block_shape_of(ctx_, i, &b.nr, &b.nq), "knc_block_shape_of");
            b.conserved.resize((size_t)(b.nr * b.nq * 4));
            b.scalar_mass.resize((size_t)(b.nr * b.nq));
            check(knc_get_block(ctx_, i, b.conserved.data(), b.scalar_mass.data()), "knc_get_block");
            s.solution.emplace(i, std::move(b));
        }
        return s;
    }

    // `fold` steps with one time step (scheme::advance's loop).
    void advance(int32_t fold) { check(knc_advance(ctx_, fold), "knc_advance"); }

private:
    int32_t count() const {
        int32_t n = 0;
        check(knc_num_blocks(ctx_, &n), "knc_num_blocks");
        return n;
    }
    void check(int st, const char* what) const {
        if (st == KNC_OK) return;
        knc_error e{};
        knc_last_error(ctx_, &e);
        if (st == KNC_ERR_HYDRO) throw HydroError(st, e);
        throw Error(st, std::string(what) + ": " + knc_status_string(st) + (e.message[0] ? std::string(": ") + e.message : ""));
    }
    knc_ctx* ctx_ = nullptr;
};

// scheme::advance: the state in, the state `fold` steps later out, through
// the engine's device (which holds hydro, mesh, model and geometry).
inline State advance(State state, Engine& engine, int32_t fold) {
    engine.load(state);
    engine.advance(fold);
    return engine.state();
}

}  // namespace knc
