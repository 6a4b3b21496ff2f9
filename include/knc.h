/*
 * knc.h — C ABI of the GB300 finite-volume stage library (libknc_gpu.so).
 *
 * The library replaces the Runge–Kutta hot path of the Clemson Kilonova Code:
 * `scheme::advance` (src/scheme.rs:212-240) together with the per-block stage
 * `try_advance_rk` (src/scheme.rs:16-173), the state operations it relies on
 * (src/state.rs:55-244), the block geometry (src/mesh.rs:119-407) and the
 * per-zone physics reached through the `Hydrodynamics` trait
 * (src/traits.rs:41-136; src/physics/relativistic_hydro.rs:42-165,
 * src/physics/newtonian_hydro.rs:34-133).
 *
 * Conventions
 *  - Every entry point returns an int status: KNC_OK (0) or a KNC_ERR_* code.
 *    A hydro failure inside a stage (negative density, negative energy,
 *    root-finder failure) is a value, never a crash, exactly as
 *    `HydroError` is in the reference (src/physics/mod.rs:83-117);
 *    `knc_last_error` returns the first failing zone with its (r, theta).
 *  - Conserved data crossing the ABI is volume-integrated (the reference's
 *    `BlockState.conserved` is U·dV, src/state.rs:62-63) and array-of-structs
 *    `[nr][nq][4]` in the reference's component order (D, S_r, S_theta, tau)
 *    for relativistic hydro and (rho, rho v_r, rho v_theta, E) for Newtonian.
 *    The scalar mass is `[nr][nq]`.
 *  - The device owns the live state; host buffers are only read or written
 *    inside the call that receives them.
 *  - One context = one CUDA stream on the current device; a context must be
 *    driven from one host thread at a time.
 */
#ifndef KNC_H
#define KNC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    KNC_OK = 0,
    KNC_ERR_INVALID_ARGUMENT = 1,   /* bad pointer, size, or parameter       */
    KNC_ERR_CONFIG = 2,             /* mesh / hydro validation failed        */
    KNC_ERR_CUDA = 3,               /* a CUDA runtime call failed            */
    KNC_ERR_NO_BLOCK = 4,           /* block index not present               */
    KNC_ERR_HYDRO = 5,              /* a zone failed in c2p (see last_error) */
    KNC_ERR_UNSUPPORTED = 6,        /* combination not built                 */
    KNC_ERR_OUT_OF_MEMORY = 7,
    KNC_ERR_TIMEOUT = 8             /* a bounded device wait gave up         */
};

/* ---- hydro error kinds (src/physics/mod.rs:83-95) ------------------------ */
enum {
    KNC_HYDRO_NONE = 0,
    KNC_HYDRO_NEGATIVE_DENSITY = 1,
    KNC_HYDRO_NEGATIVE_PRESSURE = 2,
    KNC_HYDRO_NEGATIVE_ENERGY_DENSITY = 3,
    KNC_HYDRO_ROOT_FINDER_FAILED = 4
};

/* ---- enumerations of the configuration --------------------------------- */
enum { KNC_SYSTEM_RELATIVISTIC = 0, KNC_SYSTEM_NEWTONIAN = 1 };  /* AnyHydro, src/app.rs:86-89 */
enum { KNC_RIEMANN_HLLE = 0, KNC_RIEMANN_HLLC = 1 };             /* src/physics/mod.rs:27-30   */
enum { KNC_PRECISION_FP64 = 0, KNC_PRECISION_MIXED = 1 };
enum { KNC_GUESS_PLAIN = 0, KNC_GUESS_MLP = 1 };

/* Initial / boundary models, evaluated on the device (src/traits.rs:145-164). */
enum {
    KNC_MODEL_WIND = 0,      /* cold radial wind rho ~ r^-2, u^r = const            */
    KNC_MODEL_JET = 1,       /* wind-like ambient + W=const nozzle at the inner edge */
    KNC_MODEL_SPHERE = 2,    /* Newtonian over-dense sphere at rest                  */
    KNC_MODEL_HOST = 3,      /* host callback (slow path, no graph capture)          */
    KNC_MODEL_JET_IN_CLOUD = 4,   /* src/models/jet_in_cloud.rs:74-257               */
    KNC_MODEL_KINETIC_BOMB = 5,   /* src/models/kinetic_bomb.rs:78-114               */
    KNC_MODEL_JET_IN_STAR = 6     /* src/models/jet_in_star.rs:87-236                */
};

/*
 * Mirror of `RelativisticHydro` (src/physics/relativistic_hydro.rs:15-36) and
 * `NewtonianHydro` (src/physics/newtonian_hydro.rs:15-28). Newtonian hydro
 * ignores `adaptive_time_step` (always adaptive, newtonian_hydro.rs:79-81).
 * `riemann_solver` = KNC_RIEMANN_HLLC for Newtonian selects a Toro HLLC flux,
 * an extension (the reference's Newtonian adapter is HLLE only).
 */
typedef struct knc_hydro_params {
    int32_t system;             /* KNC_SYSTEM_*                          */
    int32_t runge_kutta_order;  /* 1, 2 or 3 (RungeKuttaOrder RK1..RK3)  */
    int32_t riemann_solver;     /* KNC_RIEMANN_*                         */
    int32_t adaptive_time_step; /* 0 / 1                                 */
    double gamma_law_index;
    double plm_theta;           /* [1, 2]                                */
    double cfl_number;          /* [0, 0.7]                              */
} knc_hydro_params;

/* Mirror of `Mesh` (src/mesh.rs:84-113). Option<> fields use a has_ flag. */
typedef struct knc_mesh_params {
    double reference_radius;
    double inner_radius;
    double outer_radius;
    double inner_excision_speed;
    double outer_excision_speed;
    double excision_delay;          /* used when has_excision_delay != 0 */
    int64_t num_radial_zones;       /* per decade; used when has_num_radial_zones */
    int64_t num_polar_zones;
    int64_t block_size;
    int32_t has_num_radial_zones;
    int32_t has_excision_delay;
} knc_mesh_params;

/*
 * Device-side model selection. Parameters by kind:
 *  WIND  : p[0]=rho at r=1, p[1]=u^r, p[2]=p/rho, p[3]=noise amplitude
 *  JET   : p[0]=rho at r=1, p[1]=p/rho, p[2]=noise amplitude,
 *          p[3]=nozzle half-opening angle, p[4]=jet Lorentz factor,
 *          p[5]=jet density / ambient density, p[6]=injection radius
 *          (zones with r < p[6] and theta within p[3] of a pole carry the
 *          jet; with p[6] at the inner mesh edge only the inner ghost block
 *          does, so the jet enters through the inner boundary)
 *  SPHERE: p[0]=rho inside, p[1]=rho outside, p[2]=sphere radius,
 *          p[3]=pressure, p[4]=noise amplitude
 *  JET_IN_CLOUD: the fields of JetInCloud in declaration order
 *          (cloud_mass, engine_delay, engine_duration, engine_strength,
 *          engine_theta, engine_u, envelop_m1, envelop_slowest_beta,
 *          envelop_fastest_beta, envelop_psi)
 *  KINETIC_BOMB: (external_medium_density, launch_radius, shell_thickness,
 *          kinetic_energy, shell_mass)
 *  JET_IN_STAR: (star_mass, engine_duration, engine_energy, engine_theta,
 *          engine_u, envelope_radius, envelope_mass, volume_factor)
 * Noise multiplies the density by (1 + amp * U[0,1)) with U a counter-based
 * hash of (seed, block index, i, j); it enters only the initial data, never
 * the ghost blocks, so `primitive_at` stays a pure function of (r, theta, t).
 */
typedef struct knc_model_params {
    int32_t kind;
    int32_t reserved;
    uint64_t seed;
    double p[16];
} knc_model_params;

/* Host model callback: AnyPrimitive order [u_r, u_theta, rho, p]
 * (src/physics/mod.rs:59-63) and the scalar concentration. */
typedef void (*knc_primitive_at_fn)(double r, double theta, double t,
                                    double out_any_primitive[4],
                                    double* out_scalar, void* user);

/* First failing zone of the last failed call (HydroError, src/physics/mod.rs:109-117). */
typedef struct knc_error {
    int32_t kind;        /* KNC_HYDRO_*                 */
    int32_t block;       /* block index (i32 of BlockIndex) */
    int32_t i, j;        /* zone within the block        */
    double r, theta;     /* cell centroid                */
    double value;        /* offending value              */
    char message[256];   /* human readable, includes CUDA errors */
} knc_error;

typedef struct knc_ctx knc_ctx;

/* ---- lifecycle --------------------------------------------------------- */

/* Validate (Mesh::validate src/mesh.rs:273-299, RelativisticHydro::validate
 * relativistic_hydro.rs:46-54) and create a context on the current device. */
int knc_create(const knc_hydro_params* hydro, const knc_mesh_params* mesh,
               knc_ctx** out);
void knc_destroy(knc_ctx* ctx);
const char* knc_status_string(int status);
int knc_last_error(const knc_ctx* ctx, knc_error* out);

/* ---- model and state (src/state.rs:55-69, 107-115; src/app.rs:315-330) ---- */

int knc_set_model(knc_ctx* ctx, const knc_model_params* model);
int knc_set_host_model(knc_ctx* ctx, knc_primitive_at_fn fn, void* user);

/* State::from_model over Mesh::grid_blocks(time) (src/mesh.rs:384-397):
 * replaces every block, sets time and iteration = 0. */
int knc_init_from_model(knc_ctx* ctx, double time);

/* Insert or replace one block (BlockIndex (index, 0), src/mesh.rs:12).
 * cons_aos: [block_size][num_polar_zones][4]; scalar_mass: [..][..]. */
int knc_add_block(knc_ctx* ctx, int32_t index, const double* cons_aos,
                  const double* scalar_mass);
int knc_remove_block(knc_ctx* ctx, int32_t index);
int knc_get_block(knc_ctx* ctx, int32_t index, double* cons_aos,
                  double* scalar_mass);
int knc_num_blocks(const knc_ctx* ctx, int32_t* n);
int knc_block_indexes(const knc_ctx* ctx, int32_t* out, int32_t capacity);
int knc_block_shape(const knc_ctx* ctx, int64_t* nr, int64_t* nq);

/* Uneven blocks (no counterpart in the reference, whose blocks all have
 * Mesh::block_size x num_polar_zones zones, src/mesh.rs:84-113): indexes
 * [first, first + count) get nr[k] radial and nq[k] polar zones over the same
 * radial extent; other indexes keep the mesh's shape. nq must be the mesh's
 * num_polar_zones times a power of two (so polar grids nest), nr in
 * [2, 16383]. Where neighbours differ in nq, the halo rows are remapped: a
 * finer neighbour's zones merged conservatively and recovered, a coarser one's
 * copied. Set shapes before the blocks become live (init, add, activation);
 * changing the shape of a live block is KNC_ERR_INVALID_ARGUMENT. Block
 * arrays of knc_add_block / knc_get_block / the state copies use each block's
 * own shape. */
int knc_set_block_shapes(knc_ctx* ctx, int32_t first, int32_t count, const int32_t* nr,
                         const int32_t* nq);
int knc_block_shape_of(const knc_ctx* ctx, int32_t index, int64_t* nr, int64_t* nq);

/* Whole-state copies for host-resident drivers: blocks in ascending index
 * order, each [nr][nq][4] then [nr][nq]; sizes must match the live state. */
int knc_set_state(knc_ctx* ctx, const double* cons_aos, const double* scalar_mass);
int knc_get_state(knc_ctx* ctx, double* cons_aos, double* scalar_mass);

/* Primitives of one block recovered in FP64 from the live state, the data
 * `Products::try_from_state` exports (src/products.rs:43-66): [nr][nq][5] as
 * (rho, u_r, u_theta, p, scalar concentration). */
int knc_get_primitives(knc_ctx* ctx, int32_t index, double* prim);
/* BlockProducts::try_from_block_state (src/products.rs:43-66) of one block,
 * in the reference's layout: radial_vertices [nr+1], polar_vertices [nq+1],
 * primitive [nr][nq][4] in AnyPrimitive order (velocity_r, velocity_q,
 * mass_density, gas_pressure; four-velocity components for relativistic
 * hydro, physics/mod.rs:36-63), scalar [nr][nq] = scalar_mass /
 * lab_frame_mass of the volume-integrated state. The primitives are recovered
 * in FP64 from the live state; any output may be NULL. */
int knc_get_products(knc_ctx* ctx, int32_t index, double* radial_vertices, double* polar_vertices,
                     double* primitive, double* scalar);

/* State.time and State.iteration (Rational64 as num/den), src/state.rs:39-43 */
int knc_set_time(knc_ctx* ctx, double time, int64_t iter_num, int64_t iter_den);
int knc_get_time(const knc_ctx* ctx, double* time, int64_t* iter_num,
                 int64_t* iter_den);

/* ---- the hot path ------------------------------------------------------ */

/* State::time_step (src/state.rs:143-162). */
int knc_time_step(knc_ctx* ctx, double* dt);

/* scheme::advance (src/scheme.rs:212-240): dt once, then `fold` times
 * {add_remove_blocks if the excision surfaces move; one RK step}. */
int knc_advance(knc_ctx* ctx, int32_t fold);
/* scheme::advance with the time step given by the caller instead of
 * State::time_step: a driver that splits the mesh into radial slabs (one
 * context per slab) passes the minimum of every slab's knc_time_step, the
 * one reduction the decomposition needs per advance. No counterpart in the
 * reference, which always advances the whole state. */
int knc_advance_dt(knc_ctx* ctx, int32_t fold, double dt);
/* scheme::advance (src/scheme.rs:212-240) in its own calling convention:
 * the state goes in and a new state comes out, both in host memory (the
 * whole-state layout of knc_set_state / knc_get_state; cons_out may alias
 * cons_in and scalar_out scalar_in). Equivalent to knc_set_state, knc_advance,
 * knc_get_state, and bitwise equal to them. The mesh must be fixed (moving
 * excision surfaces change the block set, and so the arrays' size, inside
 * the fold: KNC_ERR_INVALID_ARGUMENT). With page-locked buffers
 * (knc_host_alloc or registered), a device model, no remaps, more than one
 * polar zone, the fixed SRHD time step, the separate stage form and blocks
 * of at least 2 x runge_kutta_order rows at chunk boundaries, the first
 * step's upload and the last step's download run by chunks of blocks beside
 * the stages; otherwise the three calls run in turn. On failure the output buffers are unspecified
 * and the state must be set again. */
int knc_advance_host(knc_ctx* ctx, const double* cons_in, const double* scalar_in, double* cons_out,
                     double* scalar_out, int32_t fold);

/* Chosen forms. */
int knc_set_precision(knc_ctx* ctx, int32_t precision);          /* KNC_PRECISION_* */
/* weights: the packed MLP (see knc_mlp_num_params); NULL with KNC_GUESS_PLAIN. */
int knc_set_c2p_guess(knc_ctx* ctx, int32_t guess, const float* weights,
                      size_t n_weights);
/* graph != 0: capture each `fold` of RK steps in a CUDA graph and replay it. */
int knc_set_batched(knc_ctx* ctx, int32_t graph);
/* Launch shape of a stage (no counterpart in the reference, whose stage is a
 * Rayon/Tokio task per block, src/scheme.rs:16-173).
 *   tile_rows    radial rows of an update tile (4, 8 or 16; 32 polar columns;
 *                a tile runs on (tile_rows + 1) warps), or of a warp strip
 *                (4 to 64)
 *   fused        0: a stage is four launches (ghost rows, recovery, remaps,
 *                update; the deferring recovery adds its dense pass); 1: one
 *                persistent cooperative launch whose phases are separated by
 *                bounded grid barriers (bit-identical result). Mixed
 *                precision with warp strips and KNC_RECOVERY_DEFERRED: the
 *                deferring recovery, its dense pass, the remaps and the
 *                update in that one launch
 *   ctas_per_sm  fused grid = ctas_per_sm x SMs CTAs (0: the occupancy bound;
 *                larger values are clamped to it); mixed warp strips: the
 *                CTAs per SM the strip kernel's registers are sized for
 *                (4, 5 or 6; other values: 4); the fused deferring stage:
 *                1 runs one CTA of 20 warps per SM, 5 five CTAs of 4 warps,
 *                other values four CTAs of 4 warps
 *   update_form  separate form only: KNC_UPDATE_TILE, or KNC_UPDATE_TILE_TMA
 *                (mixed precision: each tile's primitives with halo, U_in and
 *                U_base staged by tensor copies into double-buffered shared
 *                memory, one tile ahead; used when every block has
 *                nq % 4 == 0, nq >= 40 and nr >= tile_rows), or
 *                KNC_UPDATE_STRIP (one warp per strip of 28 polar columns
 *                marching down tile_rows radial rows, no shared memory; needs
 *                num_polar_zones > 1). All forms give bit-identical states. */
enum { KNC_UPDATE_TILE = 0, KNC_UPDATE_TILE_TMA = 1, KNC_UPDATE_STRIP = 2 };
typedef struct knc_tuning {
    int32_t tile_rows;
    int32_t fused;
    int32_t ctas_per_sm;
    int32_t update_form;
    int32_t recovery_form;   /* mixed: KNC_RECOVERY_* (fused: with warp strips only) */
} knc_tuning;
/* KNC_RECOVERY_INLINE: each warp recovers its zones, the FP64 ones among
 * them in place; KNC_RECOVERY_DEFERRED: zones that need the FP64 recovery
 * are listed and recovered afterwards on full warps (with the learned guess)
 * by a second launch. Same bits either way. */
enum { KNC_RECOVERY_INLINE = 0, KNC_RECOVERY_DEFERRED = 1 };
int knc_set_tuning(knc_ctx* ctx, const knc_tuning* tuning);
int knc_get_tuning(const knc_ctx* ctx, knc_tuning* tuning);
/* Autotuner: times every candidate shape (tile rows x separate / fused x CTAs
 * per SM x update form) with `reps` first-stage launches each on the live state (they write
 * only the scratch buffer and primitives, so the state is unchanged), keeps
 * the fastest and returns it with its time per stage (either output may be
 * NULL). The stages are launched from the host one by one, so the fused
 * forms are candidates only when the context is not batched: inside a
 * batched context's captured graphs the separate launches' gaps are hidden
 * and they measured faster. */
int knc_autotune(knc_ctx* ctx, int32_t reps, knc_tuning* best, double* ms_per_stage);

/* Mixed precision: the Lorentz-factor split (default 2.0). Zones whose
 * Lorentz factor estimate exceeds it recover primitives in FP64 (below it
 * recovery runs in FP32), and every face whose 4-zone stencil holds a zone
 * above it is solved in FP64, with the zones it bounds updated in FP64. */
int knc_set_mixed_w_split(knc_ctx* ctx, double w_split);

/* Bounded waits, tested without a GPU fault. No counterpart in the
 * reference (its errors are values, src/traits.rs:78-82; this keeps the
 * library's device waits in that contract). knc_set_wait_test: the fused
 * stage's grid barriers give up after `polls` polls (0: the default, about
 * 0.3 s); with `unreachable` the first barrier of each fused stage counts one
 * arrival more than the grid makes, so it cannot complete and the stage fails
 * with KNC_ERR_TIMEOUT before any state is written. The context stays usable:
 * reload the state (knc_set_state) and advance. knc_selftest_copy_wait: one
 * CTA waits on an mbarrier that nothing arrives on, with the poll loop of the
 * tensor-copy update (no copy is issued); *timed_out = 1 when the wait gave
 * up after `polls` polls. */
int knc_set_wait_test(knc_ctx* ctx, int32_t polls, int32_t unreachable);
int knc_selftest_copy_wait(int32_t polls, int32_t* timed_out);

/* Wait for all work of the context; returns the first deferred error. */
int knc_synchronize(knc_ctx* ctx);

/* ---- statistics -------------------------------------------------------- */

/* Newton iterations summed over zones and c2p calls since the last reset,
 * split by the precision they ran in. */
int knc_c2p_stats(knc_ctx* ctx, int64_t* zones, int64_t* iters_fp64,
                  int64_t* iters_fp32, int64_t* fallbacks);
int knc_reset_c2p_stats(knc_ctx* ctx);
/* Kernel launches issued by the context since creation. */
int knc_launch_count(const knc_ctx* ctx, int64_t* launches);
/* Zone-updates since creation: the live zones summed over every RK step
 * advanced (the block set of a moving mesh changes between steps). */
int knc_zone_updates(const knc_ctx* ctx, int64_t* zone_updates);

/* Per-kernel timing with CUDA events on the context's stream. While enabled,
 * every launch is bracketed by events; knc_kernel_times returns, per kind
 * (KNC_KERNEL_*), the summed milliseconds and launch counts since enabling.
 * Not available while the steps run as a CUDA graph. */
enum { KNC_KERNEL_GHOST = 0, KNC_KERNEL_C2P = 1, KNC_KERNEL_UPDATE = 2, KNC_KERNEL_FUSED = 3,
       KNC_KERNEL_KINDS = 4 };
int knc_set_profiling(knc_ctx* ctx, int32_t on);
int knc_kernel_times(knc_ctx* ctx, double* ms, int64_t* launches);

/* Events on the context's stream: knc_mark records slot (0..7);
 * knc_elapsed_ms waits for slot b and returns the time from slot a to b. */
int knc_mark(knc_ctx* ctx, int32_t slot);
int knc_elapsed_ms(knc_ctx* ctx, int32_t a, int32_t b, double* ms);

/* Page-locked host buffers for host-resident drivers (cudaHostAlloc). */
int knc_host_alloc(size_t bytes, void** ptr);
/* The GPU that contexts created afterwards on the calling thread use
 * (cudaSetDevice), and the number of GPUs: one process per GPU under a
 * launcher that starts one rank per device. No counterpart in the
 * reference, which runs on the host. */
int knc_set_device(int32_t device);
int knc_device_count(int32_t* count);
int knc_host_free(void* ptr);

/* ---- learned c2p guess: MLP 3 -> 64 -> 64 -> 1 (SiLU) ------------------ */
/*
 * Packed float layout (offsets in floats):
 *   W1 [64][3]   @ 0      b1 [64] @ 192
 *   W2 [64][64]  @ 256    b2 [64] @ 4352      (row = output unit)
 *   W3 [64]      @ 4416   b3 [1]  @ 4480
 *   x_mean [3]   @ 4481   x_scale [3] @ 4484  (fixed input normalisation)
 * Forward: xn = (x - x_mean) * x_scale; h1 = silu(bf16(W1) xn + b1);
 * h2 = silu(bf16(W2) bf16(h1) + b2) with FP32 accumulation;
 * y = bf16(W3) . h2 + b3. The target is log(p / D); the pressure guess is
 * D * exp(y), clamped to (0, (gamma - 1) tau]. Inputs, all invariant under
 * U -> k U: x = (log(tau / D), -log(1 - |S| / (D + tau)),
 * log((tau (tau + 2 D) - S^2) / D^2)); the last is E^2 - S^2 - D^2 (E = tau + D),
 * which keeps the pressure resolvable in cold, highly relativistic states.
 */
#define KNC_MLP_HIDDEN 64
#define KNC_MLP_OFF_W1 0
#define KNC_MLP_OFF_B1 192
#define KNC_MLP_OFF_W2 256
#define KNC_MLP_OFF_B2 4352
#define KNC_MLP_OFF_W3 4416
#define KNC_MLP_OFF_B3 4480
#define KNC_MLP_OFF_XMEAN 4481
#define KNC_MLP_OFF_XSCALE 4484
#define KNC_MLP_NUM_PARAMS 4487

/* Number of floats in a packed weight vector (= KNC_MLP_NUM_PARAMS). */
size_t knc_mlp_num_params(void);

/* Training pairs from the solver: writes up to `capacity` rows of
 * [D, S_r, S_theta, tau, rho, u_r, u_theta, p] (per unit volume) sampled
 * from the live state of `ctx` (every `stride`-th zone). */
int knc_sample_pairs(knc_ctx* ctx, int32_t stride, double* out, int64_t capacity,
                     int64_t* written);

/* Synthetic pairs over Lorentz factor [w_lo, w_hi] and p/rho [t_lo, t_hi]
 * (log-uniform), produced on the device with the solver's prim->cons. */
int knc_generate_pairs(double gamma_law_index, double w_lo, double w_hi,
                       double t_lo, double t_hi, uint64_t seed, int64_t n,
                       double* out_host);

/* Train on the device: `pairs` [n][8] host rows as written above. Runs
 * `steps` Adam steps of `batch` rows; returns the final loss. Weights in/out. */
typedef struct knc_mlp_train_params {
    int64_t steps;
    int32_t batch;
    int32_t reserved;
    float lr;
    float beta1, beta2, eps;
    uint64_t seed;
} knc_mlp_train_params;
int knc_mlp_train(const double* pairs, int64_t n, float* weights,
                  const knc_mlp_train_params* params, float* final_loss);

/* Device forward / backward on one batch (for gradient checks): inputs x
 * [n][3] (already normalised features), targets y [n]; outputs prediction
 * [n], loss and the gradient of the loss wrt every packed parameter. */
int knc_mlp_forward_backward(const float* weights, const float* x, const float* y,
                             int32_t n, float* pred, float* loss, float* grad);

/* Features of a conserved state (see the MLP layout above); zeros when the
 * state has no usable features (the plain guess then applies). */
void knc_mlp_features(const double u[4], float out[3]);

/* ---- primitive recovery without device allocation ----------------------
 * No counterpart in the reference. For callers that own all device memory
 * themselves and cannot let a library call cudaMalloc: a host whose pool or
 * caching allocator holds the whole GPU (a library cudaMalloc could fail or
 * fragment it), or a time-critical loop that cannot take cudaMalloc's
 * implicit device synchronisation. Same result as knc_get_primitives, bit
 * for bit, from caller-owned device buffers:
 *   d_cons   [block_size][num_polar_zones][4] volume-integrated conserved
 *   d_scalar [block_size][num_polar_zones] scalar mass
 *   d_prim   [block_size][num_polar_zones][5] out: rho, u_r, u_theta, p,
 *            scalar concentration
 * for block (block_index, 0) of `mesh`, on `stream` (a cudaStream_t; NULL
 * for the default stream). Its only working memory is a fixed per-device
 * array inside the library (KNC_NOALLOC_MAX_ZONES cell volumes plus a status
 * word, 1 MiB; every GPU that loads the library holds it until the process
 * exits). Blocks larger than KNC_NOALLOC_MAX_ZONES zones are rejected with
 * KNC_ERR_INVALID_ARGUMENT. Each call resolves that array's address on the
 * current device. Calls share the array, so calls whose GPU work overlaps
 * race on it: serialise them. Returns after synchronising `stream` and
 * reading the array's status word back to the host; a failing zone gives
 * KNC_ERR_HYDRO with `err` (optional) filled like knc_last_error. */
#define KNC_NOALLOC_MAX_ZONES 131072
int knc_recover_primitives_noalloc(const knc_hydro_params* hydro, const knc_mesh_params* mesh,
                                   int32_t block_index, const double* d_cons,
                                   const double* d_scalar, double* d_prim, void* stream,
                                   knc_error* err);

/* ---- utilities --------------------------------------------------------- */

/* Self-test of the integer-pipe conversions the mixed stage uses: for n
 * doubles, writes the integer-pipe double->float and float->double results
 * and the hardware conversions (__double2float_rn, exact widening) beside
 * them: out[4 * k + 0..3] = (integer d2f, hardware d2f, integer f2d of the
 * hardware d2f, integer-pipe x / 2). */
int knc_test_conversions(const double* in, int64_t n, double* out);

/* Measured FP64 FMA throughput of the current device (GFLOP/s, 2/FMA). */
int knc_measure_fp64_peak(double* gflops);

#ifdef __cplusplus
}
#endif
#endif /* KNC_H */
