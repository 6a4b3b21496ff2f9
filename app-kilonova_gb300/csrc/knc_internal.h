// knc_internal.h — device data layout and kernel launchers shared by the
// host runtime (knc_api.cu) and the kernel translation units.
//
// HBM layout, per radial block (BlockIndex (i, 0), src/mesh.rs:12):
//   state   buf[2]  double [5][nr][nq]     D, S_r, S_theta, tau, scalar mass
//                                           (volume-integrated, theta fastest)
//   prims   P       [5][nr+4][nq]          rho, u_r, u_theta, p, s (double in the
//                                           FP64 path, float in the mixed path);
//                                           rows 0-1 and nr+2..nr+3 hold the radial
//                                           halo (neighbour rows or ghost rows)
//           P64     [5][nr+4][nq] double   mixed path: the same, written only for
//                                           zones above the Lorentz-factor split
//   geometry ar [nr+1][nq], aq [nr][nq+1], dv [nr][nq] (FP64, mesh.rs formulas),
//            rc [nr] centroid radii, rv [nr+1] vertices; per-column tables
//            qv [nq+1], qc [nq], cot [nq]; FP32 row/column factors for the
//            mixed path (areas and volumes separate into r- and theta-parts).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/knc.h"

namespace knc {

constexpr int TILE_R = 8;      // stage tile: rows (radial)
constexpr int TILE_Q = 32;     // stage tile: columns (polar), one warp wide
constexpr int TILE_THREADS = TILE_R * TILE_Q;
constexpr int NFIELD = 5;
constexpr int STRIP_OUT = TILE_Q - 4;   // output columns of a warp strip (2 halo lanes each side)
constexpr int STRIP_WARPS = 4;          // independent strips per CTA

struct DevBlock {
    double* buf[2];        // [5][nr][nq] state ping/pong
    void* P;               // [5][nr+4][nq] primitives with halo rows
    const double* ar;      // [nr+1][nq]
    const double* aq;      // [nr][nq+1]
    const double* dv;      // [nr][nq]
    const double* rc;      // [nr]
    const double* rv;      // [nr+1]
    const double* qv;      // [nq+1]
    const double* qc;      // [nq]
    const double* cot;     // [nq]
    // mixed path geometry factors, each an unevaluated FP32 pair hi + lo
    // (about 48 bits), with the flux scale c folded into the radial factors:
    //   c A_r(i,j) = ar_r[i] * ar_q[j]    ar_r = c r_i^2,  ar_q = pi (s0+s1) |chord|
    //   c A_q(i,j) = aq_r[i] * aq_q[j]    aq_r = c pi (r1^2 - r0^2), aq_q = sin(theta_j)
    //   c dV(i,j)  = dv_r[i] * dv_q[j]    dv_r = c (r1^3 - r0^3) 2 pi / 3, dv_q = cos0 - cos1
    // dV alone (for c2p) is dv_r / c * dv_q; the plain-FP32 dv_r32 holds it.
    const float2* ar_r;    // [nr+1] (hi, lo)
    const float2* ar_q;    // [nq]
    const float2* aq_r;    // [nr]
    const float2* aq_q;    // [nq+1]
    const float2* dv_r;    // [nr]
    const float2* dv_q;    // [nq]
    const float* dv_r32;   // [nr] (r1^3 - r0^3) 2 pi / 3 in FP32, without c
    const float* rc32;     // [nr]
    const float* cot32;    // [nq]
    // mixed stage: FP64 primitives [5][nr+4][nq] like P, written only for the
    // zones whose stored FP32 primitive is above the Lorentz-factor split
    // (own rows by the recovery, halo rows by the neighbours' recovery, the
    // ghost and the remap launches), read by zone_hp; null in the FP64 stage
    double* P64;
    void* P_in_nbr;        // inner neighbour's P: my rows 0,1 go to its rows nr'+2, nr'+3
    void* P_out_nbr;       // outer neighbour's P: my rows nr-2, nr-1 go to its rows 0, 1
    int32_t nr, nq;
    int32_t index;         // block index i of BlockIndex (i, 0)
    int32_t nr_in_nbr;     // rows of the inner neighbour
    int32_t nr_out_nbr;    // rows of the outer neighbour
    int32_t slot_in;       // slot of the inner neighbour, -1 at the inner edge
    int32_t slot_out;      // slot of the outer neighbour, -1 at the outer edge
    int32_t shadow;        // 1: a copy of a neighbour's edge rows (host-state chunks)
};

// Error key: lexicographic (stage, slot, i, j) with the hydro kind in the low
// bits; atomicMin keeps the first failure in that order.
__host__ __device__ inline unsigned long long error_key(uint32_t stage, uint32_t slot, uint32_t i,
                                                       uint32_t j, uint32_t kind) {
    return ((unsigned long long)(stage & 0xffffu) << 48) | ((unsigned long long)(slot & 0x3fffu) << 34) |
           ((unsigned long long)(i & 0x3fffu) << 20) | ((unsigned long long)(j & 0xffffu) << 4) |
           (unsigned long long)(kind & 0xfu);
}
constexpr unsigned long long NO_ERROR = ~0ull;

struct DevStatus {
    unsigned long long err_key;     // NO_ERROR or error_key(...)
    int32_t err_sel;                // state buffer the failing stage read
    int32_t pad;
    unsigned long long c2p_zones;
    unsigned long long iters_fp64;
    unsigned long long iters_fp32;
    unsigned long long fallbacks;
    unsigned long long dt_bits;     // min of dl/a over zones (double bits, positive)
    unsigned long long bar_count;   // grid-barrier arrivals of fused launches since the last reset
    int32_t bar_abort;              // a grid barrier gave up waiting
    int32_t pad2;
    unsigned high_count[2];         // deferred FP64 recoveries, by stage parity
    // mixed stage, by stage parity: the stored FP32 primitives above the
    // Lorentz-factor split listed by this stage (FP64 faces around them), and
    // the work items of that list the update has claimed
    unsigned hp_count[2];
    unsigned hp_claim[2];
    // the fused deferring stage: phase A's work items (ghost-row groups, then
    // recovery tiles) claimed by warps; zero between launches (each launch
    // zeroes it once its first barrier has passed, and every status reset
    // does, for a launch whose barrier gave up)
    unsigned item_claim;
    unsigned pad3;
};

struct StageArgs {
    const DevBlock* blocks;
    const int4* tiles;      // {slot, i0, j0, 0}, TILE_R x TILE_Q (recovery, init)
    int32_t ntiles;
    const int4* utiles;     // {slot, i0, j0, 0}, utr x TILE_Q (update)
    int32_t nutiles;
    int32_t utr;            // update tile rows: 4, 8 or 16
    int32_t tma;            // mixed update: stage tiles with tensor copies (tmaps valid)
    const int4* strips;     // {slot, i0, j0, rows}: warp strips of the strip form, or null
    int32_t nstrips;
    int32_t strip_ctas;     // strip form: CTAs per SM the kernel is built for (4, 5 or 6)
    int32_t fused_wide;     // fused deferring stage: one CTA of 20 warps per SM
    // adaptive dt found on the device (the fold's first recovery reduces
    // dl / a_max into *dt_bits): dt = *dt_bits x cfl replaces dt / dt_f
    const unsigned long long* dt_bits;
    double cfl;
    const void* tmaps;      // TmaMaps per slot (knc_tma.cuh), or null
    int32_t stage;          // stage counter for error ordering
    int32_t sel_in, sel_out, sel_base;   // state buffer selectors; sel_base < 0: no average
    int32_t srhd, hllc;
    int32_t one_dimensional;
    int32_t guess;          // KNC_GUESS_*
    int32_t compute_dt;     // c2p pass also reduces dl / a_max
    double gm, plm_theta;
    double dt;
    double w1, bf;          // out = (U + dU) w1 + U0 bf when sel_base >= 0
    double cflux;           // LIGHT_SPEED (SRHD) or 1
    double w_split;         // mixed path: Lorentz factor above which c2p runs in FP64
    double gh;              // gm / (gm - 1), rounded once on the host
    // FP32 copies rounded once on the host, so no thread converts or divides
    // in FP64 for them (on GB300 the FP64 pipe is the narrow one)
    float gm_f, gm1_f, gh_f, theta_f, dt_f, cflux_f;
    float high_thr_f;       // 1 - 1 / w_split^2: |S| / (D + tau) squared above it means W > w_split
    // mixed update: a zone whose stored FP32 four-velocity has
    // u_r^2 + u_theta^2 = W^2 - 1 above uu_high_f (W above the split) makes
    // every face whose 4-zone stencil reaches it an FP64 face (zone_hp)
    float uu_high_f;
    // mixed stage: every stored FP32 primitive above the Lorentz-factor split,
    // as {slot, padded row x nq + column} of the block whose P array holds it
    // (own rows and halo rows alike), appended by the recovery, ghost and
    // remap launches (hp_count entries); the update claims its zones with
    // FP64 faces from this list (hp_claim). The update of a stage clears the
    // next stage's counters. No list (null): every strip checks its own
    // stencil and updates such zones itself.
    int2* hp_list;
    unsigned* hp_count;
    unsigned* hp_claim;
    unsigned* hp_count_next;
    unsigned* hp_claim_next;
    unsigned hp_cap;
    // mixed stage length unit L = 2^e: its FP32 geometry is in units of L
    // (areas 2^(-2e), volumes 2^(-3e)), so increments scale back by 2^(2e)
    // and recovered densities use volumes in L^3
    int32_t lscale2, lscale3;   // 2e, 3e
    double lscale3_d;           // 2^(-3e)
    // mixed recovery, separate form: zones deferred to the dense FP64 pass
    int2* high;                 // {slot, z}, capacity = zones of the layout, or null
    unsigned* high_count;       // this stage's count (status word, by stage parity)
    unsigned* high_count_next;  // the next stage's, cleared by the dense pass
    unsigned high_cap;          // entries a.high holds
    int32_t avg_half;       // w1 == bf == 1/2 (the RK2 average, halved exactly on the integer pipe)
    const float* mlp;       // packed MLP weights (device) or null
    DevStatus* status;
};

struct GhostArgs {
    void* P[2];             // target P of the innermost / outermost block
    int32_t row0[2];        // first target row (0 for inner, nr+2 for outer)
    int32_t nr_t[2];        // target block rows (row stride nr+4)
    int32_t nq[2];          // polar zones of the innermost / outermost block
    int32_t ghost_index[2];
    const double* rc;       // [2 ends][2 rows]
    const double* dv[2];    // per end [2 rows][nq]
    const double* qc[2];    // per end [nq]
    const double* host_prim[2]; // per end [2][nq][5] model values from a host callback, or null
    knc_model_params model;
    double time;
    int32_t srhd;
    int32_t stage;
    double gm;
    int32_t single_precision;   // write float P
    // mixed stage: the target's FP64 primitive array (laid out like P[end]),
    // which takes the rows whose FP32 values are above the split, or null
    double* P64[2];
    // mixed stage: stored ghost zones above the Lorentz-factor split are
    // appended to the stage's list (StageArgs::hp_list) as zones of the edge
    // blocks (slots edge_slot[end], padded rows row0[end] + 0, 1)
    int2* hp_list;
    unsigned* hp_count;
    unsigned hp_cap;
    int32_t edge_slot[2];
    float uu_high_f;
    DevStatus* status;
    // adaptive dt found on the device in the fold's first recovery: the stage
    // time is then fold_stage_time(t0, dt, order, step, sub), dt = *dt_bits x cfl
    const unsigned long long* dt_bits;
    double cfl;
    double t0;
    int32_t order, step, sub, pad_;
};

// Fused-stage extras: recovery chunks {slot, z0, nz, 0} of at most
// update_threads(utr) consecutive zones of one block, the remap items, and the
// barrier base of this launch.
constexpr int BARRIER_SPIN_LIMIT = 1 << 22;   // grid-barrier polls of >= 64 ns: about 0.3 s or more

struct FusedArgs {
    const int4* chunks;
    int32_t nchunks;
    int32_t nremap;
    const int4* remap;
    int32_t max_nq;
    int32_t spin_limit;     // polls a grid barrier waits before it gives up
    unsigned long long bar_base;
};

struct InitArgs {
    const DevBlock* blocks;
    const int4* tiles;
    int32_t sel;
    int32_t srhd;
    int32_t noise;               // seeded density noise (initial data only)
    int32_t pad_;
    double gm;
    double time;
    knc_model_params model;
    const double* host_prim;     // [nzones][5] host model values (HOST model) or null
};

// Host geometry of block `index` (src/mesh.rs formulas): cell volumes
// [nr*nq], centroid radius per row [nr], centroid theta per column [nq].
void host_block_volumes(const knc_mesh_params& mesh, int32_t index, std::vector<double>& dv,
                        std::vector<double>& rc, std::vector<double>& qc);

// ---- launchers (each returns the cudaError_t of the launch) -------------
// Set the kernels' shared-memory attributes once, before any launch or capture.
cudaError_t configure_kernels();
cudaError_t launch_init_f64(const InitArgs& a, int ntiles, cudaStream_t s);
cudaError_t launch_c2p_f64(const StageArgs& a, cudaStream_t s);
cudaError_t launch_update_f64(const StageArgs& a, cudaStream_t s);
cudaError_t launch_ghost_f64(const GhostArgs& a, cudaStream_t s);
cudaError_t launch_ghost_mixed(const GhostArgs& a, cudaStream_t s);
cudaError_t launch_c2p_mixed(const StageArgs& a, cudaStream_t s);
cudaError_t launch_update_mixed(const StageArgs& a, cudaStream_t s);
cudaError_t launch_aos_to_soa(const double* aos, const double* scalar, double* soa, int64_t nr, int64_t nq,
                              cudaStream_t s);
// Halo rows across a change of polar resolution (power-of-two ratio).
// remap = {target slot, source slot, side (0: target rows 0-1 from the source's
// last two rows; 1: target rows nr+2..nr+3 from the source's first two)}.
cudaError_t launch_remap_f64(const StageArgs& a, const int4* remap, int nremap, int max_nq, cudaStream_t s);
cudaError_t launch_remap_mixed(const StageArgs& a, const int4* remap, int nremap, int max_nq, cudaStream_t s);
// One RK stage as one cooperative launch of `grid` CTAs (utr = a.utr); grid
// must not exceed fused_max_ctas() x SMs.
cudaError_t launch_stage_fused_f64(const StageArgs& a, const GhostArgs& g, const FusedArgs& f, int grid,
                                   cudaStream_t s);
cudaError_t launch_stage_fused_mixed(const StageArgs& a, const GhostArgs& g, const FusedArgs& f, int grid,
                                     cudaStream_t s);
// Resident CTAs per SM of the fused kernel for (precision, learned guess, tile rows).
cudaError_t fused_max_ctas_f64(bool mlp, int utr, int* per_sm);
cudaError_t fused_max_ctas_mixed(bool mlp, int utr, int* per_sm);
// The mixed fused stage with warp strips only (CTAs of STRIP_WARPS warps).
cudaError_t fused_strip_max_ctas_mixed(bool mlp, int* per_sm);
// The mixed fused stage with the deferring recovery and warp strips, built
// for mb resident CTAs per SM: 4 or 5 CTAs of 4 warps, or (mb = 1) one CTA
// of 20 warps; fused_deferred_threads(mb): its CTA size.
cudaError_t fused_deferred_max_ctas_mixed(bool mlp, int mb, int* per_sm);
int fused_deferred_threads(int mb);
// Threads of a fused / update CTA for tile rows utr.
inline int stage_threads(int utr) { return (utr + 1) * TILE_Q; }
// Tile rows the fused kernel is instantiated for: utr when it is a tile
// size, else 8 (warp strips of other lengths run in a CTA of 9 warps).
inline int fused_tr(int utr) { return utr == 4 || utr == 16 ? utr : 8; }
// Whole state <-> ABI arrays over the recovery tiles (cons/scalar: device or
// device-accessible host pointers).
cudaError_t launch_state_in(const DevBlock* blocks, const int4* tiles, int ntiles, int sel, const double* cons,
                            const double* scalar, cudaStream_t s);
cudaError_t launch_state_out(const DevBlock* blocks, const int4* tiles, int ntiles, int sel, double* cons,
                             double* scalar, cudaStream_t s);
cudaError_t launch_halo_rows(const void* src, void* dst, int nq, int nr, int row0, int elem_bytes, cudaStream_t s);
cudaError_t launch_prims_to_aos(const void* P, double* out, int64_t nr, int64_t nq, cudaStream_t s);
cudaError_t launch_products(const void* P, const double* U, double* prim, double* scalar, int64_t nr, int64_t nq,
                            cudaStream_t s);
cudaError_t launch_soa_to_aos(const double* soa, double* aos, double* scalar, int64_t nr, int64_t nq,
                              cudaStream_t s);
cudaError_t launch_sample_pairs(const DevBlock* blocks, const int4* tiles, int ntiles, int sel, int stride, double gm,
                                double* out, int64_t capacity, unsigned long long* counter, cudaStream_t s);

}  // namespace knc
