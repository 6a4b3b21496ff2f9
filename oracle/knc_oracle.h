/*
 * knc_oracle.h — CPU FP64 oracle of the KNC finite-volume RK stage.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker for the GPU library: only
 * tests/, the smoke entry point and the CPU-baseline leg of bench.py load it.
 * Nothing in the shipped library calls, links or includes it.
 *
 * PARITY UNPINNED: the reference's per-zone arithmetic lives in git crates
 * that are pinned in its Cargo.lock but not vendored (hydro-srhd @ 25bf21ec,
 * hydro-euler @ fc929f9b, godunov-core @ d8dd524a, ndarray-ops @ 725bc216),
 * no Rust toolchain exists to run it, and the reference ships no test,
 * fixture or golden value for this path. The oracle restates the reference's
 * own files exactly (src/scheme.rs, src/state.rs, src/mesh.rs,
 * src/physics/{relativistic,newtonian}_hydro.rs) and writes the crate-level physics from the published
 * methods named at each function in knc_oracle.cpp.
 *
 * The API mirrors include/knc.h (same parameter structs, same semantics) so
 * a test can drive the GPU library and the oracle with identical calls.
 */
#ifndef KNC_ORACLE_H
#define KNC_ORACLE_H

#include "../include/knc.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_ctx oracle_ctx;

int oracle_create(const knc_hydro_params* hydro, const knc_mesh_params* mesh,
                  int32_t threads, oracle_ctx** out);
void oracle_destroy(oracle_ctx* ctx);
int oracle_set_model(oracle_ctx* ctx, const knc_model_params* model);
int oracle_init_from_model(oracle_ctx* ctx, double time);
int oracle_add_block(oracle_ctx* ctx, int32_t index, const double* cons_aos,
                     const double* scalar_mass);
int oracle_remove_block(oracle_ctx* ctx, int32_t index);
/* Uneven blocks: shapes (nr, nq) of indexes [first, first + count); other
 * indexes keep (block_size, num_polar_zones). Neighbouring polar resolutions
 * must differ by a power of two (halo rows are remapped, see knc_oracle.cpp). */
int oracle_set_block_shapes(oracle_ctx* ctx, int32_t first, int32_t count, const int32_t* nr,
                            const int32_t* nq);
int oracle_block_shape_of(const oracle_ctx* ctx, int32_t index, int64_t* nr, int64_t* nq);
int oracle_get_block(oracle_ctx* ctx, int32_t index, double* cons_aos,
                     double* scalar_mass);
/* [nr][nq][5] = (rho, u_r, u_theta, p, scalar concentration) of a block. */
int oracle_get_primitives(oracle_ctx* ctx, int32_t index, double* prim);
/* BlockProducts of a block: vertices [nr+1], [nq+1]; primitive [nr][nq][4] in
 * AnyPrimitive order; scalar [nr][nq] = scalar_mass / lab_frame_mass. */
int oracle_get_products(oracle_ctx* ctx, int32_t index, double* rv, double* qv, double* prim, double* scalar);
int oracle_num_blocks(const oracle_ctx* ctx, int32_t* n);
int oracle_block_indexes(const oracle_ctx* ctx, int32_t* out, int32_t capacity);
int oracle_set_time(oracle_ctx* ctx, double time, int64_t num, int64_t den);
int oracle_get_time(const oracle_ctx* ctx, double* time, int64_t* num, int64_t* den);
int oracle_time_step(oracle_ctx* ctx, double* dt);
int oracle_advance(oracle_ctx* ctx, int32_t fold);
int oracle_advance_dt(oracle_ctx* ctx, int32_t fold, double dt);
int oracle_last_error(const oracle_ctx* ctx, knc_error* out);
/* Newton iterations summed since creation (c2p calls on live and ghost blocks). */
int oracle_c2p_stats(const oracle_ctx* ctx, int64_t* zones, int64_t* iters);

/* ---- point physics (unit tests and golden vectors) --------------------- */
/* Primitive order: SRHD (rho, u_r, u_theta, p), Newtonian (rho, v_r, v_theta, p). */
void oracle_prim_to_cons(const knc_hydro_params* h, const double p[4], double u[4]);
/* c2p of a per-volume conserved state; guess < 0 selects the plain guess.
 * Returns a KNC_HYDRO_* kind (NEGATIVE_PRESSURE means floored), iterations out. */
int oracle_cons_to_prim(const knc_hydro_params* h, const double u[4], double guess,
                        double p[4], int32_t* iterations);
/* Physical flux along axis 0 (radial) or 1 (polar) and the wave speeds. */
void oracle_flux(const knc_hydro_params* h, const double p[4], int32_t axis,
                 double f[4], double* lam_minus, double* lam_plus);
/* Godunov flux (HLLE or HLLC as h->riemann_solver) of (pl, sl) | (pr, sr),
 * WITHOUT the LIGHT_SPEED factor; out[0..3] hydro, out[4] scalar. */
void oracle_riemann(const knc_hydro_params* h, const double pl[4], const double pr[4],
                    double sl, double sr, int32_t axis, double out[5]);
double oracle_plm_gradient(double theta, double a, double b, double c);
/* Geometric source per unit volume at (r, theta), without LIGHT_SPEED. */
void oracle_sources(const knc_hydro_params* h, const double p[4], double r,
                    double theta, double s[4]);
double oracle_max_signal_speed(const knc_hydro_params* h, const double p[4]);

/* Block geometry exactly as src/mesh.rs:246-264 computes it. Sizes:
 * rv[nr+1], qv[nq+1], ar[(nr+1)*nq], aq[nr*(nq+1)], dv[nr*nq], rc[nr*nq], qc[nr*nq]. */
int oracle_block_geometry(const knc_mesh_params* m, int32_t index, double* rv, double* qv,
                          double* ar, double* aq, double* dv, double* rc, double* qc);

/* ---- learned c2p guess: CPU reference of the MLP (FP64) ---------------- */
/* Forward + backward of the packed MLP on n rows; grad has knc_mlp_num_params
 * entries. With round_bf16 != 0 the weights and the first hidden layer's
 * activations are rounded to bfloat16 as the device does (gradients are
 * straight-through); with 0 everything stays FP64, for finite differences. */
void oracle_mlp_forward_backward(const float* weights, const float* x, const float* y,
                                 int32_t n, int32_t round_bf16, double* pred, double* loss,
                                 double* grad);

#ifdef __cplusplus
}
#endif
#endif
