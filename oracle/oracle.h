/*
 * CPU oracle for the shallow-water transformer's forward pass and tick loop.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker that the CUDA library is
 * compared against, and the timed CPU baseline; it is never linked into the
 * product library and the product never calls it.
 *
 * It restates, operation for operation, the reference engine's CPU path:
 *   crates/engine/src/cpu.rs:26-352     (linear, layernorm, gelu, attention,
 *                                        conv2d, upsample, forward, step)
 *   crates/engine/src/mask.rs:18-30     (Mask::allowed)
 *   crates/engine/src/project.rs:9-54   (energy, mass, project_mass,
 *                                        project_energy)
 *   crates/engine-cli/src/eval.rs:144-157 (tick loop order: step, mass
 *                                        projection, energy projection,
 *                                        energy bookkeeping)
 * The f32 build keeps the reference's f32 arithmetic and summation order
 * (no FMA contraction, sequential sums) so it reproduces the reference's
 * numbers; the f64 build runs the same algorithm in double precision and is
 * the tolerance oracle for reduced-precision GPU forms.
 */
#ifndef JC_ORACLE_H
#define JC_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_LAYERS 32

/* config.json fields the engine reads (crates/engine/src/config.rs:13-41). */
typedef struct {
    int nx, ny, patch, channels, dim, layers, heads;
    int head_dim;   /* cell-head width, from head.to_cells.weight.shape[0] */
    int ff_inner;   /* from blocks.0.ff1.weight.shape[1] */
    int meta_dim;
    int mask_kind;  /* 0 = Full, 1 = Stencil */
    int radius, dilation;
    float norm_mean[3], norm_std[3], norm_depth;
    float g, energy_r_max;
} orc_config;

/* Pointers into the checkpoint's F32 tensors, laid out exactly as
 * model.safetensors stores them (docs/pytorch-training.md:25-47). */
typedef struct {
    const float *n1g, *n1b, *qw, *qb, *kw, *kb, *vw, *vb, *pw, *pb;
    const float *n2g, *n2b, *f1w, *f1b, *f2w, *f2b;
} orc_block;

typedef struct {
    const float *embed_w, *embed_b, *meta_w, *meta_b, *pos;
    orc_block blk[ORC_MAX_LAYERS];
    const float *norm_g, *norm_b;
    const float *tm_w, *tm_b, *tc_w, *tc_b, *c1_w, *c1_b, *c2_w, *c2_b;
} orc_weights;

/* Tick-loop flags. */
#define ORC_MASS   1u   /* project_mass after each step */
#define ORC_ENERGY 2u   /* project_energy after each step */
#define ORC_SUM64  4u   /* projection sums in f64 (Neumaier) instead of the
                           reference's sequential f32 sums */

/* Attention enumeration: 0 = scan every key with the mask predicate, as
 * cpu.rs:121-158 does (O(T^2), the reference's own cost); 1 = visit only the
 * stencil candidates in increasing key order (same arithmetic, same bits). */
void orc_set_attention_mode(int mode);
void orc_set_threads(int n);
int  orc_get_threads(void);

/* forward: state [channels, ny, nx], meta [meta_dim] -> increment. */
void orc_forward_f32(const orc_config* c, const orc_weights* w,
                     const float* state, const float* meta, float* out);
void orc_forward_f64(const orc_config* c, const orc_weights* w,
                     const double* state, const double* meta, double* out);

/* Rollout of `ticks` ticks from x0. `traj` receives ticks+1 states
 * (x0 first) when non-NULL; `final_state` the last one when non-NULL;
 * `energies` ticks+1 energies when non-NULL. Returns the max relative
 * energy violation max((E_t - E_{t-1} r_max)/E_{t-1}, 0). */
double orc_rollout_f32(const orc_config* c, const orc_weights* w,
                       const float* x0, const float* meta, int ticks,
                       unsigned flags, float* traj, float* final_state,
                       double* energies);
double orc_rollout_f64(const orc_config* c, const orc_weights* w,
                       const double* x0, const double* meta, int ticks,
                       unsigned flags, double* traj, double* final_state,
                       double* energies);

/* project.rs restated, f32 sequential sums (reference arithmetic). */
float orc_mass_f32(const float* x, int n);
float orc_energy_f32(const float* x, const orc_config* c, int n);
void  orc_project_mass_f32(float* x, float target, int n);
void  orc_project_energy_f32(float* x, float prev_energy, const orc_config* c, int n);

/* Same projections with f64 compensated sums (the GPU's definition). */
double orc_mass_sum64(const float* x, int n);
double orc_energy_sum64(const float* x, const orc_config* c, int n);
void   orc_project_mass_sum64(float* x, double target, int n);
void   orc_project_energy_sum64(float* x, double prev_energy, const orc_config* c, int n);

/* ---- evaluation path (solver.c) ----
 * Shallow-water solver parameters (crates/solvers/src/shallow_water.rs:16-29). */
typedef struct {
    int nx, ny;
    float dx, dt, g, depth, nu;
} orc_sw_params;

/* State::add_drop: h += amp exp(-r^2 / (2 sigma^2)), expf of the C library. */
void   orc_sw_add_drop(const orc_sw_params* p, float* h, float cx, float cy, float amp, float sigma);
double orc_sw_mass(const float* h, int n);
/* `steps` ShallowWater::step calls on the planes h, u, v [ny, nx]. */
void   orc_sw_steps(const orc_sw_params* p, float* h, float* u, float* v, int steps);

/* metrics.rs restated. */
float orc_correlation(const float* a, const float* b, int n);
float orc_peak(const float* f, int n);
float orc_mean(const float* f, int n);
float orc_std_dev(const float* f, int n);
float orc_bias(const float* model, const float* solver, int n);
int   orc_radial_profile(const float* f, int nx, int ny, float cx, float cy, double* out, int cap);
float orc_xcorr_lag(const double* model, const double* solver, int n, int max_lag);
float orc_rmse(const float* a, const float* b, int n);
void  orc_encode(const float norm_mean[3], const float norm_std[3], float norm_depth, const float* h,
                 const float* u, const float* v, int n, float* out);
/* One eval-metrics row: corr (h,u,v), corr (h), amplitude ratio, wavefront
 * lag (cells), bias. */
void  orc_eval_score(const float norm_mean[3], const float norm_std[3], float norm_depth, int nx, int ny,
                     const float* x, const float* h, const float* u, const float* v, float cx, float cy,
                     float row[5]);

#ifdef __cplusplus
}
#endif
#endif
