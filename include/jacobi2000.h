/*
 * jacobi2000 GB300 engine: C ABI.
 *
 * A drop-in for the reference engine crate's model API. Each entry point
 * names the reference interface it replaces. Conventions:
 *   - plain pointers and sizes, caller-owned buffers; no C++ or framework types;
 *   - every function returns a jc_status; nothing panics or aborts across the
 *     boundary; jc_last_error() gives a thread-local message for the last
 *     failure on the calling thread;
 *   - states are normalized f32 [channels, ny, nx] (channel 0 = h, 1 = u,
 *     2 = v), the layout of crates/engine/src/norm.rs:1-3;
 *   - a model handle owns one CUDA stream; calls on one handle must not run
 *     concurrently from several threads (use one handle per thread).
 */
#ifndef JACOBI2000_H
#define JACOBI2000_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. 1-4 mirror lean_runtime::Error::{NoAdapter/NoDevice, Limit,
 * Map, Poll} (crates/lean-runtime/src/error.rs:6-13); the rest replace the
 * reference's panics on bad checkpoints (weights.rs:39,52-54, config.rs:71). */
typedef enum {
    JC_OK = 0,
    JC_NO_DEVICE = 1,       /* no CUDA device, or not an sm_103 device */
    JC_LIMIT = 2,           /* a size exceeds a kernel limit */
    JC_MAP = 3,             /* a host<->device copy failed */
    JC_POLL = 4,            /* waiting for the device failed */
    JC_BAD_CHECKPOINT = 5,  /* safetensors / config.json malformed or missing a tensor */
    JC_BAD_SHAPE = 6,       /* grid not divisible by the patch, shapes inconsistent */
    JC_OVER_BUDGET = 7,     /* admission refused: device memory budget */
    JC_DEVICE_TIMEOUT = 8,  /* a device-side wait hit its iteration limit */
    JC_BAD_ARGUMENT = 9,    /* null pointer, negative count, unknown flag */
    JC_CUDA_ERROR = 10,     /* any other CUDA runtime error */
    JC_NOT_FOUND = 11       /* unknown request id */
} jc_status;

/* Arithmetic of a model's kernels. FP32: f32 weights and activations on CUDA
 * cores (the reference's arithmetic). BF16: bf16 weights and activations on
 * the tcgen05 tensor cores with f32 accumulation; LayerNorm statistics,
 * softmax, residual stream and the projection scalars stay f32/f64. */
typedef enum { JC_FP32 = 0, JC_BF16 = 1 } jc_precision;

/* Tick-loop flags (crates/engine-cli/src/eval.rs:144-157 order: step, mass
 * projection, energy projection). */
#define JC_PROJECT_MASS   1u
#define JC_PROJECT_ENERGY 2u

typedef struct jc_model jc_model;

/* config.json as read by crates/engine/src/config.rs:43-67. mask_kind 0 =
 * Full, 1 = Stencil{mask_radius, mask_dilation}. */
typedef struct {
    int32_t nx, ny, patch, channels, dim, layers, heads;
    int32_t head_dim, ff_inner, meta_dim;
    int32_t mask_kind, mask_radius, mask_dilation;
    float norm_mean[3], norm_std[3], norm_depth;
    float dx, dt, g, depth, nu, energy_r_max;
} jc_config;

/* Replaces engine::Model::from_bytes + Model::to_gpu (crates/engine/src/lib.rs:45-50,
 * 64-67; gpu.rs:212-218): parse a model.safetensors image and config.json text,
 * upload the weights in the requested precision. */
jc_status jc_model_create(const uint8_t* safetensors, size_t safetensors_len,
                          const char* config_json, int32_t precision,
                          jc_model** out);

/* ---- Pre-packed checkpoints ----
 * No reference counterpart: the reference converts model.safetensors on every
 * load (weights.rs:29-48, gpu.rs:212-283). A pre-packed checkpoint is the
 * model's device weight image (every array in the layouts the kernels read,
 * for the model's precision) with its config and the identity of its source,
 * cached beside model.safetensors; the source format is unchanged.
 *
 * jc_model_pack writes it into `buf` (cap bytes) and sets *len; with buf null
 * it only sets *len. */
jc_status jc_model_pack(const jc_model* m, uint8_t* buf, size_t cap, size_t* len);

/* Creates a model from a pre-packed checkpoint: one device allocation and one
 * host->device copy of the weights, no conversion. Malformed or truncated
 * images give JC_BAD_CHECKPOINT before any device work. */
jc_status jc_model_create_packed(const uint8_t* packed, size_t len, jc_model** out);

/* The source identity a pre-packed checkpoint records (fnv1a-64 over the
 * safetensors bytes, then the config text), and the one it holds: a cache
 * is current when the two agree. Host only. */
jc_status jc_source_hash(const uint8_t* safetensors, size_t safetensors_len, const char* config_json,
                         uint64_t* out);
jc_status jc_packed_source_hash(const uint8_t* packed, size_t len, uint64_t* out);

/* Replaces dropping a GpuModel (gpu.rs:199-209). Null is accepted. */
void jc_model_destroy(jc_model* m);

/* Replaces engine::Model::cfg / GpuModel::cfg (lib.rs:30-33, gpu.rs:426-428). */
jc_status jc_model_config(const jc_model* m, jc_config* out);

/* Replaces engine::meta_of(&cfg.params()) (solver_meta.rs:9-11): the
 * [ln dx, ln dt, ln g, ln depth, ln(nu + 1e-6)] conditioning vector. */
jc_status jc_meta_of(const jc_model* m, float* meta_out);

/* Replaces Model::forward / GpuModel::forward (lib.rs:53-55, gpu.rs:374-424):
 * host state [channels, ny, nx] and meta [meta_dim] in, the predicted
 * increment out (same shape as the state). Blocks until done. */
jc_status jc_forward(jc_model* m, const float* state, const float* meta, float* increment);

/* Replaces Model::step / GpuModel::step (lib.rs:58-60, gpu.rs:431-437):
 * next = state + forward(state, meta). */
jc_status jc_step(jc_model* m, const float* state, const float* meta, float* next_state);

/* Replaces the tick loops of crates/engine-cli/src/main.rs:117-121 and
 * eval.rs:144-157 (and, on a reverse checkpoint, the web demo's rewind,
 * crates/web/src/lib.rs:383-409): `ticks` steps from x0, each followed by the
 * projections `flags` selects, done on the device with f64 compensated sums
 * (mass target = box mean of x0's channel 0; energy bound = previous tick's
 * energy times energy_r_max). Writes the final state to `final_state`; when
 * `trajectory` is non-null it receives ticks+1 states (x0 first); when
 * `energies` is non-null it receives ticks+1 energies (f64). */
jc_status jc_rollout(jc_model* m, const float* x0, const float* meta, int32_t ticks,
                     uint32_t flags, float* final_state, float* trajectory,
                     double* energies);

/* Device-resident forms of jc_forward / jc_rollout for callers that keep
 * state in device memory: all pointers are device pointers, `stream` is a
 * cudaStream_t (null = the model's own stream). They enqueue and return. */
jc_status jc_forward_device(jc_model* m, const float* d_state, const float* d_meta,
                            float* d_increment, void* stream);
jc_status jc_rollout_device(jc_model* m, const float* d_x0, const float* d_meta,
                            int32_t ticks, uint32_t flags, float* d_final,
                            double* d_energies, void* stream);

/* ---- Batched rollouts ----
 * The reference runs one state per call (batch size 1, crates/engine/src/lib.rs:1-4);
 * this runs many rollouts together, as the batched loops of
 * crates/engine-cli/src/eval.rs:126-176 would if their trajectories were
 * stepped side by side. A batch is created over a list of models that share
 * every hyper-parameter, mask, normalizer, g and energy_r_max (a checkpoint
 * family: one model per grid size, or a forward and a reverse checkpoint).
 * Instances whose models share every tensor but `pos` run in the same
 * launches; each model group gets its own launches. */
typedef struct jc_batch jc_batch;

typedef struct {
    int32_t model;        /* index into the batch's model list (reconstruct: the forward checkpoint) */
    int32_t ticks;        /* rollout length / reconstruct horizon H, >= 0 */
    uint32_t flags;       /* JC_PROJECT_* for this instance (rollouts) */
    int32_t task;         /* 0 = rollout (forward, or rewind on a reverse checkpoint), 2 = reconstruct */
    const float* x0;      /* rollout: initial state [channels, ny, nx]; reconstruct: values [H+1, 3, ny, nx] */
    const float* meta;    /* [meta_dim] */
    float* final_state;   /* rollout: state after `ticks` ticks; reconstruct: volume [H+1, 3, ny, nx] */
    double* energy;       /* optional [2]: rollout: final energy, max relative energy violation;
                             reconstruct: sweeps run, last max |change| */
    const uint8_t* known; /* reconstruct: [H+1, ny, nx], 1 = known cell */
    int32_t reverse_model;/* reconstruct: index of the reverse checkpoint (same grid) */
    int32_t max_sweeps;   /* reconstruct: sweep limit, >= 1 */
    float tol;            /* reconstruct: stop when the largest change is below tol */
    int32_t reserved;     /* must be 0 */
} jc_instance;

/* max_instances / max_cells bound one jc_batch_rollout call; the workspace is
 * allocated here, once. */
jc_status jc_batch_create(jc_model* const* models, int32_t n_models, int32_t max_instances,
                          int64_t max_cells, jc_batch** out);
void jc_batch_destroy(jc_batch* b);

/* Runs every instance to its own horizon; blocks until the results are
 * written. Rollouts run their ticks; reconstruct instances then run Jacobi
 * sweeps (the rule of JC_TASK_RECONSTRUCT below) inside one CUDA-graph
 * conditional while loop that ends on the device when every reconstruct
 * instance has converged or reached its sweep limit; the whole call is one
 * graph launch, cached by the batch's shape. device_pointers = 0:
 * x0/meta/final_state/known are host memory (copied in and out inside the
 * call); 1: they are device memory. `stream` is a cudaStream_t (null = the
 * batch's own stream). */
jc_status jc_batch_rollout(jc_batch* b, const jc_instance* instances, int32_t n,
                           int32_t device_pointers, void* stream);

/* ---- Serving ----
 * A request loop with continuous batching: requests of different grid sizes
 * and tasks that arrive while others run are admitted as the workspace and
 * the device memory budget allow, and share the same launches; their states
 * stay on the device until they finish. The loop runs chunks of ticks with
 * no host round trip inside a chunk; a chunk ends when a waiting request
 * could be admitted, or after a few milliseconds of device time when none
 * waits. Results do not depend on the other requests in the mix or on how
 * a request's ticks fall into chunks. Tasks:
 *   FORWARD:     ticks steps of the forward model from x = X_0, projected
 *                (the eval.rs:144-157 loop);
 *   REWIND:      ticks steps of the reverse model from x = X_H, projected
 *                (the web demo's rewind, crates/web/src/lib.rs:383-409);
 *   RECONSTRUCT: x = values [ticks+1, 3, ny, nx], known = mask [ticks+1, ny, nx]
 *                (1 = known cell, all channels); Jacobi sweeps
 *                X_t <- known ? value : mean(step_F(X_{t-1}), step_R(X_{t+1}))
 *                from X = 0 at unknown cells, until the largest change is
 *                below tol or max_sweeps ran; no projection. No counterpart
 *                in the reference. The result is the volume [ticks+1, 3, ny, nx]. */
typedef struct jc_server jc_server;

enum { JC_TASK_FORWARD = 0, JC_TASK_REWIND = 1, JC_TASK_RECONSTRUCT = 2 };

/* Request flag: x, known and meta are caller-owned buffers that stay valid
 * until the request is done, and so is jc_server_wait's `out`: device memory,
 * or page-locked host memory (cudaMallocHost / cudaHostRegister), which the
 * copies then read or write by DMA. Without it, inputs and results are host
 * memory of any kind: jc_server_submit copies the inputs into the server's
 * page-locked staging buffers, and the result comes back through them. Either
 * way a finished request's result stays in the server's device memory (counted
 * against its budget) until jc_server_wait copies it out, so requests that are
 * never collected keep their memory. */
#define JC_REQUEST_DEVICE_BUFFERS 0x100u

typedef struct {
    int32_t task;         /* JC_TASK_* */
    int32_t grid;         /* index into the server's model lists */
    int32_t ticks;        /* horizon H >= 1 */
    uint32_t flags;       /* JC_PROJECT_* (forward and rewind), JC_REQUEST_DEVICE_BUFFERS */
    const float* x;       /* see above; host memory is copied by jc_server_submit */
    const uint8_t* known; /* reconstruct only */
    const float* meta;    /* [meta_dim] */
    int32_t max_sweeps;   /* reconstruct */
    float tol;            /* reconstruct: stop when max |change| < tol */
} jc_request;

typedef struct {
    double latency_s;     /* submit to result */
    double queue_s;       /* submit to admission */
    int32_t sweeps;       /* reconstruct sweeps run */
    float residual;       /* reconstruct: last max |change| */
    double energy;        /* forward / rewind: final energy */
    double max_violation; /* forward / rewind: max relative energy violation */
    int64_t out_len;      /* floats written to `out` */
} jc_result;

typedef struct {
    int64_t completed;
    double cell_ticks;    /* sum of nx * ny * ticks of completed requests */
    double busy_s;        /* time the loop spent in iterations */
    double span_s;        /* first submit to last completion (host clock) */
    int32_t iterations, active, pending;
    double device_span_s; /* device time (CUDA events on the server's stream) from the start
                             of the first iteration to the end of the latest one */
    int64_t launches;     /* kernel launches the loop made (forward, projection, reconstruct) */
} jc_server_stats;

/* forward_models[i] and reverse_models[i] (reverse may be null: forward only)
 * hold grid i; every model of one direction shares all tensors but `pos`.
 * max_active_cells bounds the cells stepped per tick (the workspace is
 * allocated for it here); hbm_fraction caps the device memory in use
 * (requests wait in the queue while admitting them would exceed it). */
jc_status jc_server_create(jc_model* const* forward_models, jc_model* const* reverse_models,
                           int32_t n_grids, int64_t max_active_cells, double hbm_fraction,
                           jc_server** out);
/* Stops the loop after the current tick; pending and active requests are dropped. */
void jc_server_destroy(jc_server* s);
/* Copies the request's inputs and queues it; returns at once with its id. */
jc_status jc_server_submit(jc_server* s, const jc_request* r, uint64_t* id);
/* Blocks until request `id` is done (timeout_s < 0: no limit), writes its
 * result to out (out_len floats available) and its statistics to info
 * (either may be null), and forgets the request. */
jc_status jc_server_wait(jc_server* s, uint64_t id, float* out, size_t out_len, jc_result* info,
                         double timeout_s);
jc_status jc_server_get_stats(jc_server* s, jc_server_stats* out);
/* Zeroes the statistics; the next iteration starts a new device span. */
jc_status jc_server_reset_stats(jc_server* s);
/* Instrumentation, with no counterpart in the reference: enable = 1 clears
 * and starts per-kernel timing (CUDA events around every kernel launch of the
 * loop, which adds a little host work per launch); enable = 0 stops it and,
 * when report is non-null, writes one "name,launches,total_ms" line per
 * kernel over the iterations in between (NUL-terminated, truncated to cap
 * bytes). */
jc_status jc_server_profile(jc_server* s, int32_t enable, char* report, size_t cap);

/* Instrumentation, with no counterpart in the reference: runs the instances
 * once, outside any graph, with CUDA events around every kernel launch, and
 * writes one "name,launches,total_ms" line per kernel into `report`
 * (NUL-terminated, truncated to `cap` bytes). Final states are not copied
 * out. */
jc_status jc_batch_profile(jc_batch* b, const jc_instance* instances, int32_t n,
                           int32_t device_pointers, char* report, size_t cap);

/* The forward pass of jc_forward_device for callers that cannot allocate
 * device memory when they run the model: a host application whose own pool
 * allocator has reserved the whole device up front (an extra cudaMalloc then
 * fails or fragments that pool), or a plugin that is handed device buffers
 * by its host and must not grow the process's footprint behind its back.
 * This entry point has no counterpart in the reference. It allocates
 * nothing: every intermediate buffer lives in one fixed 12 MiB device array
 * inside the library, which every GPU that loads the library holds until the
 * process exits. It always runs the FP32 kernels (f32 weights and
 * activations), for a model created with either precision. Grids whose
 * buffers exceed 12 MiB are refused with JC_LIMIT (the dim 128, 4-layer
 * model fits grids up to 128 x 128 cells). All calls share that array:
 * calls that overlap on the GPU (on different streams, or from different
 * threads) race and corrupt each other's results; serialise them. The first
 * call on each device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it; make that first call before any
 * stream capture begins. cudaDeviceReset discards the array with the
 * context: do not use the library's handles across a reset. Pointers are
 * device pointers; `stream` is a cudaStream_t (null = the legacy default
 * stream); the call enqueues and returns. */
jc_status jc_forward_device_noalloc(jc_model* m, const float* d_state, const float* d_meta,
                                    float* d_increment, void* stream);

/* Host-side projections, engine::project (crates/engine/src/project.rs:22-54),
 * with f64 compensated sums. n = cells per channel; x is [3, n]. */
double jc_mass(const float* x, int64_t n);
double jc_energy(const float* x, const jc_config* cfg, int64_t n);
void   jc_project_mass(float* x, double target, int64_t n);
void   jc_project_energy(float* x, double prev_energy, const jc_config* cfg, int64_t n);

/* Autotuning of the BF16 schedules (no counterpart in the reference, whose
 * GPU backend has one fixed workgroup shape per kernel). With enable = 1 (the
 * default; environment JC_AUTOTUNE=0 starts with it off) the first BF16
 * launch outside a stream capture for each row-count bucket (powers of two of
 * token rows) times the candidate schedules with CUDA events, once, and later
 * launches and graph captures use the fastest, where a candidate replaces
 * the fixed schedule only when it is at least 5% faster: the fused MLP's hidden chunk
 * width (32 or 64 columns per step) and the attention's form (shared-memory
 * tiles, or one thread per (row, head) in 64-, 128- or 256-thread CTAs).
 * enable = 0 selects the fixed schedule (64 columns; attention tiles where
 * the mask is radius 1, dilation 1, else 256 threads); enable < 0 only
 * queries.
 * Returns the setting before the call. If JC_AUTOTUNE_CACHE names a file,
 * tuned schedules (with the candidates' times) are appended to it as JSON
 * lines and read back by models created later. Results are identical under
 * every schedule: the candidates differ in tiling and staging, not in the
 * arithmetic or the order of any sum, so an instance's result does not depend
 * on the batch it runs in. */
int32_t jc_autotune(int32_t enable);

/* ---- Evaluation on the device ----------------------------------------------
 * The `eval-metrics` loop (crates/engine-cli/src/eval.rs:126-176) with its
 * reference solver and scores on the GPU: solvers::ShallowWater
 * (crates/solvers/src/shallow_water.rs), engine::metrics
 * (crates/engine/src/metrics.rs) and the model's rollout, side by side. */

/* solvers::Params (crates/solvers/src/shallow_water.rs:16-29). */
typedef struct {
    int32_t nx, ny;
    float dx, dt, g, depth, nu;
} jc_sw_params;

/* `steps` ShallowWater::step calls (shallow_water.rs:149-238) on each of
 * `count` independent solver states, in place. states: [count][3][ny][nx], the
 * planes h (total depth), u, v in physical units. The arithmetic is the
 * reference's f32 arithmetic, operation for operation, so the results are
 * bit-identical to it. jc_sw_run takes host buffers and blocks;
 * jc_sw_run_device takes a device buffer, enqueues on `stream` (a
 * cudaStream_t, null = legacy default stream) and returns. */
jc_status jc_sw_run(const jc_sw_params* p, float* states, int32_t count, int32_t steps);
jc_status jc_sw_run_device(const jc_sw_params* p, float* d_states, int32_t count, int32_t steps,
                           void* stream);

/* State::add_drop (shallow_water.rs:102-111) on one host h plane [ny][nx]:
 * h += amp exp(-((x - cx)^2 + (y - cy)^2) / (2 sigma^2)), with the C
 * library's expf as the reference's f32::exp. */
jc_status jc_sw_add_drop(const jc_sw_params* p, float* h, float cx, float cy, float amp, float sigma);

/* One solver trajectory of dump-dataset (crates/engine-cli/src/dump_dataset.rs:
 * 157-190): from its initial state, `ticks` ShallowWater::step calls, and after
 * step t the fields of the drops landing at tick t added to h (the pending
 * drops of apply_pending, :90-99). frames receives ticks + 1 states in the
 * file layout of traj-NNNNN.f32: all h frames, then all u, then all v, each
 * channel tick-major ([3][ticks + 1][ny][nx]). Host buffers. */
typedef struct {
    int32_t ticks;              /* >= 0 */
    const float* x0;            /* initial state [3][ny][nx] (h, u, v) */
    int32_t n_drops;            /* pending drops, >= 0 */
    const int32_t* drop_ticks;  /* [n_drops], each in [1, ticks] */
    const float* drop_fields;   /* [n_drops][ny][nx]: amp exp(-r^2 / (2 sigma^2)) as State::add_drop forms
                                   it (jc_sw_add_drop on a zero plane gives it) */
    float* frames;              /* [3][ticks + 1][ny][nx] */
} jc_sw_trajectory;

/* All trajectories advance together on the device (one solver launch per
 * tick); the frames equal the reference's bit for bit. */
jc_status jc_sw_trajectories(const jc_sw_params* p, const jc_sw_trajectory* t, int32_t n);

/* One Gaussian drop: centre in cell coordinates, amplitude, radius in cells. */
typedef struct {
    float cx, cy, amp, sigma;
} jc_drop;

/* One eval-metrics row (eval.rs:101-108, 158-171): Pearson correlation over
 * (h, u, v) and over h, amplitude ratio (model peak |h| over solver peak
 * |h|), wavefront lag in cells (cross-correlation of the radial |h|
 * profiles, sub-cell refined) and bias ((mean model h - mean solver h) / std
 * solver h). */
typedef struct {
    float corr, corr_h, amplitude_ratio, lag, bias;
} jc_eval_row;

/* Scores `count` normalized model states x [count][3][ny][nx] against solver
 * states truth [count][3][ny][nx] (physical h, u, v), each about its drop
 * centre centres[2 k], centres[2 k + 1]. cfg supplies nx, ny and the
 * normalizer. Host buffers. Peaks, amplitude ratios, radial profiles and
 * the f32 means and standard deviation of the bias follow metrics.rs's
 * summation order exactly; the f64 correlation sums are tree-ordered, which
 * can move a correlation by one f32 rounding step. */
jc_status jc_eval_score(const jc_config* cfg, const float* x, const float* truth, const float* centres,
                        int32_t count, jc_eval_row* rows);

/* An evaluator for one model: device buffers for up to max_trajectories
 * trajectories and a batch runner for the model's rollouts. */
typedef struct jc_eval jc_eval;
jc_status jc_eval_create(jc_model* m, int32_t max_trajectories, jc_eval** out);
void jc_eval_destroy(jc_eval* e);

/* eval-metrics for the given drops. Trajectory k starts from State::flat
 * (h = depth, u = v = 0) plus drops[k]; the reference solver and the model
 * (step, then the projections in `flags`, per tick) advance side by side in
 * one captured graph, and at each horizon every trajectory is scored as in
 * jc_eval_score. horizons: strictly ascending, >= 1. rows: [n_horizons][n].
 * max_violation (optional): the largest relative energy violation
 * max((E_t - E_{t-1} r_max) / E_{t-1}, 0) over all trajectories and ticks.
 * The drops are the caller's: the reference's trajectory sampler and its
 * horizon filter (eval.rs:126-134) live on the caller's side. */
jc_status jc_eval_run(jc_eval* e, const jc_drop* drops, int32_t n, const int32_t* horizons,
                      int32_t n_horizons, uint32_t flags, jc_eval_row* rows, double* max_violation);

/* ---- Rewind round trip ------------------------------------------------------
 * Forward N ticks with a forward checkpoint, then N ticks with its reverse
 * checkpoint (same grid and hyper-parameters), scored against the start
 * state: the round-trip runs of the reference
 * (docs/runs/2026-09-20-rewind-round-trip.md:17-32), which drive
 * engine::Model::step with both checkpoints (crates/web/src/lib.rs:383-409 is
 * the interactive rewind). All trajectories and horizons run as batches on
 * the device. */
typedef struct jc_roundtrip jc_roundtrip;

/* One round-trip row: Pearson correlation over (h, u, v) of the rewound and
 * the start state (metrics.rs:9-23), amplitude ratio (peak |h| of the rewound
 * over the start state, decoded as metrics.rs:105-107), RMSE of the rewound
 * against the start state and RMSE of the N-tick state against the start
 * state (metrics.rs:109-112, normalized units; the latter is what a rewind
 * that changes nothing would score). */
typedef struct {
    float corr, amplitude_ratio, rmse, change_rmse;
} jc_roundtrip_row;

jc_status jc_roundtrip_create(jc_model* forward, jc_model* reverse, int32_t max_trajectories,
                              int32_t max_horizons, jc_roundtrip** out);
void jc_roundtrip_destroy(jc_roundtrip* r);

/* Trajectory k starts from State::flat plus drops[k] (encoded); horizons are
 * strictly ascending and >= 1; `flags` (JC_PROJECT_*) apply to both
 * directions, the projections' references taken at the start of each
 * direction. rows: [n_horizons][n]. */
jc_status jc_roundtrip_run(jc_roundtrip* r, const jc_drop* drops, int32_t n, const int32_t* horizons,
                           int32_t n_horizons, uint32_t flags, jc_roundtrip_row* rows);

/* Self-test of the bounded device-side waits, with no counterpart in the
 * reference (whose error surface for a stalled device is
 * lean_runtime::Error::Poll, crates/lean-runtime/src/error.rs:6-13). Every
 * spin-wait in this library's kernels gives up after a time limit, sets an
 * error flag and returns, and the call that launched it reports
 * JC_DEVICE_TIMEOUT. This runs the same mbarrier wait in a one-CTA kernel
 * with a limit of limit_us microseconds (1 .. 2,000,000): with satisfy = 0
 * nothing ever arrives on the barrier, the wait runs out and the call
 * returns JC_DEVICE_TIMEOUT with the kernel finished and the context usable;
 * with satisfy = 1 the barrier completes and the call returns JC_OK. */
jc_status jc_selftest_device_wait(int32_t satisfy, uint32_t limit_us);

/* Thread-local description of the last failure on this thread ("" if none). */
const char* jc_last_error(void);

/* Library version string. */
const char* jc_version(void);

#ifdef __cplusplus
}
#endif
#endif
