// Host runtime of the engine: checkpoint parsing, device weights, launch
// workspaces, the rollout loop and the batch runner.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/jacobi2000.h"
#include "engine.hpp"

namespace jc {

// An error carrying the C-ABI status it maps to.
struct Error : std::runtime_error {
    jc_status code;
    Error(jc_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char* what, jc_status code = JC_CUDA_ERROR);

struct HostTensor {
    std::vector<int64_t> shape;
    std::vector<float> data;
    size_t numel() const { return data.size(); }
};
using TensorMap = std::map<std::string, HostTensor>;

// crates/engine/src/weights.rs:29-48 with the panics replaced by
// JC_BAD_CHECKPOINT errors (bounds and dtype are checked).
TensorMap parse_safetensors(const uint8_t* p, size_t n);

// crates/engine/src/config.rs:70-100 into a jc_config; validates shapes
// (grid divisible by the patch, every tensor present with its expected shape).
jc_config parse_config(const char* json, const TensorMap& t);

// Device allocations owned by one object, freed with it.
//
// Weight image: between begin_image() and end_image(), upload() and
// upload_bytes() append the arrays to one host image (256-byte aligned) and
// return provisional addresses; end_image() makes one device allocation and
// one host->device copy of the whole image and rebases the given pointer
// slots (every array uploaded in between must have exactly one slot).
struct DeviceArena {
    std::vector<void*> ptrs;
    void* alloc(size_t bytes);
    template <class T>
    T* alloc_n(size_t n) { return static_cast<T*>(alloc(n * sizeof(T))); }
    float* upload(const std::vector<float>& v);
    const void* upload_bytes(const void* src, size_t bytes);
    void release(void* p);
    ~DeviceArena();

    void begin_image();
    // Returns the slots' offsets into the image.
    std::vector<uint64_t> end_image(const std::vector<const void**>& slots);
    std::vector<uint8_t> image;     // host image while building
    void* image_base = nullptr;     // device image after end_image()
    size_t image_len = 0;

   private:
    bool imaging_ = false;
    size_t image_arrays_ = 0;
};

class BF16Path;  // tensor-core forward (bf16_path.cu)
class Model;

// Launch workspace for packs of up to max_rows token rows, max_cells cells
// and max_inst instances, plus the state/meta slabs of those instances.
struct Workspace {
    int max_rows = 0, max_inst = 0;
    long long max_cells = 0;
    Pack base{};            // pointers at offset 0; packs are views into it
    float* states = nullptr;  // [3 * max_cells]
    float* metas = nullptr;   // [max_inst * 64]
    void alloc(DeviceArena& a, const Dims& d, int rows, long long cells, int inst, const BF16Path* bf);
    // A pack view over rows [row_base, ...), cells [cell_base, ...) and
    // instances [inst_base, inst_base + n), with the given tile counts.
    Pack view(const Dims& d, int inst_base, int n, int row_base, int rows, long long cell_base, long long cells,
              int tiles, int ttiles, int ctiles) const;
    // Throws JC_DEVICE_TIMEOUT (and clears the flag) when a device-side wait
    // gave up since the last check; `s` must be idle.
    void check_timeout(cudaStream_t s) const;
};

// Reads a device-side wait flag (set by a kernel whose bounded wait gave up)
// after the work on `s`; throws JC_DEVICE_TIMEOUT and clears the flag when
// it is set.
void check_wait_flag(int* flag, cudaStream_t s);

// Device-side wait self-test (selftest.cu): one CTA waits on an mbarrier
// with a limit of limit_us microseconds; with satisfy = 0 nothing ever
// arrives, so the wait gives up and the call reports JC_DEVICE_TIMEOUT.
void selftest_device_wait(int satisfy, unsigned limit_us);

// Tile counts of one instance's grids.
int cell_tiles(int nx, int ny);   // 16x16 cells
int conv_tiles(int w, int h);     // 8x16 positions

// Device weights of one checkpoint.
struct DeviceWeights {
    WeightsF32 f32{};
    const float* pos = nullptr;  // [T, D]
    std::unique_ptr<BF16Path> bf16;
    std::unique_ptr<Conv2Params> conv2;  // host copy behind f32.c2p
    uint64_t shared_hash = 0;    // hash of every tensor but `pos`
};

class Model {
   public:
    Model(const uint8_t* st, size_t st_len, const char* config_json, int precision);
    // From a pre-packed image written by pack(): one device allocation and
    // one host->device copy of the weights, no conversion.
    Model(const uint8_t* packed, size_t len);
    ~Model();

    // The pre-packed checkpoint: header (config, precision, source hash,
    // slot offsets, conv2 parameters) followed by the device weight image.
    std::vector<uint8_t> pack() const;
    uint64_t source_hash = 0;  // fnv1a-64 of the safetensors bytes and the config text

    jc_config cfg{};
    Dims dims{};
    int precision = JC_FP32;
    cudaStream_t stream = nullptr;
    DeviceArena arena;
    DeviceWeights w;
    size_t state_len = 0;

    void meta_of(float* out) const;
    void forward_host(const float* state, const float* meta, float* inc);
    void step_host(const float* state, const float* meta, float* next);
    void rollout_host(const float* x0, const float* meta, int ticks, uint32_t flags, float* final_state,
                      float* traj, double* energies);
    void forward_device(const float* d_state, const float* d_meta, float* d_inc, cudaStream_t s);
    void rollout_device(const float* d_x0, const float* d_meta, int ticks, uint32_t flags, float* d_final,
                        double* d_energies, cudaStream_t s);
    // Per-kernel device time of `iters` forwards of this model's grid.
    std::map<std::string, std::pair<int, double>> profile_forward(int iters);

    // Forward of every instance of a pack with this model's weights.
    void forward_pack(const Pack& p, int mode, cudaStream_t s) const;

   private:
    std::vector<uint64_t> slot_off_;  // weight slots' offsets into the device image
    void finish_init();
    Workspace ws_;
    Pack pack_{};
    InstDev inst_{};
    float* d_inc_ = nullptr;
    double* d_energies_ = nullptr;
    int energies_cap_ = 0;
    float* h_pinned_ = nullptr;  // staging for host calls: state | out | meta
    void put_instance(float* state, float* out, const float* meta, uint32_t flags, cudaStream_t s);
    void enqueue_rollout(int ticks, double* d_energies_out, float* d_traj, cudaStream_t s);
    struct GraphKey {
        int ticks;
        const void* e;
        const void* t;
        cudaStream_t s;
        int tune;  // autotuning switch at capture time
        bool operator<(const GraphKey& o) const {
            if (tune != o.tune) return tune < o.tune;
            if (ticks != o.ticks) return ticks < o.ticks;
            if (e != o.e) return e < o.e;
            if (t != o.t) return t < o.t;
            return s < o.s;
        }
    };
    std::map<GraphKey, cudaGraphExec_t> graphs_;
    cudaGraphExec_t graph_for(const GraphKey& k, double* e, float* t);
};

// Work that a batch rollout enqueues after every tick, inside its captured
// graph (the evaluator steps its solver and scores there).
struct TickHook {
    virtual ~TickHook() = default;
    // Before capture or launch: per caller instance index, the device state
    // that the tick loop updates in place. Enqueues any upload on `s`.
    virtual void bind(const std::vector<float*>& states, cudaStream_t s) = 0;
    // After tick t (1-based) of every instance.
    virtual void after_tick(int t, cudaStream_t s) const = 0;
    // Identifies the launches after_tick makes (buffers, shapes), for the
    // graph cache.
    virtual long long key() const = 0;
};

// Many instances of (possibly) different grids, one launch sequence per tick.
// Instances whose models share every tensor but `pos` share launches.
class Batch {
   public:
    Batch(jc_model* const* models, int n_models, int max_inst, long long max_cells);
    ~Batch();
    void rollout(const jc_instance* inst, int n, bool device_ptrs, cudaStream_t s, TickHook* hook = nullptr);
    std::map<std::string, std::pair<int, double>> profile(const jc_instance* inst, int n, bool device_ptrs);

   private:
    std::vector<Model*> models_;
    std::vector<int> group_of_;  // model -> weight group (index of its first model)
    Dims dims_{};
    int precision_ = JC_FP32;
    DeviceArena arena_;
    Workspace ws_;
    cudaStream_t stream_ = nullptr;
    cudaStream_t stream2_ = nullptr;  // captures the body of the reconstruct while loop
    float* recon_f_ = nullptr;        // reconstruct volumes, step results and values
    uint8_t* recon_u8_ = nullptr;     // reconstruct masks
    size_t recon_f_cap_ = 0, recon_u8_cap_ = 0;
    ReconDev* d_recon_ = nullptr;
    int recon_cap_ = 0;
    float* h_states_ = nullptr;  // pinned [3 * max_cells]
    float* h_metas_ = nullptr;   // pinned [max_inst * 64]
    ProjSlot* h_slots_ = nullptr;
    struct Plan {
        std::vector<int> order;     // caller index of each packed instance
        std::vector<InstDev> inst;  // packed descriptors
        struct Group {
            int model, inst_base, n, row_base, cell_base_i;
            long long cell_base, max_cells;
            std::vector<int> ticks;     // per packed instance, descending
            std::vector<int> rows, tiles, ttiles, ctiles;
            std::vector<long long> cells;  // prefix ends
        };
        std::vector<Group> groups;
        std::vector<long long> state_off;  // per packed instance, floats
        int max_ticks = 0;
        // reconstruct instances and their sweep-phase groups
        struct Recon {
            int order;  // caller index
            int H, nx, ny, max_sweeps;
            float tol;
            long long cells;
            size_t off_vol, off_F, off_R, off_vals, off_known;
        };
        std::vector<Recon> recons;
        std::vector<Group> sgroups;
        int n_tick_inst = 0;
        std::vector<std::pair<size_t, size_t>> sub_off;  // sweep sub-instances: (state, out) slab offsets
        size_t recon_floats = 0, recon_bytes = 0;
    };
    Plan plan(const jc_instance* inst, int n) const;
    void bind_recon(Plan& p);
    void enqueue(const Plan& p, cudaStream_t s, bool capture) const;
    void enqueue_sweep(const Plan& p, cudaStream_t s) const;
    void upload_recon(const Plan& p, const jc_instance* in, bool device_ptrs, cudaStream_t s);
    void prepare_maps(const Plan& p, cudaStream_t s) const;
    std::map<std::vector<long long>, cudaGraphExec_t> graphs_;
    const TickHook* hook_ = nullptr;  // set while a hooked rollout is captured
};

// Serving loop (server.cu).
jc_status server_create(jc_model* const* fwd, jc_model* const* rev, int32_t n, int64_t max_cells, double frac,
                        jc_server** out);
void server_destroy(jc_server* s);
uint64_t server_submit(jc_server* s, const jc_request* r);
void server_wait(jc_server* s, uint64_t id, float* out, size_t n, jc_result* info, double timeout);
void server_stats(jc_server* s, jc_server_stats* st);
void server_reset_stats(jc_server* s);
void server_profile(jc_server* s, int enable, char* report, size_t cap);

// fnv1a-64 of a safetensors image and its config text: the source identity a
// pre-packed checkpoint records.
uint64_t source_hash(const uint8_t* st, size_t st_len, const char* config_json);
// Reads the source hash from a pre-packed image's header (no device work).
uint64_t packed_source_hash(const uint8_t* packed, size_t len);

// Evaluation path (evaluate.cu): the reference solver, the scores and the
// evaluator behind jc_sw_*, jc_eval_score and jc_eval_*.
void sw_run_host(const jc_sw_params& p, float* states, int count, int steps);
void sw_run_device(const jc_sw_params& p, float* d_states, int count, int steps, cudaStream_t s);
void sw_add_drop_host(const jc_sw_params& p, float* h, float cx, float cy, float amp, float sigma);
void sw_trajectories_host(const jc_sw_params& p, const jc_sw_trajectory* t, int n);
void eval_score_host(const jc_config& c, const float* x, const float* truth, const float* centres, int count,
                     jc_eval_row* rows);
jc_eval* eval_create(jc_model* m, int max_traj);
void eval_destroy(jc_eval* e);
void eval_run(jc_eval* e, const jc_drop* drops, int n, const int32_t* horizons, int nh, uint32_t flags,
              jc_eval_row* rows, double* max_violation);

// Rewind round trip (roundtrip.cu), behind jc_roundtrip_*.
jc_roundtrip* roundtrip_create(jc_model* fwd, jc_model* rev, int max_traj, int max_h);
void roundtrip_destroy(jc_roundtrip* r);
void roundtrip_run(jc_roundtrip* r, const jc_drop* drops, int n, const int32_t* horizons, int nh, uint32_t flags,
                   jc_roundtrip_row* rows);

// The FP32 forward of m's own grid with every buffer in the library's fixed
// no-alloc scratch array (noalloc.cu); allocates nothing.
void forward_noalloc(const Model& m, const float* d_state, const float* d_meta, float* d_inc, cudaStream_t s);

}  // namespace jc

struct jc_model {
    jc::Model* m;
};
struct jc_batch {
    jc::Batch* b;
};
