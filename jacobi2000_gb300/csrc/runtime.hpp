// Host runtime of the engine: checkpoint parsing, device weights, launch
// packs and the rollout loop.
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

// A device allocation owned by a Model.
struct DeviceArena {
    std::vector<void*> ptrs;
    void* alloc(size_t bytes);
    template <class T>
    T* alloc_n(size_t n) { return static_cast<T*>(alloc(n * sizeof(T))); }
    float* upload(const std::vector<float>& v);
    ~DeviceArena();
};

class BF16Path;  // tensor-core forward (bf16_path.cu)

class Model {
   public:
    Model(const uint8_t* st, size_t st_len, const char* config_json, int precision);
    ~Model();

    jc_config cfg{};
    Dims dims{};
    int precision = JC_FP32;
    cudaStream_t stream = nullptr;

    void meta_of(float* out) const;
    void forward_host(const float* state, const float* meta, float* inc);
    void step_host(const float* state, const float* meta, float* next);
    void rollout_host(const float* x0, const float* meta, int ticks, uint32_t flags, float* final_state,
                      float* traj, double* energies);
    void forward_device(const float* d_state, const float* d_meta, float* d_inc, cudaStream_t s);
    void rollout_device(const float* d_x0, const float* d_meta, int ticks, uint32_t flags, float* d_final,
                        double* d_energies, cudaStream_t s);

    // Forward of every instance of a pack with this model's weights.
    void forward_pack(const Pack& p, int mode, cudaStream_t s);

    // Device weights.
    DeviceArena arena;
    WeightsF32 wf32{};
    const float* d_pos = nullptr;  // [T, D]
    std::unique_ptr<BF16Path> bf16;

    // Single-instance pack over this model's own grid.
    Pack pack{};
    InstDev host_inst{};
    float *d_state = nullptr, *d_inc = nullptr, *d_meta = nullptr;
    double* d_energies = nullptr;
    int energies_cap = 0;
    float* h_pinned = nullptr;  // staging for host calls: state | meta | out
    size_t state_len = 0;

   private:
    void alloc_pack_workspace(Pack& p);
    void set_single_instance(float* state, float* out, const float* meta);
    void enqueue_rollout(int ticks, uint32_t flags, double* d_energies_out, float* d_traj, cudaStream_t s);
    // cached rollout graphs: key = (ticks, flags, energies?, traj?)
    struct GraphKey {
        int ticks; uint32_t flags; const void* e; const void* t; cudaStream_t s;
        bool operator<(const GraphKey& o) const {
            if (ticks != o.ticks) return ticks < o.ticks;
            if (flags != o.flags) return flags < o.flags;
            if (e != o.e) return e < o.e;
            if (t != o.t) return t < o.t;
            return s < o.s;
        }
    };
    std::map<GraphKey, cudaGraphExec_t> graphs_;
};

}  // namespace jc
