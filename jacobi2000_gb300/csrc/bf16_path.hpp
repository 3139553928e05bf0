// Tensor-core (tcgen05) BF16 forward path: bf16 weights and activations on
// the tensor cores with f32 accumulation in tensor memory; LayerNorm
// statistics, softmax, the residual stream and the projection stay f32/f64.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include <atomic>
#include <map>
#include <mutex>

#include "runtime.hpp"

namespace jc {

// A schedule the autotuner picks per (row-count bucket): the MLP's hidden
// chunk width and the attention kernel's form. Every schedule gives the same
// bits: the candidates change tiling, never the order of a sum, so an
// instance's result does not depend on the batch it runs in.
struct Tuning {
    int nc;            // 32 or 64 hidden columns per MLP step
    int attn_threads;  // 64, 128 or 256 threads per attention CTA; 0 = shared-memory tiles
};

// 1 (default; environment JC_AUTOTUNE=0 turns it off): BF16 launches time the
// candidate schedules once per row-count bucket and keep the fastest; 0: the
// fixed default schedule {MLP with 64 hidden columns per step; shared-memory
// attention tiles where they apply, else 256 attention threads}.
extern std::atomic<int> g_autotune;

class BF16Path {
   public:
    // With `t`, converts and uploads the weights through `arena`; without,
    // leaves the weight pointers for the caller to set (pre-packed load).
    BF16Path(const Dims& d, const TensorMap* t, DeviceArena* arena);
    // Addresses of every weight pointer, in a fixed order.
    void weight_slots(std::vector<const void**>& out) const;
    // Allocates this path's token- and cell-level buffers into p.bt / p.bc
    // and its per-instance tensor-map array into p.tmaps.
    void alloc_workspace(DeviceArena& a, const Dims& d, Pack& p, int rows, long long cells, int max_inst) const;
    // Encodes and uploads the per-instance tensor maps of a pack view whose
    // host-side descriptors are `hinst` (same order as the device array).
    // With `hstage` (page-locked, room for the view's maps, not reused until
    // the copy has run) the maps are encoded there and copied asynchronously;
    // without, through a temporary host array and a stream synchronisation.
    void prepare(const Dims& d, const Pack& p, const InstDev* hinst, cudaStream_t s,
                 CUtensorMap* hstage = nullptr) const;
    void forward(const Dims& d, const WeightsF32& w32, const Pack& p, int mode, cudaStream_t s) const;
    // Picks the schedule for p's row count (timing the candidates on p's own
    // workspace) unless it is known or autotuning is off. Never call while
    // `s` is capturing a graph.
    void tune(const Dims& d, const WeightsF32& w32, const Pack& p, cudaStream_t s) const;
    Tuning tuning_for(int rows) const;

    // Weights in the tensor-core operand layout ([block][K/8][rows][8] bf16).
    const __nv_bfloat16 *wqkv[kMaxLayers], *wp[kMaxLayers];
    // the MLP weights arranged for each chunk width: [0] nc 64, [1] nc 128
    const __nv_bfloat16 *w1v[2][kMaxLayers], *w2v[2][kMaxLayers];  // chunk widths 32 | 64
    int n_nc = 1;
    const __nv_bfloat16 *wtm, *wtc, *wc1, *wc2;
    int bn_qkv;  // N block of the q/k/v GEMM
    int bn_tm;   // N block of the token_mix convolution

   private:
    static constexpr size_t kMlpSmemMax = 200 * 1024;
    int dims_D_ = 0, dims_F_ = 0;
    Dims dims_{};
    Tuning def_tuning_{64, 256};
    int n_sms_ = 1;
    bool mlp_fits(int nc) const;
    // The fused MLP of layer l; with m_attn (attention rows) the layer's output
    // projection + LayerNorm2 runs first in the same kernel (proj_fuses).
    void launch_mlp(const Dims& d, const WeightsF32& w, int l, const Tuning& tu, const CUtensorMap& m_ln, const Pack& p,
                    cudaStream_t s, const CUtensorMap* m_attn = nullptr) const;
    bool proj_fuses(const Tuning& tu) const;
    mutable std::mutex tune_mu_;
    mutable std::map<int, Tuning> tuned_;  // row-count bucket -> schedule
    std::string cache_key_;
    void load_cache();
    void upload_weights(const Dims& d, const TensorMap& t, DeviceArena& arena);
    void set_kernel_attributes();
    void save_cache(int bucket, const Tuning& t, const std::string& timings) const;
};

}  // namespace jc
