// Tensor-core (tcgen05) BF16 forward path: bf16 weights and activations on
// the tensor cores with f32 accumulation in tensor memory; LayerNorm
// statistics, softmax, the residual stream and the projection stay f32/f64.
#pragma once

#include <cuda_bf16.h>

#include "runtime.hpp"

namespace jc {

class BF16Path {
   public:
    BF16Path(const Dims& d, const TensorMap& t, DeviceArena& arena);
    // Allocates this path's token- and cell-level buffers into p.bt / p.bc
    // and its per-instance tensor-map array into p.tmaps.
    void alloc_workspace(DeviceArena& a, const Dims& d, Pack& p, int rows, long long cells, int max_inst) const;
    // Encodes and uploads the per-instance tensor maps of a pack view whose
    // host-side descriptors are `hinst` (same order as the device array).
    void prepare(const Dims& d, const Pack& p, const InstDev* hinst, cudaStream_t s) const;
    void forward(const Dims& d, const WeightsF32& w32, const Pack& p, int mode, cudaStream_t s) const;

    // Weights in the tensor-core operand layout ([block][K/8][rows][8] bf16).
    const __nv_bfloat16 *wqkv[kMaxLayers], *wp[kMaxLayers], *w1[kMaxLayers], *w2[kMaxLayers];
    const __nv_bfloat16 *wtm, *wtc, *wc1;
    int nc_mlp;  // MLP chunk width (columns of ff1 per step)
    int bn_qkv;  // N block of the q/k/v GEMM
    int bn_tm;   // N block of the token_mix convolution
};

}  // namespace jc
