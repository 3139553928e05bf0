// Internal interfaces between the host runtime and the kernel files.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace jc {

constexpr int kMaxLayers = 32;
constexpr int kZcStride = 36;  // channel-last stride of the cell-head input: 32 z + 3 state + 1 zero

// Model hyper-parameters shared by every instance of a launch.
struct Dims {
    int D, L, heads, F, HD, C, P, meta_dim;
    int mask_kind, radius, dilation;
    float norm_mean[3], norm_std[3], norm_depth, g, energy_r_max;
};

// FP32 device weights, in the layouts the FP32 kernels read.
struct WeightsF32 {
    const float *embed_w, *embed_b;   // [C*P*P, D], [D]
    const float *meta_w, *meta_b;     // [meta_dim, D], [D]
    struct Blk {
        const float *n1g, *n1b;       // [D]
        const float *wqkv, *bqkv;     // [D, 3D] (q | k | v along the output), [3D]
        const float *wp, *bp;         // [D, D], [D]
        const float *n2g, *n2b;       // [D]
        const float *w1, *b1;         // [D, F], [F]
        const float *w2, *b2;         // [F, D], [D]
    } blk[kMaxLayers];
    const float *norm_g, *norm_b;     // [D]
    const float *tm_w, *tm_b;         // [9*D, D]: row (tap*D + ci), column co
    const float *tc_w, *tc_b;         // [D, HD]
    const float *c1_w, *c1_b;         // [9*kZcStride, HD]
    const float *c2_w, *c2_b;         // [C, HD, 3, 3] as stored, [C]
};

// A packed launch over several instances, with its workspace.
struct Pack {
    int n_inst;
    int R;            // total token rows
    long long NC;     // total cells
    InstDev* inst;    // device array [n_inst]
    int* row_inst;    // device [R]
    int* cell_inst;   // device [NC]
    ProjSlot* proj;   // device [n_inst]
    // FP32 workspace
    float *x, *qkv, *attn, *ff1, *xn, *t1, *z0, *zc, *c1;
};

enum TickMode { kWriteIncrement = 0, kWriteNextState = 1 };

// FP32 forward of every instance of `p`; writes the increment or the next
// state to each instance's `out`.
void forward_f32(const Dims& d, const WeightsF32& w, const Pack& p, int mode, cudaStream_t s);

// Projection of every instance's `out` state (mass, then energy), f64 sums.
// init = 1 records mass0 and the energy of the state without changing it.
void projection(const Dims& d, const Pack& p, uint32_t flags, int init, cudaStream_t s);

}  // namespace jc
