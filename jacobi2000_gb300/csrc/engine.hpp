// Internal interfaces between the host runtime and the kernel files.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "common.cuh"

namespace jc {

constexpr int kMaxLayers = 32;
constexpr int kMapsPerInst = 7;  // BF16 path: ln halo, zc halo, t1 store, c1 store, qkv halo, q block, c1 halo
constexpr int kZcStride = 36;  // channel-last stride of the cell-head input: 32 z + 3 state + 1 zero

// Model hyper-parameters shared by every instance of a launch.
struct Dims {
    int D, L, heads, F, HD, C, P, meta_dim;
    int mask_kind, radius, dilation;
    float norm_mean[3], norm_std[3], norm_depth, g, energy_r_max;
};

// head.conv2 weights as the conv2 kernel takes them by value (in its
// parameter space): w[(ci * 9 + tap) * 3 + co], bias b[co]; C = 3, HD = 32.
struct Conv2Params {
    float w[32 * 9 * 3];
    float b[3];
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
    const Conv2Params* c2p;           // host copy of c2_w / c2_b in the conv2 kernel's order
};

// A packed launch over the first n_inst instances of `inst`, with the
// workspace it writes. R, NC and n_tiles cover exactly those instances.
struct Pack {
    int n_inst;
    int R;            // token rows
    long long NC;     // cells
    int n_tiles;      // 16x16 cell tiles
    int n_ttiles;     // 8x16 token tiles
    int n_ctiles;     // 8x16 cell tiles
    long long max_inst_cells;  // cells of the largest instance
    InstDev* inst;    // device array, sorted by row0 / cell0 / tile0
    ProjSlot* proj;   // device array parallel to inst
    void* tmaps;      // device array: kMapsPerInst tensor maps per instance (BF16 path)
    int* err;         // device flag set when a device-side wait times out
    // FP32 workspace
    float *x, *qkv, *attn, *ff1, *xn, *t1, *z0, *zc, *c1;
    // BF16-path workspace: token-level buffers (row stride in bytes) and
    // cell-level buffers (cell stride in bytes)
    static constexpr int kTokBufs = 4, kCellBufs = 2;
    char* bt[kTokBufs];
    int bt_stride[kTokBufs];
    char* bc[kCellBufs];
    int bc_stride[kCellBufs];
    long long bc_plane[kCellBufs];  // bytes between the 8-channel planes of a plane-major cell buffer
};

enum TickMode { kWriteIncrement = 0, kWriteNextState = 1 };

// FP32 forward of every instance of `p`; writes the increment or the next
// state to each instance's `out`.
void forward_f32(const Dims& d, const WeightsF32& w, const Pack& p, int mode, cudaStream_t s);

// head.conv2 + the step's residual over f32 c1 [cells, HD], in the reference's
// f32 order (the FP32 path; the BF16 form runs its own tensor-core conv2).
void conv2_step(const Dims& d, const float* c1, const WeightsF32& w, const Pack& p, int mode, const char* name,
                cudaStream_t s);

// Projection of every instance's state (mass, then energy, per the instance's
// flags), f64 sums. init = 1 records mass0 and the energy of the state.
void projection(const Dims& d, const Pack& p, int init, cudaStream_t s);

// One reconstruct instance of a batch: its space-time volume X[0..H], the
// step results F_t = step_F(X_{t-1}) (t = 1..H) and R_t = step_R(X_{t+1})
// (t = 0..H-1), the known values and mask, and its sweep bookkeeping.
struct ReconDev {
    float* vol;            // [H+1][3][cells]
    const float* F;        // [H][3][cells]
    const float* R;        // [H][3][cells]
    const float* vals;     // [H+1][3][cells]
    const uint8_t* known;  // [H+1][cells]
    long long cells;
    int H, max_sweeps;
    float tol;
    int sweeps, frozen;
    unsigned resid_bits;   // max |change| of this sweep, as float bits
    float last_resid;
};

// X <- known ? value : 0 and bookkeeping reset, for n reconstruct instances
// (max_cells / max_h: the largest cell count and horizon among them).
void recon_init(ReconDev* d, int n, long long max_cells, int max_h, cudaStream_t s);
// X_t <- known_t ? value : mean of the available step results, for every
// instance not yet frozen; records each instance's largest change.
void recon_update(ReconDev* d, int n, long long max_cells, int max_h, cudaStream_t s);
// Counts the sweep, freezes converged or exhausted instances and, when
// use_handle, sets the graph's while condition to "some instance still runs".
void recon_finalize(ReconDev* d, int n, unsigned long long handle, int use_handle, cudaStream_t s);

// Optional per-launch timing with CUDA events (profiling only; never active
// during graph capture). Kernels are timed by name on the launching stream.
struct KernelTimer {
    struct Rec {
        const char* name;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    cudaStream_t stream = nullptr;
    const char* open = nullptr;
    cudaEvent_t open_ev = nullptr;
    void begin(const char* name, cudaStream_t s);
    void end();
    // name -> (launches, total ms); synchronizes.
    std::map<std::string, std::pair<int, double>> summary();
    ~KernelTimer();
};
extern thread_local KernelTimer* g_ktimer;
// Kernel launches of the forward, projection and reconstruct paths made by
// the calling thread (every such launch is wrapped in one KScope).
extern thread_local long long g_launches;

struct KScope {
    KScope(const char* name, cudaStream_t s) {
        g_launches++;
        if (g_ktimer) g_ktimer->begin(name, s);
    }
    ~KScope() {
        if (g_ktimer) g_ktimer->end();
    }
};

}  // namespace jc
