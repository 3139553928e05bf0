// FP32 forward path and the tick projection. The kernel sequence restates
// crates/engine/src/cpu.rs:249-352 (forward) and project.rs:22-54
// (projections) on CUDA cores; operation order within a row follows the
// reference (bias first, sequential reductions in key order for the
// attention softmax), so results agree with the reference's f32 CPU path to
// rounding.
#include <algorithm>
#include <atomic>
#include <stdexcept>
#include <string>

#include <cooperative_groups.h>

#include "engine.hpp"
#include "fp32_kernels.cuh"
#include "launch.hpp"

namespace cg = cooperative_groups;

namespace jc {

thread_local KernelTimer* g_ktimer = nullptr;
thread_local long long g_launches = 0;

void KernelTimer::begin(const char* name, cudaStream_t s) {
    stream = s;
    open = name;
    if (pool.empty()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        pool.push_back(e);
    }
    open_ev = pool.back();
    pool.pop_back();
    cudaEventRecord(open_ev, s);
}

void KernelTimer::end() {
    if (!open) return;
    cudaEvent_t e;
    if (pool.empty()) cudaEventCreate(&e);
    else { e = pool.back(); pool.pop_back(); }
    cudaEventRecord(e, stream);
    recs.push_back(Rec{open, open_ev, e});
    open = nullptr;
}

std::map<std::string, std::pair<int, double>> KernelTimer::summary() {
    std::map<std::string, std::pair<int, double>> out;
    for (auto& r : recs) {
        cudaEventSynchronize(r.b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        auto& v = out[r.name];
        v.first += 1;
        v.second += ms;
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    recs.clear();
    return out;
}

KernelTimer::~KernelTimer() {
    for (auto& r : recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
}

static void cuda_check_attr(cudaError_t e) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
}

// Raises a kernel's dynamic shared-memory limit on the current device, once
// per device: the attribute belongs to the device's context, so a process
// that uses several GPUs sets it on each. `done` holds one bit per device.
template <class K>
static void set_smem_per_device(K kernel, int bytes, std::atomic<unsigned long long>& done) {
    int dev = 0;
    cuda_check_attr(cudaGetDevice(&dev));
    const unsigned long long bit = dev >= 0 && dev < 64 ? 1ull << dev : 0ull;
    if (bit && (done.load() & bit)) return;
    cuda_check_attr(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    done.fetch_or(bit);
}

static void check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

namespace f32k {

// Patchify + embed + pos + meta (cpu.rs:253-280). One CTA per 16 rows;
// threads stride over the D outputs. Token t = ty*tx + tx, feature
// c*P*P + py*P + px.
constexpr int kEmbedTok = 16;

__global__ void embed_kernel(Dims d, const float* __restrict__ We, const float* __restrict__ be,
                             const float* __restrict__ Wm, const float* __restrict__ bm, const InstDev* inst,
                             int n_inst, int R, float* __restrict__ x) {
    extern __shared__ float patch[];  // [kEmbedTok][C*P*P]
    __shared__ int rinst[kEmbedTok];
    const int pd = d.C * d.P * d.P;
    const int r0 = blockIdx.x * kEmbedTok;
    if (threadIdx.x < kEmbedTok) rinst[threadIdx.x] = r0 + (int)threadIdx.x < R ? inst_of_row(inst, n_inst, r0 + threadIdx.x) : 0;
    __syncthreads();
    for (int e = threadIdx.x; e < kEmbedTok * pd; e += blockDim.x) {
        int i = e / pd, f = e % pd, r = r0 + i;
        float v = 0.f;
        if (r < R) {
            const InstDev& I = inst[rinst[i]];
            int t = r - I.row0, c = f / (d.P * d.P), py = (f / d.P) % d.P, px = f % d.P;
            int y = (t / I.tx) * d.P + py, xx = (t % I.tx) * d.P + px;
            v = I.state[((size_t)c * I.ny + y) * I.nx + xx];
        }
        patch[e] = v;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kEmbedTok * d.D; e += blockDim.x) {
        int i = e / d.D, o = e % d.D, r = r0 + i;
        if (r >= R) continue;
        const InstDev& I = inst[rinst[i]];
        float acc = be[o];
        const float* p = patch + i * pd;
        for (int f = 0; f < pd; f++) acc = fmaf(p[f], We[(size_t)f * d.D + o], acc);
        float m = bm[o];
        for (int f = 0; f < d.meta_dim; f++) m = fmaf(I.meta[f], Wm[(size_t)f * d.D + o], m);
        x[(size_t)r * d.D + o] = (acc + I.pos[(size_t)(r - I.row0) * d.D + o]) + m;
    }
}

// Stencil-masked multi-head attention (cpu.rs:97-164, mask.rs:18-30). One
// warp per (row, head); lanes over the head's features (head width <= 64). Candidate keys are
// enumerated in increasing key index (the order the reference's scan meets
// them): scores, max, exp(s - max) with the denominator, then
// out = sum (e / denom) v. qkv is [R, 3D] (q | k | v).
__device__ __forceinline__ int n_candidates(const Dims& d, const InstDev& I) {
    if (d.mask_kind == 0) return I.tx * I.ty;
    int s = 2 * d.radius + 1;
    return s * s;
}
// Key row of candidate j of the query at token (qy, qx), or -1 when the
// candidate falls outside the grid.
__device__ __forceinline__ int candidate_row(const Dims& d, const InstDev& I, int qy, int qx, int j) {
    if (d.mask_kind == 0) return I.row0 + j;
    int s = 2 * d.radius + 1;
    int ky = qy + (j / s - d.radius) * d.dilation, kx = qx + (j % s - d.radius) * d.dilation;
    if (ky < 0 || kx < 0 || ky >= I.ty || kx >= I.tx) return -1;
    return I.row0 + ky * I.tx + kx;
}

__global__ void attention_kernel(Dims d, const float* __restrict__ qkv, const InstDev* inst, int n_inst, int R,
                                 float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int wg = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int row = wg / d.heads, head = wg % d.heads;
    if (row >= R) return;
    const int hd = d.D / d.heads, D3 = 3 * d.D;
    const InstDev& I = inst[inst_of_row(inst, n_inst, row)];
    const int t = row - I.row0, qy = t / I.tx, qx = t % I.tx;
    const float scale = 1.0f / sqrtf((float)hd);
    const float* q = qkv + (size_t)row * D3 + head * hd;
    float qv0 = lane < hd ? q[lane] : 0.f;
    float qv1 = lane + 32 < hd ? q[lane + 32] : 0.f;
    const int nc = n_candidates(d, I);

    auto score = [&](int kr) {
        const float* k = qkv + (size_t)kr * D3 + d.D + head * hd;
        float p = (lane < hd ? qv0 * k[lane] : 0.f) + (lane + 32 < hd ? qv1 * k[lane + 32] : 0.f);
        return warp_sum(p) * scale;
    };
    // scores of the first 32 candidates stay in registers (lane j holds
    // candidate j); later candidates are recomputed
    float sreg = -INFINITY;
    float smax = -INFINITY;
    for (int j = 0; j < nc; j++) {
        int kr = candidate_row(d, I, qy, qx, j);
        if (kr < 0) continue;
        float s = score(kr);
        if (j < 32 && lane == j) sreg = s;
        smax = fmaxf(smax, s);
    }
    auto score_j = [&](int j, int kr) {
        return j < 32 ? __shfl_sync(0xffffffffu, sreg, j) : score(kr);
    };
    float denom = 0.f;
    for (int j = 0; j < nc; j++) {
        int kr = candidate_row(d, I, qy, qx, j);
        if (kr >= 0) denom += expf(score_j(j, kr) - smax);
    }
    float o0 = 0.f, o1 = 0.f;
    for (int j = 0; j < nc; j++) {
        int kr = candidate_row(d, I, qy, qx, j);
        if (kr < 0) continue;
        float e = expf(score_j(j, kr) - smax);
        if (e == 0.f) continue;
        float wn = e / denom;
        const float* v = qkv + (size_t)kr * D3 + 2 * d.D + head * hd;
        if (lane < hd) o0 = fmaf(wn, v[lane], o0);
        if (lane + 32 < hd) o1 = fmaf(wn, v[lane + 32], o1);
    }
    float* o = out + (size_t)row * d.D + head * hd;
    if (lane < hd) o[lane] = o0;
    if (lane + 32 < hd) o[lane + 32] = o1;
}

// Row LayerNorm (cpu.rs:49-65), one warp per row.
__global__ void layernorm_kernel(const float* __restrict__ x, const float* __restrict__ g,
                                 const float* __restrict__ b, int R, int D, float* __restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= R) return;
    const float* xr = x + (size_t)row * D;
    float s = 0.f;
    for (int i = lane; i < D; i += 32) s += xr[i];
    float mean = warp_sum(s) / (float)D;
    float v = 0.f;
    for (int i = lane; i < D; i += 32) { float t = xr[i] - mean; v += t * t; }
    float rstd = 1.0f / sqrtf(warp_sum(v) / (float)D + 1e-5f);
    for (int i = lane; i < D; i += 32) y[(size_t)row * D + i] = (xr[i] - mean) * rstd * g[i] + b[i];
}

// Upsample z0 (token level, [rows, HD]) by P along y then x with edge
// replicate and weights (i + 0.5)/P (cpu.rs:211-245), and concatenate the
// state channels (cpu.rs:339-342): zc [cells, kZcStride], one thread per cell.
__global__ void upsample_concat_kernel(Dims d, const float* __restrict__ z0, const InstDev* inst, int n_inst,
                                       long long NC, float* __restrict__ zc) {
    long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= NC) return;
    const InstDev& I = inst[inst_of_cell(inst, n_inst, cell)];
    long long cl = cell - I.cell0;
    int y = (int)(cl / I.nx), x = (int)(cl % I.nx);
    int yt = y / d.P, iy = y % d.P, xt = x / d.P, ix = x % d.P;
    int yt2 = min(yt + 1, I.ty - 1), xt2 = min(xt + 1, I.tx - 1);
    float wy = ((float)iy + 0.5f) / (float)d.P, wx = ((float)ix + 0.5f) / (float)d.P;
    const float4* a = reinterpret_cast<const float4*>(z0 + (size_t)(I.row0 + yt * I.tx + xt) * d.HD);
    const float4* b = reinterpret_cast<const float4*>(z0 + (size_t)(I.row0 + yt * I.tx + xt2) * d.HD);
    const float4* c = reinterpret_cast<const float4*>(z0 + (size_t)(I.row0 + yt2 * I.tx + xt) * d.HD);
    const float4* e = reinterpret_cast<const float4*>(z0 + (size_t)(I.row0 + yt2 * I.tx + xt2) * d.HD);
    float4* o = reinterpret_cast<float4*>(zc + (size_t)cell * kZcStride);
    const float uy = 1.0f - wy, ux = 1.0f - wx;
#pragma unroll 4
    for (int q = 0; q < d.HD / 4; q++) {
        float4 A = a[q], B = b[q], Cc = c[q], E = e[q], r;
        // upsample_y at columns xt and xt2, then upsample_x
        r.x = (A.x * uy + Cc.x * wy) * ux + (B.x * uy + E.x * wy) * wx;
        r.y = (A.y * uy + Cc.y * wy) * ux + (B.y * uy + E.y * wy) * wx;
        r.z = (A.z * uy + Cc.z * wy) * ux + (B.z * uy + E.z * wy) * wx;
        r.w = (A.w * uy + Cc.w * wy) * ux + (B.w * uy + E.w * wy) * wx;
        o[q] = r;
    }
    size_t plane = (size_t)I.nx * I.ny;
    float tail[4] = {0.f, 0.f, 0.f, 0.f};
    for (int ch = 0; ch < d.C; ch++) tail[ch] = I.state[ch * plane + cl];
    o[d.HD / 4] = make_float4(tail[0], tail[1], tail[2], tail[3]);
}

// head.conv2 (3x3, HD -> C, zero padding; cpu.rs:171-205, 347-348) and the
// step's residual (cpu.rs:84-88) over one 16 x 16 cell tile per CTA, for
// C = 3 and HD = 32. The tile's c1 values plus a one-cell halo arrive in four
// stages of 8 channels (32 bytes per position, whole DRAM sectors) by
// asynchronous copies, double-buffered so the next stage is in flight while
// the current one is summed; a stage holds two planes of 4 channels, one
// 16-byte chunk per position, so the halo reads of a thread are fixed offsets
// from one base address. The weights come by value in the kernel's parameter
// space and enter the FMAs as constant operands (no loads). Each of the 128
// threads owns a vertical pair of cells and reuses each halo value across the
// pair. Per cell, the sum runs in the reference's order: bias, then channel,
// ky, kx.
constexpr int kConv2Threads = 128;
constexpr int kConv2S = kCellTile + 2;                // halo tile side
constexpr int kConv2Plane = kConv2S * kConv2S * 4;    // floats per 4-channel plane
constexpr int kConv2Smem = 2 * 2 * kConv2Plane * 4;   // two stages of two planes

template <int C, int HD>
__global__ void __launch_bounds__(kConv2Threads, 8) conv2_step_kernel(const float* __restrict__ c1,
                                                                      const __grid_constant__ Conv2Params cw,
                                                                      const InstDev* inst, int n_inst, int mode) {
    static_assert(C == 3 && HD == 32, "conv2 is built for 3 channels and a cell-head width of 32");
    JC_PDL_ENTRY;
    constexpr int S = kConv2S, NG = HD / 8;
    extern __shared__ __align__(16) float c2smem[];
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (inst[mid].tile0 <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const InstDev I = inst[lo];
    const int tiles_x = (I.nx + kCellTile - 1) / kCellTile;
    const int tl = blockIdx.x - I.tile0;
    const int y0 = (tl / tiles_x) * kCellTile, x0 = (tl % tiles_x) * kCellTile;
    auto load_stage = [&](int g) {
        float* dst = c2smem + (g & 1) * 2 * kConv2Plane;
        for (int e = threadIdx.x; e < S * S * 2; e += kConv2Threads) {
            const int j = e & 1, p = e >> 1, sy = p / S, sx = p - sy * S;
            const int y = y0 + sy - 1, x = x0 + sx - 1;
            const bool in = y >= 0 && x >= 0 && y < I.ny && x < I.nx;
            const float* src = in ? c1 + ((size_t)I.cell0 + (size_t)y * I.nx + x) * HD + 8 * g + 4 * j : c1;
            cp_async16(dst + j * kConv2Plane + 4 * p, src, in);  // zero outside the grid
        }
        cp_async_commit();
    };
    load_stage(0);
    const int tx = threadIdx.x % kCellTile, sy = (threadIdx.x / kCellTile) * 2;  // cells (tx, sy), (tx, sy + 1)
    float acc[2][C];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int co = 0; co < C; co++) acc[i][co] = cw.b[co];
#pragma unroll
    for (int g = 0; g < NG; g++) {
        if (g + 1 < NG) {
            load_stage(g + 1);
            cp_async_wait_group<1>();
        } else {
            cp_async_wait_group<0>();
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const float4* pl =
                reinterpret_cast<const float4*>(c2smem + (g & 1) * 2 * kConv2Plane + j * kConv2Plane) + sy * S + tx;
            float4 a[4][3];  // halo rows sy..sy+3, columns tx..tx+2, channels 8 g + 4 j ..
#pragma unroll
            for (int r = 0; r < 4; r++)
#pragma unroll
                for (int kx = 0; kx < 3; kx++) a[r][kx] = pl[r * S + kx];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const int ci = 8 * g + 4 * j + c;
#pragma unroll
                for (int ky = 0; ky < 3; ky++)
#pragma unroll
                    for (int kx = 0; kx < 3; kx++) {
                        const int wi = (ci * 9 + ky * 3 + kx) * 3;  // a constant after unrolling
#pragma unroll
                        for (int i = 0; i < 2; i++) {
                            const float4 av = a[i + ky][kx];
                            const float v = c == 0 ? av.x : c == 1 ? av.y : c == 2 ? av.z : av.w;
                            acc[i][0] = fmaf(v, cw.w[wi], acc[i][0]);
                            acc[i][1] = fmaf(v, cw.w[wi + 1], acc[i][1]);
                            acc[i][2] = fmaf(v, cw.w[wi + 2], acc[i][2]);
                        }
                    }
            }
        }
        __syncthreads();  // every thread is done with this buffer before it is refilled
    }
    const size_t plane = (size_t)I.nx * I.ny;
    const int x = x0 + tx;
    if (x >= I.nx) return;
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const int y = y0 + sy + i;
        if (y >= I.ny) break;
        const size_t cl = (size_t)y * I.nx + x;
#pragma unroll
        for (int co = 0; co < C; co++) {
            float v = acc[i][co];
            if (mode == kWriteNextState) v = v + I.state[co * plane + cl];
            I.out[co * plane + cl] = v;
        }
    }
}

// Double-f32 sums for the block trees of the projection: a value hi + lo,
// added error-free (two-sum), so a tree over 512 threads keeps about 2^-44
// relative accuracy on the FP32 pipes; this GPU's f64 rate is a small
// fraction of its f32 rate, and the trees would otherwise be f64 shuffles and
// adds.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_add(DF x, DF y) {
    const float s = __fadd_rn(x.hi, y.hi);
    const float bb = __fsub_rn(s, x.hi);
    const float e = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, bb)), __fsub_rn(y.hi, bb));
    const float t = __fadd_rn(e, __fadd_rn(x.lo, y.lo));
    const float hi = __fadd_rn(s, t);
    return DF{hi, __fsub_rn(t, __fsub_rn(hi, s))};
}
__device__ __forceinline__ DF warp_sum_df(DF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v = df_add(v, DF{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
    return v;
}
// Block sums of two per-thread values in the fixed tree of warp_sum_df:
// warps, then warp 0 over the warp totals; the totals as f64 in thread 0 (the
// only thread that uses them: f64 work in every thread would cost the FP64
// pipe 512 times over).
__device__ void block_sum_df2(DF a, DF b, double& A, double& B, DF* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    a = warp_sum_df(a);
    b = warp_sum_df(b);
    __syncthreads();
    if (lane == 0) {
        red[warp] = a;
        red[32 + warp] = b;
    }
    __syncthreads();
    if (warp == 0) {
        const DF z{0.f, 0.f};
        DF ta = lane < nw ? red[lane] : z, tb = lane < nw ? red[32 + lane] : z;
        ta = warp_sum_df(ta);
        tb = warp_sum_df(tb);
        if (lane == 0) {
            A = (double)ta.hi + (double)ta.lo;
            B = (double)tb.hi + (double)tb.lo;
        }
    }
}

// Mass then energy projection (eval.rs:148-153 order; project.rs:33-54). One
// thread-block cluster of kProjCluster CTAs per instance; each CTA keeps its
// slice of the state in shared memory (when it fits) for the three passes:
//   1. sum h                                   -> mass shift (f32)
//   2. apply the shift; sum potential, kinetic -> energy scale (f32)
//   3. apply the scale; sum potential, kinetic -> energy of the stored state
// Per-cell terms use the reference's f32 arithmetic (project.rs:9-19,
// unfused). Each thread sums its few cells with Kahan compensation in f32;
// the per-thread sums are combined in a fixed-order block tree in
// double-f32, converted to f64, and the cluster's partials are added in f64
// in segment order through distributed shared memory, so every CTA and every
// run sees the same totals. f64 is used only for these combinations and for
// the mass shift and energy scale, which thread 0 forms once per CTA and
// shares (the FP64 rate of this GPU is a small fraction of its FP32 rate, so
// f64 work per cell or per thread would dominate the kernel).
constexpr int kProjCluster = 8;  // largest cluster (the launch picks 1..8 CTAs per instance)
constexpr int kProjThreads = 512;
constexpr int kProjSmemCells = 16384;  // 192 KB of state per CTA at most

__device__ __forceinline__ void pk_terms(const Dims& d, float xh, float xu, float xv, float& pot, float& kin) {
    const float h = __fadd_rn(__fmul_rn(xh, d.norm_std[0]), __fadd_rn(d.norm_mean[0], d.norm_depth));
    const float u = __fadd_rn(__fmul_rn(xu, d.norm_std[1]), d.norm_mean[1]);
    const float v = __fadd_rn(__fmul_rn(xv, d.norm_std[2]), d.norm_mean[2]);
    pot = __fmul_rn(__fmul_rn(__fmul_rn(0.5f, d.g), h), h);
    kin = __fmul_rn(__fmul_rn(0.5f, h), __fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v)));
}

// Kahan-compensated f32 accumulator for a thread's cells.
struct Kahan {
    float s, c;
    __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
    __device__ __forceinline__ void add(float v) {
        const float y = __fsub_rn(v, c);
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
};

// Reduction segments: an instance's cells are cut into segments of
// kProjSeg cells; a segment's sums are always formed the same way (thread t
// takes cells t, t + 512, ... with f32 Kahan compensation, then the fixed
// block tree in double-f32, converted to f64), and the instance total adds
// the segment totals in f64 in
// segment order. A CTA of the cluster owns a contiguous run of segments, so
// the totals do not depend on the cluster size the launch picked, nor on the
// other instances of the launch.
constexpr int kProjSeg = 4096;

// Instance totals of nv (<= 2) values from this CTA's per-segment totals
// mine[k][v] (k < nk): thread 0 reads every rank's segments through
// distributed shared memory and adds them in segment order.
// The cluster's totals of one pass: every CTA's segment totals, in segment
// order. One lane per peer copies that peer's totals into `gather` (the
// remote reads of all peers overlap), then thread 0 adds them in order.
__device__ void cluster_total(cg::cluster_group& cluster, double* mine, int nv, double* out, double* gather,
                              int stride) {
    const int cs = (int)cluster.num_blocks();
    cluster.sync();
    if (threadIdx.x < 32) {
        for (int r = threadIdx.x; r < cs; r += 32) {
            const double* peer = cs == 1 ? mine : cluster.map_shared_rank(mine, r);
            const int nk = (int)peer[0];  // slot 0 holds the segment count
            double* dst = gather + (size_t)r * stride;
            dst[0] = (double)nk;
            for (int i = 0; i < 2 * nk; i++) dst[1 + i] = peer[1 + i];
        }
        __syncwarp();
        if (threadIdx.x == 0) {
            double t[2] = {0.0, 0.0};
            for (int r = 0; r < cs; r++) {
                const double* g = gather + (size_t)r * stride;
                const int nk = (int)g[0];
                for (int k = 0; k < nk; k++)
                    for (int v = 0; v < nv; v++) t[v] += g[1 + 2 * k + v];
            }
            for (int v = 0; v < nv; v++) out[v] = t[v];
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kProjThreads)
projection_kernel(Dims d, const InstDev* inst, ProjSlot* slots, int init, int cap, int seg_cap) {
    JC_PDL_ENTRY;
    // [3][cap] f32: this CTA's cells when they fit; then 3 x (1 + 2 seg_cap)
    // f64: per pass, the segment count and this CTA's segment totals
    extern __shared__ __align__(16) float sst[];
    __shared__ __align__(16) double red[64];  // the block trees' DF scratch (64 pairs)
    __shared__ double tot[4];
    __shared__ float bc[2];  // the mass shift and the energy scale, formed once by thread 0
    cg::cluster_group cluster = cg::this_cluster();
    const int cs = (int)cluster.num_blocks();
    const int ii = blockIdx.x / cs, rank = (int)cluster.block_rank();
    const InstDev& I = inst[ii];
    if (I.flags & 4u) return;  // no projection and no energy record for this instance (the whole cluster)
    ProjSlot& S = I.slot ? *I.slot : slots[ii];
    float* s = I.state;
    const unsigned flags = init ? 0u : I.flags;
    const long long n = (long long)I.nx * I.ny;
    const int nseg = (int)((n + kProjSeg - 1) / kProjSeg);
    const int k0 = (int)((long long)nseg * rank / cs), k1 = (int)((long long)nseg * (rank + 1) / cs);
    const long long c0 = (long long)k0 * kProjSeg, c1 = std::min<long long>((long long)k1 * kProjSeg, n);
    const int m = (int)(c1 > c0 ? c1 - c0 : 0);
    const bool staged = m <= cap;
    double* segs = reinterpret_cast<double*>(sst + 3 * (size_t)cap);  // [3][1 + 2 seg_cap]
    // this CTA's cells, in shared memory if they fit, else in place
    float* H = staged ? sst : s + c0;
    float* U = staged ? sst + cap : s + n + c0;
    float* V = staged ? sst + 2 * cap : s + 2 * n + c0;
    if (staged) {
        // asynchronous copies: every thread's loads are in flight at once,
        // 16 bytes each where the state and the slice allow it
        const bool v4 = ((reinterpret_cast<uintptr_t>(s) | (uintptr_t)n | (uintptr_t)c0 | (uintptr_t)m) & 3u) == 0 &&
                        (reinterpret_cast<uintptr_t>(s) & 15u) == 0;
        if (v4) {
            for (int i = 4 * threadIdx.x; i < m; i += 4 * blockDim.x) {
                cp_async16(H + i, s + c0 + i, true);
                cp_async16(U + i, s + n + c0 + i, true);
                cp_async16(V + i, s + 2 * n + c0 + i, true);
            }
        } else {
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                cp_async4(H + i, s + c0 + i, true);
                cp_async4(U + i, s + n + c0 + i, true);
                cp_async4(V + i, s + 2 * n + c0 + i, true);
            }
        }
        cp_async_wait_all();
        __syncthreads();
    }
    // per-segment sums of term(i) -> (a, b) over this CTA's segments, into
    // pass slot `ps`, then the instance totals
    auto reduce = [&](int ps, int nv, auto&& term) {
        double* mine = segs + (size_t)ps * (1 + 2 * seg_cap);
        if (threadIdx.x == 0) mine[0] = (double)(k1 - k0);
        for (int k = k0; k < k1; k++) {
            Kahan a, b;
            a.init();
            b.init();
            const int base = (k - k0) * kProjSeg;
            for (int j = threadIdx.x; j < kProjSeg; j += blockDim.x) {
                const int i = base + j;
                if (i < m) {
                    float ta, tb;
                    term(i, ta, tb);
                    a.add(ta);
                    if (nv > 1) b.add(tb);
                }
            }
            double A = 0.0, B = 0.0;
            block_sum_df2(DF{a.s, -a.c}, DF{b.s, -b.c}, A, B, reinterpret_cast<DF*>(red));
            if (threadIdx.x == 0) {
                mine[1 + 2 * (k - k0)] = A;
                mine[2 + 2 * (k - k0)] = B;
            }
        }
        __syncthreads();
        cluster_total(cluster, mine, nv, tot, segs + 3 * (size_t)(1 + 2 * seg_cap), 1 + 2 * seg_cap);
    };
    const double prev = S.energy;
    // pass 1: mass
    double M = 0.0;
    if (init || (flags & 1u)) {
        reduce(0, 1, [&](int i, float& a, float& b) {
            a = H[i];
            b = 0.f;
        });
        M = tot[0];
    }
    // pass 2: mass shift, then potential and kinetic energy
    if (threadIdx.x == 0) bc[0] = (flags & 1u) ? (float)(S.mass0 - M / (double)n) : 0.0f;
    __syncthreads();
    const float delta = bc[0];
    reduce(1, 2, [&](int i, float& pot, float& kin) {
        float h = H[i];
        if (flags & 1u) {
            h = __fadd_rn(h, delta);
            H[i] = h;
        }
        pk_terms(d, h, U[i], V[i], pot, kin);
    });
    double P = tot[0], K = tot[1];
    if (init) {
        if (rank == 0 && threadIdx.x == 0) {
            S.mass0 = M / (double)n;
            S.energy = P + K;
            S.max_viol = 0.0;
            S.last_scale = 1.0;
        }
    } else {
        // pass 3: energy scale of (u, v), then the energy of the stored state
        if (flags & 2u) {
            double sc = 1.0;
            if (threadIdx.x == 0) {
                const double bound = prev * (double)d.energy_r_max;
                double budget = bound - P;
                if (!(budget > 0.0)) budget = 0.0;
                sc = sqrt(budget / (K > 1e-12 ? K : 1e-12));
                sc = sc < 0.0 ? 0.0 : (sc > 1.0 ? 1.0 : sc);
                bc[1] = (float)sc;
            }
            __syncthreads();
            const float s32 = bc[1];
            reduce(2, 2, [&](int i, float& pot, float& kin) {
                float u = __fadd_rn(__fmul_rn(U[i], d.norm_std[1]), d.norm_mean[1]);
                float v = __fadd_rn(__fmul_rn(V[i], d.norm_std[2]), d.norm_mean[2]);
                u = __fdiv_rn(__fsub_rn(__fmul_rn(u, s32), d.norm_mean[1]), d.norm_std[1]);
                v = __fdiv_rn(__fsub_rn(__fmul_rn(v, s32), d.norm_mean[2]), d.norm_std[2]);
                U[i] = u;
                V[i] = v;
                pk_terms(d, H[i], u, v, pot, kin);
            });
            P = tot[0];
            K = tot[1];
            if (rank == 0 && threadIdx.x == 0) S.last_scale = sc;
        }
        if (rank == 0 && threadIdx.x == 0) {
            const double E = P + K;
            const double viol = (E - prev * (double)d.energy_r_max) / prev;
            if (viol > S.max_viol) S.max_viol = viol;
            S.energy = E;
        }
    }
    if (staged && (flags & 3u)) {
        __syncthreads();
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            if (flags & 1u) s[c0 + i] = H[i];
            if (flags & 2u) {
                s[n + c0 + i] = U[i];
                s[2 * n + c0 + i] = V[i];
            }
        }
    }
    cluster.sync();  // peers may still read this CTA's segment totals
}

}  // namespace f32k

template <int BN, class AL, class EP>
static void gemm(const char* name, const AL& a, const float* W, const float* b, int R, int N, int K, const EP& e,
                 cudaStream_t s) {
    KScope k(name, s);
    dim3 grid((N + BN - 1) / BN, (R + 63) / 64);
    f32k::gemm_kernel<BN, AL, EP><<<grid, BN * 4, 0, s>>>(a, W, b, R, N, K, e);
    check_launch(name);
}

void forward_f32(const Dims& d, const WeightsF32& w, const Pack& p, int mode, cudaStream_t s) {
    using namespace f32k;
    const int R = p.R, D = d.D, n = p.n_inst;
    {
        KScope k("f32_embed", s);
        int pd = d.C * d.P * d.P;
        embed_kernel<<<(R + kEmbedTok - 1) / kEmbedTok, 128, kEmbedTok * pd * sizeof(float), s>>>(
            d, w.embed_w, w.embed_b, w.meta_w, w.meta_b, p.inst, n, R, p.x);
        check_launch("embed");
    }
    for (int l = 0; l < d.L; l++) {
        const auto& B = w.blk[l];
        gemm<64>("f32_ln_qkv", ALayerNorm{p.x, B.n1g, B.n1b, R, D}, B.wqkv, B.bqkv, R, 3 * D, D,
                 EStore{p.qkv, 3 * D}, s);
        {
            KScope k("f32_attention", s);
            long long warps = (long long)R * d.heads;
            attention_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(d, p.qkv, p.inst, n, R, p.attn);
            check_launch("attention");
        }
        gemm<64>("f32_proj", APlain{p.attn, D, R, D}, B.wp, B.bp, R, D, D, EResid{p.x, D}, s);
        gemm<64>("f32_ln_ff1", ALayerNorm{p.x, B.n2g, B.n2b, R, D}, B.w1, B.b1, R, d.F, D, EGelu{p.ff1, d.F}, s);
        gemm<64>("f32_ff2", APlain{p.ff1, d.F, R, d.F}, B.w2, B.b2, R, D, d.F, EResid{p.x, D}, s);
    }
    {
        KScope k("f32_final_ln", s);
        layernorm_kernel<<<(R + 7) / 8, 256, 0, s>>>(p.x, w.norm_g, w.norm_b, R, D, p.xn);
        check_launch("layernorm");
    }
    gemm<64>("f32_token_mix", ATokConv3{p.xn, p.inst, n, R, D}, w.tm_w, w.tm_b, R, D, 9 * D,
             EGeluResidFrom{p.xn, p.t1, D}, s);
    gemm<32>("f32_to_cells", APlain{p.t1, D, R, D}, w.tc_w, w.tc_b, R, d.HD, D, EStore{p.z0, d.HD}, s);
    const long long NC = p.NC;
    {
        KScope k("f32_upsample_concat", s);
        upsample_concat_kernel<<<(unsigned)((NC + 255) / 256), 256, 0, s>>>(d, p.z0, p.inst, n, NC, p.zc);
        check_launch("upsample_concat");
    }
    gemm<32>("f32_conv1", ACellConv3{p.zc, p.inst, n, (int)NC, kZcStride}, w.c1_w, w.c1_b, (int)NC, d.HD,
             9 * kZcStride, EGelu{p.c1, d.HD}, s);
    conv2_step(d, p.c1, w, p, mode, "f32_conv2_step", s);
}

void conv2_step(const Dims& d, const float* c1, const WeightsF32& w, const Pack& p, int mode, const char* name,
                cudaStream_t s) {
    KScope k(name, s);
    if (d.C != 3 || d.HD != 32) throw std::runtime_error("conv2 is built for 3 channels and a cell-head width of 32");
    static std::atomic<unsigned long long> attr{0};
    set_smem_per_device(f32k::conv2_step_kernel<3, 32>, f32k::kConv2Smem, attr);
    if (!w.c2p) throw std::runtime_error("conv2 weights missing");
    const cudaError_t e = launch_pdl(f32k::conv2_step_kernel<3, 32>, dim3(p.n_tiles), dim3(f32k::kConv2Threads),
                                     f32k::kConv2Smem, s, 1u, c1, *w.c2p, (const InstDev*)p.inst, p.n_inst, mode);
    if (e != cudaSuccess) throw std::runtime_error(std::string(name) + ": " + cudaGetErrorString(e));
    check_launch(name);
}

void projection(const Dims& d, const Pack& p, int init, cudaStream_t s) {
    KScope k("projection", s);
    static std::atomic<unsigned long long> attr{0};
    set_smem_per_device(f32k::projection_kernel, 200 * 1024, attr);
    // cluster size: the smallest whose slices fit in shared memory, and about
    // one CTA per SM (152 here) when the instances are few; the sums do not
    // depend on it (segment totals in segment order)
    const long long nseg = (p.max_inst_cells + f32k::kProjSeg - 1) / f32k::kProjSeg;
    int cs = 1;
    while (cs < f32k::kProjCluster && (nseg + cs - 1) / cs * f32k::kProjSeg > f32k::kProjSmemCells) cs *= 2;
    while (cs < f32k::kProjCluster && (long long)p.n_inst * cs < 152 && nseg >= 2LL * cs) cs *= 2;
    const long long seg_cap = (nseg + cs - 1) / cs;
    // staged in shared memory when a CTA's cells fit, else passes run in place
    const int cap = seg_cap * f32k::kProjSeg <= f32k::kProjSmemCells ? (int)(seg_cap * f32k::kProjSeg) : 1;
    const size_t smem = (size_t)3 * cap * 4 + (size_t)(3 + cs) * (1 + 2 * seg_cap) * 8;
    cuda_check_attr(launch_pdl(f32k::projection_kernel, dim3((unsigned)(p.n_inst * cs)), dim3(f32k::kProjThreads), smem,
                               s, (unsigned)cs, d, (const InstDev*)p.inst, p.proj, init, cap, (int)seg_cap));
    check_launch("projection");
}

}  // namespace jc
