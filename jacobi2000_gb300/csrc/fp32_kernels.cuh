// FP32 CUDA-core kernels: the plain path, the reference's arithmetic
// (crates/engine/src/cpu.rs) on the GPU. Token-level buffers are row-major
// [rows, features] over the rows of all instances of a launch; cell-level
// buffers are channel-last [cells, channels].
#pragma once

#include "common.cuh"

namespace jc {
namespace f32k {

// ---------------------------------------------------------------------------
// A-operand loaders of the tiled GEMM. `prologue` runs once per CTA for the
// CTA's rows; `load(r, k)` returns A[r][k] (0 outside [0,R) x [0,K)).

struct APlain {
    const float* A;
    int lda;
    int R, K;
    __device__ void prologue(int, int, float*) const {}
    __device__ float load(int r, int k, const float*) const {
        return (r < R && k < K) ? A[(size_t)r * lda + k] : 0.0f;
    }
};

// LayerNorm of X's rows fused into the load (cpu.rs:49-65: two-pass mean and
// biased variance, eps 1e-5 before the sqrt). K = D. Row statistics for the
// CTA's BM rows are computed in the prologue into `stats` (2 * BM floats).
struct ALayerNorm {
    const float* X;
    const float* gamma;
    const float* beta;
    int R, D;
    __device__ void prologue(int row0, int bm, float* stats) const {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
        for (int i = warp; i < bm; i += nw) {
            int r = row0 + i;
            float mean = 0.f, rstd = 0.f;
            if (r < R) {
                const float* x = X + (size_t)r * D;
                float s = 0.f;
                for (int d = lane; d < D; d += 32) s += x[d];
                s = warp_sum(s);
                mean = s / (float)D;
                float v = 0.f;
                for (int d = lane; d < D; d += 32) { float t = x[d] - mean; v += t * t; }
                v = warp_sum(v);
                rstd = 1.0f / sqrtf(v / (float)D + 1e-5f);
            }
            if (lane == 0) { stats[2 * i] = mean; stats[2 * i + 1] = rstd; }
        }
    }
    __device__ float load(int r, int k, const float* stats, int row0) const {
        if (r >= R || k >= D) return 0.0f;
        int i = r - row0;
        return (X[(size_t)r * D + k] - stats[2 * i]) * stats[2 * i + 1] * gamma[k] + beta[k];
    }
};

// 3x3 zero-padded cross-correlation over each instance's token grid
// (cpu.rs:171-205 on t0 [D, ty, tx]) as an implicit GEMM: A[r][tap*C + c] =
// X[neighbour(r, tap)][c], or 0 outside the grid. K = 9 * C.
struct ATokConv3 {
    const float* X;          // [rows, C]
    const int* row_inst;     // row -> instance
    const InstDev* inst;
    int R, C;
    __device__ void prologue(int, int, float*) const {}
    __device__ float load(int r, int k, const float*) const {
        if (r >= R || k >= 9 * C) return 0.0f;
        int tap = k / C, c = k - tap * C;
        const InstDev& I = inst[row_inst[r]];
        int t = r - I.row0;
        int y = t / I.tx + tap / 3 - 1, x = t % I.tx + tap % 3 - 1;
        if (y < 0 || x < 0 || y >= I.ty || x >= I.tx) return 0.0f;
        return X[(size_t)(I.row0 + y * I.tx + x) * C + c];
    }
};

// Same over each instance's cell grid: rows are cells, X is [cells, C].
struct ACellConv3 {
    const float* X;
    const int* cell_inst;
    const InstDev* inst;
    int R, C, Cin;           // C = row stride (padded), Cin = real channels
    __device__ void prologue(int, int, float*) const {}
    __device__ float load(int r, int k, const float*) const {
        if (r >= R || k >= 9 * C) return 0.0f;
        int tap = k / C, c = k - tap * C;
        if (c >= Cin) return 0.0f;
        const InstDev& I = inst[cell_inst[r]];
        long long cl = r - I.cell0;
        int y = (int)(cl / I.nx) + tap / 3 - 1, x = (int)(cl % I.nx) + tap % 3 - 1;
        if (y < 0 || x < 0 || y >= I.ny || x >= I.nx) return 0.0f;
        return X[(size_t)(I.cell0 + (long long)y * I.nx + x) * C + c];
    }
};

// Epilogues: v already includes the bias.
struct EStore {
    float* out; int ld;
    __device__ void operator()(int r, int n, float v) const { out[(size_t)r * ld + n] = v; }
};
struct EGelu {
    float* out; int ld;
    __device__ void operator()(int r, int n, float v) const { out[(size_t)r * ld + n] = gelu_erf(v); }
};
struct EResid {  // x += v (cpu.rs:306,312 add_inplace)
    float* x; int ld;
    __device__ void operator()(int r, int n, float v) const { x[(size_t)r * ld + n] += v; }
};
struct EGeluResidFrom {  // out = src + gelu(v) (cpu.rs:327-328)
    const float* src; float* out; int ld;
    __device__ void operator()(int r, int n, float v) const {
        out[(size_t)r * ld + n] = src[(size_t)r * ld + n] + gelu_erf(v);
    }
};

template <class AL>
__device__ __forceinline__ float aload_call(const AL& a, int r, int k, const float* stats, int) {
    return a.load(r, k, stats);
}
template <>
__device__ __forceinline__ float aload_call<ALayerNorm>(const ALayerNorm& a, int r, int k, const float* stats,
                                                        int row0) {
    return a.load(r, k, stats, row0);
}

// out[r][n] = epi(bias[n] + sum_k A[r][k] W[k][n]). W is [K, N] row-major
// (the checkpoint's Linear layout). BM x BN tile per CTA, TM x TN per thread,
// K in steps of BK through shared memory.
template <int BM, int BN, int BK, int TM, int TN, class AL, class EP>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gemm_kernel(AL aload, const float* __restrict__ W, const float* __restrict__ bias, int R, int N, int K, EP epi) {
    constexpr int NT = (BM / TM) * (BN / TN);
    __shared__ float As[BK][BM + 4];
    __shared__ float Bs[BK][BN + 4];
    __shared__ float stats[2 * BM];
    const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;
    const int tid = threadIdx.x;
    const int tr = (tid / (BN / TN)) * TM, tc = (tid % (BN / TN)) * TN;
    aload.prologue(row0, BM, stats);
    __syncthreads();

    // the accumulator starts from the bias, as cpu.rs:28 does
    float acc[TM][TN];
#pragma unroll
    for (int j = 0; j < TN; j++) {
        int n = col0 + tc + j;
        float b0 = n < N ? bias[n] : 0.0f;
#pragma unroll
        for (int i = 0; i < TM; i++) acc[i][j] = b0;
    }

    for (int k0 = 0; k0 < K; k0 += BK) {
        for (int e = tid; e < BM * BK; e += NT) {
            int i = e / BK, kk = e % BK;
            As[kk][i] = aload_call(aload, row0 + i, k0 + kk, stats, row0);
        }
        for (int e = tid; e < BK * BN; e += NT) {
            int kk = e / BN, j = e % BN;
            int k = k0 + kk, n = col0 + j;
            Bs[kk][j] = (k < K && n < N) ? W[(size_t)k * N + n] : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            float a[TM], b[TN];
#pragma unroll
            for (int i = 0; i < TM; i++) a[i] = As[kk][tr + i];
#pragma unroll
            for (int j = 0; j < TN; j++) b[j] = Bs[kk][tc + j];
#pragma unroll
            for (int i = 0; i < TM; i++)
#pragma unroll
                for (int j = 0; j < TN; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < TM; i++) {
        int r = row0 + tr + i;
        if (r >= R) continue;
#pragma unroll
        for (int j = 0; j < TN; j++) {
            int n = col0 + tc + j;
            if (n < N) epi(r, n, acc[i][j]);
        }
    }
}

}  // namespace f32k
}  // namespace jc
