// FP32 CUDA-core kernels: the plain path, the reference's arithmetic
// (crates/engine/src/cpu.rs) on the GPU. Token-level buffers are row-major
// [rows, features] over the rows of all instances of a launch; cell-level
// buffers are channel-last [cells, channels].
#pragma once

#include "common.cuh"

namespace jc {
namespace f32k {

// Per-row context a loader may cache in shared memory in its prologue.
struct RowCtx {
    int base;   // first row (token loaders) or cell (cell loaders) of the instance
    int y, x;   // coordinates inside the instance's grid
    int w, h;   // grid width and height
};

// ---------------------------------------------------------------------------
// A-operand loaders of the tiled GEMM. `prologue` runs once per CTA for its
// BM rows; `load4(r, k, ctx)` returns A[r][k..k+3] (zeros outside the
// matrix); K and the loaders' channel counts are multiples of 4.

struct APlain {
    const float* A;
    int lda, R, K;
    __device__ void prologue(int, int, float*, RowCtx*) const {}
    __device__ float4 load4(int r, int k, int, const float*, const RowCtx*) const {
        if (r >= R || k >= K) return make_float4(0.f, 0.f, 0.f, 0.f);
        return *reinterpret_cast<const float4*>(A + (size_t)r * lda + k);
    }
};

// LayerNorm of X's rows fused into the load (cpu.rs:49-65: two-pass mean and
// biased variance, eps 1e-5 before the sqrt). K = D.
struct ALayerNorm {
    const float* X;
    const float* gamma;
    const float* beta;
    int R, D;
    __device__ void prologue(int row0, int bm, float* stats, RowCtx*) const {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
        for (int i = warp; i < bm; i += nw) {
            int r = row0 + i;
            float mean = 0.f, rstd = 0.f;
            if (r < R) {
                const float* x = X + (size_t)r * D;
                float s = 0.f;
                for (int d = lane; d < D; d += 32) s += x[d];
                mean = warp_sum(s) / (float)D;
                float v = 0.f;
                for (int d = lane; d < D; d += 32) { float t = x[d] - mean; v += t * t; }
                rstd = 1.0f / sqrtf(warp_sum(v) / (float)D + 1e-5f);
            }
            if (lane == 0) { stats[2 * i] = mean; stats[2 * i + 1] = rstd; }
        }
    }
    __device__ float4 load4(int r, int k, int i, const float* stats, const RowCtx*) const {
        if (r >= R || k >= D) return make_float4(0.f, 0.f, 0.f, 0.f);
        float4 x = *reinterpret_cast<const float4*>(X + (size_t)r * D + k);
        float4 g = *reinterpret_cast<const float4*>(gamma + k);
        float4 b = *reinterpret_cast<const float4*>(beta + k);
        const float m = stats[2 * i], s = stats[2 * i + 1];
        return make_float4((x.x - m) * s * g.x + b.x, (x.y - m) * s * g.y + b.y, (x.z - m) * s * g.z + b.z,
                           (x.w - m) * s * g.w + b.w);
    }
};

// 3x3 zero-padded cross-correlation (cpu.rs:171-205) as an implicit GEMM:
// A[r][tap*C + c] = X[neighbour(r, tap)][c], or 0 outside the grid; K = 9 C.
// Token variant: rows are tokens of each instance's token grid.
struct ATokConv3 {
    const float* X;  // [rows, C]
    const InstDev* inst;
    int n_inst, R, C;
    __device__ void prologue(int row0, int bm, float*, RowCtx* ctx) const {
        for (int i = threadIdx.x; i < bm; i += blockDim.x) {
            int r = row0 + i;
            RowCtx c{0, -100, -100, 0, 0};
            if (r < R) {
                const InstDev& I = inst[inst_of_row(inst, n_inst, r)];
                int t = r - I.row0;
                c = RowCtx{I.row0, t / I.tx, t % I.tx, I.tx, I.ty};
            }
            ctx[i] = c;
        }
    }
    __device__ float4 load4(int r, int k, int i, const float*, const RowCtx* ctx) const {
        const RowCtx c = ctx[i];
        int tap = k / C, ch = k - tap * C;
        int y = c.y + tap / 3 - 1, x = c.x + tap % 3 - 1;
        if (r >= R || tap >= 9 || y < 0 || x < 0 || y >= c.h || x >= c.w) return make_float4(0.f, 0.f, 0.f, 0.f);
        return *reinterpret_cast<const float4*>(X + (size_t)(c.base + y * c.w + x) * C + ch);
    }
};

// Cell variant: rows are cells of each instance's cell grid, X [cells, C].
struct ACellConv3 {
    const float* X;
    const InstDev* inst;
    int n_inst, R, C;
    __device__ void prologue(int row0, int bm, float*, RowCtx* ctx) const {
        for (int i = threadIdx.x; i < bm; i += blockDim.x) {
            int r = row0 + i;
            RowCtx c{0, -100, -100, 0, 0};
            if (r < R) {
                const InstDev& I = inst[inst_of_cell(inst, n_inst, r)];
                int cl = (int)(r - I.cell0);
                c = RowCtx{(int)I.cell0, cl / I.nx, cl % I.nx, I.nx, I.ny};
            }
            ctx[i] = c;
        }
    }
    __device__ float4 load4(int r, int k, int i, const float*, const RowCtx* ctx) const {
        const RowCtx c = ctx[i];
        int tap = k / C, ch = k - tap * C;
        int y = c.y + tap / 3 - 1, x = c.x + tap % 3 - 1;
        if (r >= R || tap >= 9 || y < 0 || x < 0 || y >= c.h || x >= c.w) return make_float4(0.f, 0.f, 0.f, 0.f);
        return *reinterpret_cast<const float4*>(X + ((size_t)c.base + (size_t)y * c.w + x) * C + ch);
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

// out[r][n] = epi(bias[n] + sum_k A[r][k] W[k][n]). W is [K, N] row-major
// (the checkpoint's Linear layout). 64 x 64 tile per CTA, 4 x 4 per thread,
// K in steps of 16 through double-buffered shared memory: the next tile is
// fetched into registers while the current one is multiplied.
template <int BN, class AL, class EP>
__global__ void __launch_bounds__(BN * 4)
gemm_kernel(AL aload, const float* __restrict__ W, const float* __restrict__ bias, int R, int N, int K, EP epi) {
    constexpr int BM = 64, BK = 16, TM = 4, TN = 4, NT = BN * 4;
    static_assert((BM / TM) * (BN / TN) == NT, "thread count");
    __shared__ __align__(16) float As[2][BK][BM + 4];
    __shared__ __align__(16) float Bs[2][BK][BN + 4];
    __shared__ float stats[2 * BM];
    __shared__ RowCtx ctx[BM];
    const int row0 = blockIdx.y * BM, col0 = blockIdx.x * BN;
    const int tid = threadIdx.x;
    const int tr = (tid / (BN / TN)) * TM, tc = (tid % (BN / TN)) * TN;
    aload.prologue(row0, BM, stats, ctx);
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

    // A: BM*BK/4 float4 per tile; B: BK*BN/4 float4 per tile
    constexpr int A4 = BM * BK / 4, B4 = BK * BN / 4;
    float4 ra[(A4 + NT - 1) / NT], rb[(B4 + NT - 1) / NT];
    auto fetch = [&](int k0) {
#pragma unroll
        for (int q = 0; q < (A4 + NT - 1) / NT; q++) {
            int e = tid + q * NT;
            if (e < A4) {
                int i = e / (BK / 4), kk = (e % (BK / 4)) * 4;
                ra[q] = aload.load4(row0 + i, k0 + kk, i, stats, ctx);
            }
        }
#pragma unroll
        for (int q = 0; q < (B4 + NT - 1) / NT; q++) {
            int e = tid + q * NT;
            if (e < B4) {
                int kk = e / (BN / 4), j = (e % (BN / 4)) * 4;
                int k = k0 + kk, n = col0 + j;
                rb[q] = (k < K && n < N) ? *reinterpret_cast<const float4*>(W + (size_t)k * N + n)
                                         : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    };
    auto stash = [&](int buf) {
#pragma unroll
        for (int q = 0; q < (A4 + NT - 1) / NT; q++) {
            int e = tid + q * NT;
            if (e < A4) {
                int i = e / (BK / 4), kk = (e % (BK / 4)) * 4;
                As[buf][kk + 0][i] = ra[q].x;
                As[buf][kk + 1][i] = ra[q].y;
                As[buf][kk + 2][i] = ra[q].z;
                As[buf][kk + 3][i] = ra[q].w;
            }
        }
#pragma unroll
        for (int q = 0; q < (B4 + NT - 1) / NT; q++) {
            int e = tid + q * NT;
            if (e < B4) {
                int kk = e / (BN / 4), j = (e % (BN / 4)) * 4;
                *reinterpret_cast<float4*>(&Bs[buf][kk][j]) = rb[q];
            }
        }
    };

    const int nk = (K + BK - 1) / BK;
    fetch(0);
    stash(0);
    __syncthreads();
    for (int kt = 0; kt < nk; kt++) {
        const int buf = kt & 1;
        if (kt + 1 < nk) fetch((kt + 1) * BK);
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            float4 a = *reinterpret_cast<const float4*>(&As[buf][kk][tr]);
            float4 b = *reinterpret_cast<const float4*>(&Bs[buf][kk][tc]);
            float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < TM; i++)
#pragma unroll
                for (int j = 0; j < TN; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        if (kt + 1 < nk) stash(buf ^ 1);
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
