// BF16 tensor-core forward path (sm_103a).
//
// Per tick and model group (crates/engine/src/cpu.rs:249-352 restated):
//   embed (CUDA cores)      patchify + embed + pos + meta -> x (f32), LN1(x) (bf16)
//   per layer:
//     qkv   (tcgen05 GEMM)  LN1(x) @ Wqkv + b                      -> qkv (bf16)
//     attention (CUDA cores) stencil-masked softmax over <= (2r+1)^2 keys -> attn (bf16)
//     proj  (tcgen05 GEMM)  x += attn @ Wp + b; LN2(x)             -> x (f32), LN2(x) (bf16)
//     mlp   (tcgen05, fused) x += gelu(LN2(x) @ W1 + b1) @ W2 + b2; LN(x) for the next step
//   token_mix (tcgen05 conv) t1 = xn + gelu(conv3x3(xn) + b)        (bf16)
//   to_cells (tcgen05 GEMM) z0 = t1 @ Wtc + b                      (f32)
//   upsample (CUDA cores)   zc = [upsample(z0), state]             (bf16, 48 channels)
//   conv1 (tcgen05 conv)    c1 = gelu(conv3x3(zc) + b)             (bf16)
//   conv2 + step (CUDA cores) next = state + conv3x3(c1) + b       (f32)
// The two 3x3 convolutions are implicit GEMMs without an im2col copy: a
// halo tile (10 x 18 positions, all channels) is loaded once by TMA in the
// no-swizzle core-matrix layout and each of the 9 taps is the same tile
// addressed through a shifted shared-memory descriptor.
#include <cuda.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>

#include "bf16_path.hpp"
#include "tc.cuh"

namespace jc {

typedef __nv_bfloat16 bf16;

static void check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
// host: bf16 conversion and tensor maps

static uint16_t f2bf(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40);  // NaN stays NaN
    u += 0x7fffu + ((u >> 16) & 1u);  // round to nearest even
    return (uint16_t)(u >> 16);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        cuda_check(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q),
                   "cuTensorMapEncodeTiled entry point");
        if (q != cudaDriverEntryPointSuccess || !p) throw Error(JC_CUDA_ERROR, "cuTensorMapEncodeTiled unavailable");
        fn = (EncodeTiledFn)p;
    }
    return fn;
}

// bf16 tensor of `rank` dims (innermost first), strides in bytes of dims
// 1..rank-1, box dims; no swizzle, zero fill out of bounds.
static CUtensorMap make_map(const void* base, int rank, const uint64_t* dims, const uint64_t* strides,
                            const uint32_t* box) {
    CUtensorMap m;
    cuuint64_t gd[5], gs[4];
    cuuint32_t bx[5], es[5];
    for (int i = 0; i < rank; i++) {
        gd[i] = dims[i];
        bx[i] = box[i];
        es[i] = 1;
    }
    for (int i = 0; i < rank - 1; i++) gs[i] = strides[i];
    CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, rank, const_cast<void*>(base), gd, gs, bx, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error(JC_CUDA_ERROR, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return m;
}

// Rows of a [rows, cols] bf16 matrix, loaded as 8-column x 128-row boxes.
static CUtensorMap rows_map(const void* base, int cols, int rows) {
    uint64_t dims[2] = {(uint64_t)cols, (uint64_t)(rows > 0 ? rows : 1)};
    uint64_t strides[1] = {(uint64_t)cols * 2};
    uint32_t box[2] = {8, 128};
    return make_map(base, 2, dims, strides, box);
}

// One instance's [ny, nx, C] channel-last grid, loaded as 8-channel x 10 x 18 halo boxes.
static CUtensorMap halo_map(const void* base, int C, int nx, int ny) {
    uint64_t dims[3] = {(uint64_t)C, (uint64_t)nx, (uint64_t)ny};
    uint64_t strides[2] = {(uint64_t)C * 2, (uint64_t)nx * C * 2};
    uint32_t box[3] = {8, kConvTX + 2, kConvTY + 2};
    return make_map(base, 3, dims, strides, box);
}

// ---------------------------------------------------------------------------
// device

// bf16 cell-head input channels: 32 z, then the state split exactly into
// bf16 parts, s = hi + lo: [hi (3), lo (3), hi (3)] multiplied by the conv1
// weights [W_hi, W_hi, W_lo], so the state enters conv1 with ~16-bit rather
// than 8-bit precision; the remaining 7 channels are zero.
constexpr int kZcCh = 48;
constexpr int kZcState = 32;
constexpr int kHaloW = kConvTX + 2, kHaloH = kConvTY + 2;
// bytes of one 8-channel plane of a halo tile (2880 used), padded so every
// plane starts on a 128-byte boundary for TMA
constexpr int kHaloPlane = (kHaloW * kHaloH * 16 + 127) / 128 * 128;

__device__ __forceinline__ float bf2f(bf16 v) { return __bfloat162float(v); }

// Token embedding and the first LayerNorm (cpu.rs:253-280, 289). One CTA per
// 64 token rows: the embed weights and the 64 patches are staged in shared
// memory (patches gathered x-contiguously from the state), then one warp per
// token computes its D outputs (lane handles o = lane + 32 j), adds pos and
// the meta linear, writes x (f32) and LayerNorm(x) (bf16).
constexpr int kEmbedRows = 64;

template <int DPL>
__global__ void __launch_bounds__(256) bf_embed_kernel(Dims d, const float* __restrict__ We,
                                                       const float* __restrict__ be, const float* __restrict__ Wm,
                                                       const float* __restrict__ bm, const float* __restrict__ g,
                                                       const float* __restrict__ b, const InstDev* inst, int n_inst,
                                                       int R, float* __restrict__ x, bf16* __restrict__ ln) {
    extern __shared__ float esm[];
    const int D = d.D, P = d.P, pd = d.C * P * P;
    float* sW = esm;                 // [pd][D]
    float* sP = esm + (size_t)pd * D;  // [kEmbedRows][pd]
    __shared__ int rinst[kEmbedRows];
    const int r0 = blockIdx.x * kEmbedRows;
    for (int i = threadIdx.x; i < pd * D; i += blockDim.x) sW[i] = We[i];
    if (threadIdx.x < kEmbedRows)
        rinst[threadIdx.x] = r0 + (int)threadIdx.x < R ? inst_of_row(inst, n_inst, r0 + threadIdx.x) : -1;
    __syncthreads();
    for (int e = threadIdx.x; e < kEmbedRows * pd; e += blockDim.x) {
        const int px = e % P, i = (e / P) % kEmbedRows, cpy = e / (P * kEmbedRows);
        const int c = cpy / P, py = cpy % P;
        float v = 0.f;
        if (rinst[i] >= 0) {
            const InstDev& I = inst[rinst[i]];
            const int t = r0 + i - I.row0;
            const int y = (t / I.tx) * P + py, xx = (t % I.tx) * P + px;
            v = I.state[((size_t)c * I.ny + y) * I.nx + xx];
        }
        sP[i * pd + c * P * P + py * P + px] = v;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = warp; i < kEmbedRows; i += (int)(blockDim.x >> 5)) {
        const int r = r0 + i;
        if (r >= R) break;
        const InstDev& I = inst[rinst[i]];
        const int t = r - I.row0;
        float v[DPL];
#pragma unroll
        for (int j = 0; j < DPL; j++) {
            const int o = lane + 32 * j;
            v[j] = o < D ? be[o] : 0.f;
        }
        const float* pp = sP + i * pd;
        for (int f = 0; f < pd; f++) {
            const float pv = pp[f];
#pragma unroll
            for (int j = 0; j < DPL; j++) {
                const int o = lane + 32 * j;
                if (o < D) v[j] = fmaf(pv, sW[f * D + o], v[j]);
            }
        }
        float sum = 0.f;
#pragma unroll
        for (int j = 0; j < DPL; j++) {
            const int o = lane + 32 * j;
            if (o < D) {
                float m = bm[o];
                for (int f = 0; f < d.meta_dim; f++) m = fmaf(I.meta[f], Wm[(size_t)f * D + o], m);
                v[j] = (v[j] + I.pos[(size_t)t * D + o]) + m;
                x[(size_t)r * D + o] = v[j];
                sum += v[j];
            }
        }
        const float mean = warp_sum(sum) / (float)D;
        float q = 0.f;
#pragma unroll
        for (int j = 0; j < DPL; j++)
            if (lane + 32 * j < D) q += (v[j] - mean) * (v[j] - mean);
        const float rstd = 1.0f / sqrtf(warp_sum(q) / (float)D + 1e-5f);
#pragma unroll
        for (int j = 0; j < DPL; j++) {
            const int o = lane + 32 * j;
            if (o < D) ln[(size_t)r * D + o] = __float2bfloat16((v[j] - mean) * rstd * g[o] + b[o]);
        }
    }
}

// Stencil-masked attention on bf16 q/k/v (cpu.rs:97-164, mask.rs:18-30).
// One warp per query token, all heads at once: lane l holds features
// [FPL l, FPL l + FPL) and heads occupy 32/heads consecutive lanes. Scores are
// reduced within a head's lanes; softmax is the online (running max) form in
// f32 over the candidates in increasing key index.
template <int FPL>
struct BfVec;
template <>
struct BfVec<1> {
    __device__ static void load(const bf16* p, float* o) { o[0] = bf2f(p[0]); }
    __device__ static void store(bf16* p, const float* o) { p[0] = __float2bfloat16(o[0]); }
};
template <>
struct BfVec<4> {
    __device__ static void load(const bf16* p, float* o) {
        uint2 u = *reinterpret_cast<const uint2*>(p);
        __nv_bfloat162 a = *reinterpret_cast<__nv_bfloat162*>(&u.x), b = *reinterpret_cast<__nv_bfloat162*>(&u.y);
        float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
        o[0] = fa.x; o[1] = fa.y; o[2] = fb.x; o[3] = fb.y;
    }
    __device__ static void store(bf16* p, const float* o) {
        __nv_bfloat162 a = __floats2bfloat162_rn(o[0], o[1]), b = __floats2bfloat162_rn(o[2], o[3]);
        uint2 u;
        u.x = *reinterpret_cast<uint32_t*>(&a);
        u.y = *reinterpret_cast<uint32_t*>(&b);
        *reinterpret_cast<uint2*>(p) = u;
    }
};
template <>
struct BfVec<8> {
    __device__ static void load(const bf16* p, float* o) {
        uint4 u = *reinterpret_cast<const uint4*>(p);
        const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&w[i]);
            float2 f = __bfloat1622float2(h);
            o[2 * i] = f.x;
            o[2 * i + 1] = f.y;
        }
    }
    __device__ static void store(bf16* p, const float* o) {
        uint32_t w[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            __nv_bfloat162 h = __floats2bfloat162_rn(o[2 * i], o[2 * i + 1]);
            w[i] = *reinterpret_cast<uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(p) = make_uint4(w[0], w[1], w[2], w[3]);
    }
};

template <int FPL>
__global__ void __launch_bounds__(256) bf_attention_kernel(Dims d, const bf16* __restrict__ qkv, const InstDev* inst,
                                                           int n_inst, int R, bf16* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= R) return;
    const int D = d.D, D3 = 3 * D;
    const int lph = 32 / d.heads;  // lanes per head
    const InstDev& I = inst[inst_of_row(inst, n_inst, r)];
    const int t = r - I.row0, qy = t / I.tx, qx = t % I.tx;
    const float scale = 1.0f / sqrtf((float)(D / d.heads));
    float q[FPL];
    BfVec<FPL>::load(qkv + (size_t)r * D3 + lane * FPL, q);
    const int side = 2 * d.radius + 1;
    const int nc = d.mask_kind == 0 ? I.tx * I.ty : side * side;
    float m = -INFINITY, l = 0.f, acc[FPL];
#pragma unroll
    for (int i = 0; i < FPL; i++) acc[i] = 0.f;
    for (int j = 0; j < nc; j++) {
        int kr;
        if (d.mask_kind == 0) {
            kr = I.row0 + j;
        } else {
            int ky = qy + (j / side - d.radius) * d.dilation, kx = qx + (j % side - d.radius) * d.dilation;
            if (ky < 0 || kx < 0 || ky >= I.ty || kx >= I.tx) continue;
            kr = I.row0 + ky * I.tx + kx;
        }
        float k[FPL], v[FPL];
        BfVec<FPL>::load(qkv + (size_t)kr * D3 + D + lane * FPL, k);
        BfVec<FPL>::load(qkv + (size_t)kr * D3 + 2 * D + lane * FPL, v);
        float p = 0.f;
#pragma unroll
        for (int i = 0; i < FPL; i++) p = fmaf(q[i], k[i], p);
        for (int o = 1; o < lph; o <<= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
        const float s = p * scale;
        const float mn = fmaxf(m, s);
        const float c = __expf(m - mn), e = __expf(s - mn);
        l = l * c + e;
#pragma unroll
        for (int i = 0; i < FPL; i++) acc[i] = acc[i] * c + e * v[i];
        m = mn;
    }
    const float inv = 1.0f / l;
#pragma unroll
    for (int i = 0; i < FPL; i++) acc[i] *= inv;
    BfVec<FPL>::store(out + (size_t)r * D + lane * FPL, acc);
}

// Radius-1 stencil (3 x 3 candidates, any dilation), unrolled: the nine key
// and value vectors are loaded up front as packed bf16 words, then scores,
// max, exp, denominator and the (e / denom)-weighted sum follow the
// reference's order (cpu.rs:121-158).
template <int FPL>
__global__ void __launch_bounds__(256) bf_attention_r1_kernel(Dims d, const bf16* __restrict__ qkv,
                                                              const InstDev* inst, int n_inst, int R,
                                                              bf16* __restrict__ out) {
    constexpr int W = FPL / 2 > 0 ? FPL / 2 : 1;  // 32-bit words per lane per vector
    const int lane = threadIdx.x & 31;
    const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (r >= R) return;
    const int D = d.D, D3 = 3 * D;
    const int lph = 32 / d.heads;
    const InstDev& I = inst[inst_of_row(inst, n_inst, r)];
    const int t = r - I.row0, qy = t / I.tx, qx = t % I.tx, dil = d.dilation;
    const float scale = 1.0f / sqrtf((float)(D / d.heads));
    float q[FPL];
    BfVec<FPL>::load(qkv + (size_t)r * D3 + lane * FPL, q);
    uint32_t kw[9][W], vw[9][W];
    bool in[9];
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const int ky = qy + (j / 3 - 1) * dil, kx = qx + (j % 3 - 1) * dil;
        in[j] = ky >= 0 && kx >= 0 && ky < I.ty && kx < I.tx;
        const size_t kr = in[j] ? (size_t)(I.row0 + ky * I.tx + kx) : (size_t)r;
        const bf16* kp = qkv + kr * D3 + D + lane * FPL;
        const bf16* vp = kp + D;
        if (FPL == 1) {
            kw[j][0] = *reinterpret_cast<const uint16_t*>(kp);
            vw[j][0] = *reinterpret_cast<const uint16_t*>(vp);
        } else if (FPL == 4) {
            const uint2 a = *reinterpret_cast<const uint2*>(kp), b = *reinterpret_cast<const uint2*>(vp);
            kw[j][0] = a.x; kw[j][W > 1 ? 1 : 0] = a.y;
            vw[j][0] = b.x; vw[j][W > 1 ? 1 : 0] = b.y;
        } else {
            const uint4 a = *reinterpret_cast<const uint4*>(kp), b = *reinterpret_cast<const uint4*>(vp);
            const uint32_t aw[4] = {a.x, a.y, a.z, a.w}, bw[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < W; i++) { kw[j][i] = aw[i]; vw[j][i] = bw[i]; }
        }
    }
    auto unpack = [&](const uint32_t* w, float* f) {
        if (FPL == 1) {
            f[0] = __uint_as_float(w[0] << 16);
        } else {
#pragma unroll
            for (int i = 0; i < W; i++) {
                f[2 * i] = __uint_as_float(w[i] << 16);
                f[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
            }
        }
    };
    float sc[9];
    float smax = -INFINITY;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        float k[FPL];
        unpack(kw[j], k);
        float p = 0.f;
#pragma unroll
        for (int i = 0; i < FPL; i++) p = fmaf(q[i], k[i], p);
        for (int o = 1; o < lph; o <<= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
        sc[j] = p * scale;
        if (in[j]) smax = fmaxf(smax, sc[j]);
    }
    float denom = 0.f;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        sc[j] = in[j] ? __expf(sc[j] - smax) : 0.f;
        denom += sc[j];
    }
    const float inv = 1.0f / denom;
    float acc[FPL];
#pragma unroll
    for (int i = 0; i < FPL; i++) acc[i] = 0.f;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        float v[FPL];
        unpack(vw[j], v);
        const float wn = sc[j] * inv;
#pragma unroll
        for (int i = 0; i < FPL; i++) acc[i] = fmaf(wn, v[i], acc[i]);
    }
    BfVec<FPL>::store(out + (size_t)r * D + lane * FPL, acc);
}

// z0 (f32 [rows, HD]) -> zc (bf16 [cells, 48]): upsample along y then x
// (cpu.rs:211-245), state channels appended (cpu.rs:339-342), zero padding.
__global__ void bf_upsample_kernel(Dims d, const float* __restrict__ z0, const InstDev* inst, int n_inst,
                                   long long NC, bf16* __restrict__ zc) {
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
    const float uy = 1.0f - wy, ux = 1.0f - wx;
    float vals[kZcCh];
#pragma unroll
    for (int i = 0; i < kZcCh; i++) vals[i] = 0.f;
    for (int q = 0; q < d.HD / 4; q++) {
        float4 A = a[q], B = b[q], Cc = c[q], E = e[q];
        vals[4 * q + 0] = (A.x * uy + Cc.x * wy) * ux + (B.x * uy + E.x * wy) * wx;
        vals[4 * q + 1] = (A.y * uy + Cc.y * wy) * ux + (B.y * uy + E.y * wy) * wx;
        vals[4 * q + 2] = (A.z * uy + Cc.z * wy) * ux + (B.z * uy + E.z * wy) * wx;
        vals[4 * q + 3] = (A.w * uy + Cc.w * wy) * ux + (B.w * uy + E.w * wy) * wx;
    }
    const size_t plane = (size_t)I.nx * I.ny;
    for (int ch = 0; ch < d.C; ch++) {
        const float sv = I.state[ch * plane + cl];
        const float hi = bf2f(__float2bfloat16(sv));
        vals[kZcState + ch] = hi;
        vals[kZcState + 3 + ch] = sv - hi;  // exact in f32; rounded to bf16 below
        vals[kZcState + 6 + ch] = hi;
    }
    uint4* o = reinterpret_cast<uint4*>(zc + (size_t)cell * kZcCh);
#pragma unroll
    for (int q = 0; q < kZcCh / 8; q++) {
        uint32_t w[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            __nv_bfloat162 h = __floats2bfloat162_rn(vals[8 * q + 2 * i], vals[8 * q + 2 * i + 1]);
            w[i] = *reinterpret_cast<uint32_t*>(&h);
        }
        o[q] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// ---------------------------------------------------------------------------
// tensor-core kernels

// Epilogue helpers: thread (warp w, lane) owns TMEM lane 32 w + lane = tile row.
__device__ __forceinline__ uint32_t lane_addr(uint32_t tmem) {
    return tmem + (((threadIdx.x >> 5) & 3u) * 32u << 16);
}

__device__ __forceinline__ void store_bf16x16(bf16* p, const float* v) {
    BfVec<8>::store(p, v);
    BfVec<8>::store(p + 8, v + 8);
}

// Exact-form GELU, 0.5 x (1 + erf(x / sqrt 2)), with erf from Abramowitz &
// Stegun 7.1.26 (|error| <= 1.5e-7 for the formula; the reciprocal and
// exponential use the hardware approximations). Used where the result is
// rounded to bf16 or feeds bf16 arithmetic.
__device__ __forceinline__ float gelu_fast(float x) {
    const float z = fabsf(x) * 0.70710678118654752440f;
    const float t = __fdividef(1.0f, fmaf(0.3275911f, z, 1.0f));
    const float poly =
        t * fmaf(t, fmaf(t, fmaf(t, fmaf(t, 1.061405429f, -1.453152027f), 1.421413741f), -0.284496736f), 0.254829592f);
    const float erf_abs = 1.0f - poly * __expf(-z * z);
    const float erf_x = copysignf(erf_abs, x);
    return 0.5f * x * (1.0f + erf_x);
}

__device__ __forceinline__ int slot_swz(int r, int D) { return D >= 128 ? (r & 31) : (r & (D / 4 - 1)); }

// Stage columns [c0, c1) of this thread's TMEM lane (tile row `r`) into the
// shared f32 tile [128][D]; float4 slot q of row r is stored at slot
// q ^ slot_swz(r, D), which keeps both the row-per-thread writes here and the
// row-per-warp reads below free of bank conflicts.
__device__ __forceinline__ void stage_rows(uint32_t ta, int r, int D, int c0, int c1, float* tile) {
    for (int c = c0; c < c1; c += 16) {
        float a[16];
        tc::tmem_ld16(ta + c, a);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int q = c / 4 + i;
            reinterpret_cast<float4*>(tile + (size_t)r * D)[q ^ slot_swz(r, D)] =
                make_float4(a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]);
        }
    }
}

// One warp per tile row: x[row] += acc + bias, then LayerNorm of the new row
// (two-pass mean and biased variance, eps 1e-5) into `ln` as bf16. Lane l
// handles float4 slots l + 32 j, so x and ln are read and written coalesced.
template <int SPL>  // float4 slots per lane: D / 128
__device__ void rows_resid_ln(const float* tile, int D, int m0, int R, const float* __restrict__ bias,
                              float* __restrict__ x, const float* __restrict__ g, const float* __restrict__ b,
                              bf16* __restrict__ ln, int warp, int nwarps) {
    const int lane = threadIdx.x & 31;
    float4 bb[SPL], gg[SPL], be[SPL];
#pragma unroll
    for (int j = 0; j < SPL; j++) {
        const int q = lane + 32 * j;
        bb[j] = reinterpret_cast<const float4*>(bias)[q];
        gg[j] = reinterpret_cast<const float4*>(g)[q];
        be[j] = reinterpret_cast<const float4*>(b)[q];
    }
    constexpr int G = 4;  // rows in flight per warp
    for (int r0 = warp * G; r0 < 128; r0 += nwarps * G) {
        float4 a[G][SPL], xv[G][SPL];
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int r = r0 + k, row = m0 + r;
#pragma unroll
            for (int j = 0; j < SPL; j++) {
                const int q = lane + 32 * j;
                a[k][j] = reinterpret_cast<const float4*>(tile + (size_t)r * D)[q ^ (r & 31)];
                xv[k][j] = row < R ? reinterpret_cast<const float4*>(x + (size_t)row * D)[q] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int row = m0 + r0 + k;
            if (row >= R) break;
            float4 v[SPL];
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < SPL; j++) {
                v[j] = make_float4(xv[k][j].x + (a[k][j].x + bb[j].x), xv[k][j].y + (a[k][j].y + bb[j].y),
                                   xv[k][j].z + (a[k][j].z + bb[j].z), xv[k][j].w + (a[k][j].w + bb[j].w));
                s += (v[j].x + v[j].y) + (v[j].z + v[j].w);
            }
            const float mean = warp_sum(s) / (float)D;
            float q2 = 0.f;
#pragma unroll
            for (int j = 0; j < SPL; j++) {
                const float e0 = v[j].x - mean, e1 = v[j].y - mean, e2 = v[j].z - mean, e3 = v[j].w - mean;
                q2 += (e0 * e0 + e1 * e1) + (e2 * e2 + e3 * e3);
            }
            const float rstd = 1.0f / sqrtf(warp_sum(q2) / (float)D + 1e-5f);
#pragma unroll
            for (int j = 0; j < SPL; j++) {
                const int q = lane + 32 * j;
                reinterpret_cast<float4*>(x + (size_t)row * D)[q] = v[j];
                float o[4] = {(v[j].x - mean) * rstd * gg[j].x + be[j].x, (v[j].y - mean) * rstd * gg[j].y + be[j].y,
                              (v[j].z - mean) * rstd * gg[j].z + be[j].z, (v[j].w - mean) * rstd * gg[j].w + be[j].w};
                BfVec<4>::store(ln + (size_t)row * D + 4 * q, o);
            }
        }
    }
}

// D-dispatch of rows_resid_ln (D = 128 SPL 1, 256 SPL 2; D = 32 uses the
// first 8 lanes of one slot each).
__device__ void rows_resid_ln_any(const float* tile, int D, int m0, int R, const float* bias, float* x,
                                  const float* g, const float* b, bf16* ln, int warp, int nwarps) {
    if (D == 256) rows_resid_ln<2>(tile, D, m0, R, bias, x, g, b, ln, warp, nwarps);
    else if (D == 128) rows_resid_ln<1>(tile, D, m0, R, bias, x, g, b, ln, warp, nwarps);
    else {
        // narrow rows (D = 32): lanes 0..7 each own one float4 slot
        const int lane = threadIdx.x & 31;
        for (int r = warp; r < 128; r += nwarps) {
            const int row = m0 + r;
            if (row >= R) break;
            const bool on = lane < D / 4;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (on) {
                const float4 a = reinterpret_cast<const float4*>(tile + (size_t)r * D)[lane ^ (r & (D / 4 - 1))];
                const float4 xv = reinterpret_cast<const float4*>(x + (size_t)row * D)[lane];
                const float4 bb = reinterpret_cast<const float4*>(bias)[lane];
                v = make_float4(xv.x + (a.x + bb.x), xv.y + (a.y + bb.y), xv.z + (a.z + bb.z), xv.w + (a.w + bb.w));
            }
            const float mean = warp_sum((v.x + v.y) + (v.z + v.w)) / (float)D;
            float q2 = 0.f;
            if (on) q2 = (v.x - mean) * (v.x - mean) + (v.y - mean) * (v.y - mean) + (v.z - mean) * (v.z - mean) +
                         (v.w - mean) * (v.w - mean);
            const float rstd = 1.0f / sqrtf(warp_sum(q2) / (float)D + 1e-5f);
            if (on) {
                const float4 gg = reinterpret_cast<const float4*>(g)[lane], be = reinterpret_cast<const float4*>(b)[lane];
                reinterpret_cast<float4*>(x + (size_t)row * D)[lane] = v;
                float o[4] = {(v.x - mean) * rstd * gg.x + be.x, (v.y - mean) * rstd * gg.y + be.y,
                              (v.z - mean) * rstd * gg.z + be.z, (v.w - mean) * rstd * gg.w + be.w};
                BfVec<4>::store(ln + (size_t)row * D + 4 * lane, o);
            }
        }
    }
}

enum { EPI_BF16 = 0, EPI_F32 = 1, EPI_RESID_LN = 2 };

struct GemmEpi {
    const float* bias;
    bf16* out_bf;    // EPI_BF16 / EPI_RESID_LN (LayerNorm output)
    float* out_f;    // EPI_F32
    float* x;        // EPI_RESID_LN residual stream
    const float* g;  // EPI_RESID_LN LayerNorm
    const float* b;
    int ldo;         // output row stride (elements)
};

// C[128-row tile, BN-column block] = A[rows, K] @ B^T. A via TMA (8-column
// boxes), B (one pre-arranged [K/8][BN][8] block) via a bulk copy; all of K
// is staged at once (K <= 512), one thread issues the MMAs, four warps run
// the epilogue from TMEM.
template <int EPI>
__global__ void __launch_bounds__(128) tc_gemm_kernel(const __grid_constant__ CUtensorMap tmA,
                                                      const bf16* __restrict__ Bblk, int K, int BN, int R,
                                                      GemmEpi ep, int* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;                       // [K/8][128][8]
    uint8_t* sB = smem + (size_t)K * 256;     // [K/8][BN][8]
    __shared__ uint64_t bar_load, bar_mma;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    const int warp = threadIdx.x >> 5;
    const int m0 = blockIdx.x * 128, nb = blockIdx.y;
    const uint32_t ncols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar_load, 1);
        tc::mbar_init(&bar_mma, 1);
        tc::fence_barrier_init();
        failed = 0;
        if (tc::smem_u32(smem) & 1023u) {  // operand tiles need aligned shared memory
            failed = 1;
            atomicExch(err, 2);
        }
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    if (threadIdx.x == 0 && !failed) {
        const uint32_t bytes_b = (uint32_t)K * BN * 2;
        tc::mbar_expect_tx(&bar_load, (uint32_t)K * 256 + bytes_b);
        for (int kc = 0; kc < K / 8; kc++) tc::tma_load_2d(sA + kc * 2048, &tmA, kc * 8, m0, &bar_load);
        tc::bulk_load(sB, Bblk + (size_t)nb * K * BN, bytes_b, &bar_load);
        if (tc::mbar_wait(&bar_load, 0, err, &failed)) {
            tc::tc_fence_after();
            const uint32_t idesc = tc::idesc_bf16(128, BN);
            const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
            for (int k = 0; k < K / 16; k++) {
                uint64_t ad = tc::sdesc(a0 + k * 4096, 2048, 128);
                uint64_t bd = tc::sdesc(b0 + k * 2 * BN * 16, BN * 16, 128);
                tc::mma_bf16(tmem, ad, bd, idesc, k > 0 ? 1u : 0u);
            }
            tc::mma_commit(&bar_mma);
        }
    }
    __syncwarp();
    const bool ok = __syncthreads_and(tc::mbar_wait(&bar_mma, 0, err, &failed) ? 1 : 0) != 0;
    tc::tc_fence_after();
    if (ok) {
        const int row = m0 + threadIdx.x;
        const uint32_t ta = lane_addr(tmem);
        const int n0 = nb * BN;
        if (EPI == EPI_RESID_LN) {
            // every MMA and TMA write is complete: the operand tiles' shared
            // memory now holds the f32 accumulator tile
            float* tile = reinterpret_cast<float*>(smem);
            stage_rows(ta, threadIdx.x, BN, 0, BN, tile);
            __syncthreads();
            rows_resid_ln_any(tile, BN, m0, R, ep.bias, ep.x, ep.g, ep.b, ep.out_bf, warp, 4);
        } else {
            for (int c = 0; c < BN; c += 16) {
                float a[16];
                tc::tmem_ld16(ta + c, a);  // collective: every lane of the warp loads
                if (row < R) {
#pragma unroll
                    for (int i = 0; i < 16; i++) a[i] += ep.bias[n0 + c + i];
                    if (EPI == EPI_BF16) {
                        store_bf16x16(ep.out_bf + (size_t)row * ep.ldo + n0 + c, a);
                    } else {
                        float4* o = reinterpret_cast<float4*>(ep.out_f + (size_t)row * ep.ldo + n0 + c);
#pragma unroll
                        for (int i = 0; i < 4; i++) o[i] = make_float4(a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]);
                    }
                }
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// Fused MLP: x += gelu(LN2(x) @ W1 + b1) @ W2 + b2, then LayerNorm of the new
// x (the next block's norm1, or the final norm) into `ln`. Per chunk of NC
// hidden columns: S = A @ W1_chunk (TMEM), h = gelu(S + b1) written to
// shared memory as bf16 by all 8 warps (two per TMEM lane quarter, one
// column half each), O += h @ W2_chunk (TMEM). The hidden activations never
// leave the SM. The residual + LayerNorm epilogue stages O through shared
// memory and runs one warp per row.
constexpr int kMlpThreads = 256;

__global__ void __launch_bounds__(kMlpThreads) tc_mlp_kernel(const __grid_constant__ CUtensorMap tmA,
                                                             const bf16* __restrict__ W1, const bf16* __restrict__ W2,
                                                             const float* __restrict__ b1,
                                                             const float* __restrict__ b2, int D, int F, int NC, int R,
                                                             float* __restrict__ x, const float* __restrict__ g,
                                                             const float* __restrict__ b, bf16* __restrict__ ln,
                                                             int* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;                           // [D/8][128][8]
    uint8_t* sB1 = sA + (size_t)D * 256;          // [D/8][NC][8]
    uint8_t* sB2 = sB1 + (size_t)D * NC * 2;      // [NC/8][D][8]
    uint8_t* sH = sB2 + (size_t)D * NC * 2;       // [NC/8][128][8]
    __shared__ float sb1[1024];
    __shared__ uint64_t bar_a, bar_w, bar_s, bar_o;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quarter = warp & 3, half = warp >> 2;
    const int m0 = blockIdx.x * 128;
    const uint32_t ncols = D <= 128 ? 256 : 512;
    const uint32_t s_col = D <= 128 ? 128 : 256;  // O in [0, D), S in [s_col, s_col + NC)
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar_a, 1);
        tc::mbar_init(&bar_w, 1);
        tc::mbar_init(&bar_s, 1);
        tc::mbar_init(&bar_o, 1);
        tc::fence_barrier_init();
        failed = 0;
        if (tc::smem_u32(smem) & 1023u) {  // operand tiles need aligned shared memory
            failed = 1;
            atomicExch(err, 2);
        }
    }
    for (int i = threadIdx.x; i < F; i += blockDim.x) sb1[i] = b1[i];
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tO = tmem_base, tS = tmem_base + s_col;
    const uint32_t a0 = tc::smem_u32(sA), w1s = tc::smem_u32(sB1), w2s = tc::smem_u32(sB2), hs = tc::smem_u32(sH);
    if (threadIdx.x == 0 && !failed) {
        tc::mbar_expect_tx(&bar_a, (uint32_t)D * 256);
        for (int kc = 0; kc < D / 8; kc++) tc::tma_load_2d(sA + kc * 2048, &tmA, kc * 8, m0, &bar_a);
    }
    const int nchunks = F / NC;
    const uint32_t wbytes = (uint32_t)D * NC * 2;
    bool ok = true;
    for (int j = 0; j < nchunks && ok; j++) {
        if (threadIdx.x == 0 && !failed) {
            tc::mbar_expect_tx(&bar_w, 2 * wbytes);
            tc::bulk_load(sB1, W1 + (size_t)j * D * NC, wbytes, &bar_w);
            tc::bulk_load(sB2, W2 + (size_t)j * D * NC, wbytes, &bar_w);
            bool good = (j > 0 || tc::mbar_wait(&bar_a, 0, err, &failed)) && tc::mbar_wait(&bar_w, j & 1, err, &failed);
            if (good) {
                tc::tc_fence_after();
                const uint32_t idesc = tc::idesc_bf16(128, NC);
                for (int k = 0; k < D / 16; k++)
                    tc::mma_bf16(tS, tc::sdesc(a0 + k * 4096, 2048, 128), tc::sdesc(w1s + k * 2 * NC * 16, NC * 16, 128),
                                 idesc, k > 0 ? 1u : 0u);
                tc::mma_commit(&bar_s);
            }
        }
        __syncwarp();
        ok = __syncthreads_and(tc::mbar_wait(&bar_s, j & 1, err, &failed) ? 1 : 0) != 0;
        tc::tc_fence_after();
        if (!ok) break;
        {
            // h = gelu(S + b1) -> bf16 -> shared memory in the core-matrix layout
            const int r = quarter * 32 + lane;
            const uint32_t ta = lane_addr(tS);
            const int c0 = half * (NC / 2), c1 = c0 + NC / 2;
            for (int c = c0; c < c1; c += 16) {
                float a[16];
                tc::tmem_ld16(ta + c, a);
#pragma unroll
                for (int i = 0; i < 16; i++) a[i] = gelu_fast(a[i] + sb1[j * NC + c + i]);
                BfVec<8>::store(reinterpret_cast<bf16*>(sH + (size_t)(c / 8) * 2048 + r * 16), a);
                BfVec<8>::store(reinterpret_cast<bf16*>(sH + (size_t)(c / 8 + 1) * 2048 + r * 16), a + 8);
            }
        }
        tc::fence_async_shared();
        tc::tc_fence_before();
        __syncthreads();
        tc::tc_fence_after();
        if (threadIdx.x == 0 && !failed) {
            const uint32_t idesc = tc::idesc_bf16(128, D);
            for (int k = 0; k < NC / 16; k++)
                tc::mma_bf16(tO, tc::sdesc(hs + k * 4096, 2048, 128), tc::sdesc(w2s + k * 2 * D * 16, D * 16, 128), idesc,
                             (j > 0 || k > 0) ? 1u : 0u);
            tc::mma_commit(&bar_o);
        }
        __syncwarp();
        ok = __syncthreads_and(tc::mbar_wait(&bar_o, j & 1, err, &failed) ? 1 : 0) != 0;
        tc::tc_fence_after();
    }
    if (ok) {
        // every MMA is complete: reuse the operand shared memory for the f32 O tile
        float* tile = reinterpret_cast<float*>(smem);
        stage_rows(lane_addr(tO), quarter * 32 + lane, D, half * (D / 2), (half + 1) * (D / 2), tile);
        __syncthreads();
        rows_resid_ln_any(tile, D, m0, R, b2, x, g, b, ln, warp, kMlpThreads / 32);
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem_base, ncols);
}

// 3x3 zero-padded convolution over each instance's grid as an implicit GEMM
// (cpu.rs:171-205): tile = 8 x 16 positions (M = 128, row r <-> position
// (y0 + r/8, x0 + r%8)); the halo tile [C/8 planes][18][10][8] is loaded by
// TMA (zero fill outside the grid); tap (ky, kx) is the halo addressed from
// offset (ky*10 + kx)*16 bytes. B per tap: [C/8][BN][8] (the N block `nb`).
// Epilogues: TOKMIX: out = xn + gelu(acc + b) (cpu.rs:326-328), bf16;
//            CONV1:  out = gelu(acc + b)      (cpu.rs:345-346), f32.
enum { CONV_TOKMIX = 0, CONV_CELL1 = 1 };

template <int KIND>
__global__ void __launch_bounds__(128) tc_conv3_kernel(const CUtensorMap* __restrict__ maps, int map_slot,
                                                       const bf16* __restrict__ Wt, const float* __restrict__ bias,
                                                       int C, int BN, int N, const InstDev* inst, int n_inst,
                                                       void* __restrict__ out, int* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sHalo = smem;                                   // [C/8][18][10][8]
    uint8_t* sB = smem + (size_t)(C / 8) * kHaloPlane;       // 2 x [C/8][BN][8]
    __shared__ uint64_t bar_h, bar_b[2], bar_m[2], bar_done;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    const int warp = threadIdx.x >> 5;
    // tile -> instance
    const int tile = blockIdx.x, nb = blockIdx.y;
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        int t0 = KIND == CONV_TOKMIX ? inst[mid].tt0 : inst[mid].ct0;
        if (t0 <= tile) lo = mid; else hi = mid - 1;
    }
    const InstDev& I = inst[lo];
    const int gw = KIND == CONV_TOKMIX ? I.tx : I.nx, gh = KIND == CONV_TOKMIX ? I.ty : I.ny;
    const int tiles_x = (gw + kConvTX - 1) / kConvTX;
    const int tl = tile - (KIND == CONV_TOKMIX ? I.tt0 : I.ct0);
    const int x0 = (tl % tiles_x) * kConvTX, y0 = (tl / tiles_x) * kConvTY;
    const CUtensorMap* map = maps + 2 * lo + map_slot;
    const uint32_t ncols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar_h, 1);
        tc::mbar_init(&bar_done, 1);
        for (int i = 0; i < 2; i++) {
            tc::mbar_init(&bar_b[i], 1);
            tc::mbar_init(&bar_m[i], 1);
        }
        tc::fence_barrier_init();
        failed = 0;
        if (tc::smem_u32(smem) & 1023u) {  // operand tiles need aligned shared memory
            failed = 1;
            atomicExch(err, 2);
        }
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t wtap = (uint32_t)C * BN * 2;  // bytes of one tap's B block
    const bf16* Wn = Wt + (size_t)nb * 9 * C * BN;
    if (threadIdx.x == 0 && !failed) {
        tc::tensormap_acquire(map);
        tc::mbar_expect_tx(&bar_h, (uint32_t)(C / 8) * (kHaloW * kHaloH * 16));
        for (int kc = 0; kc < C / 8; kc++)
            tc::tma_load_3d(sHalo + kc * kHaloPlane, map, kc * 8, x0 - 1, y0 - 1, &bar_h);
        for (int t = 0; t < 2; t++) {
            tc::mbar_expect_tx(&bar_b[t], wtap);
            tc::bulk_load(sB + t * wtap, Wn + (size_t)t * C * BN, wtap, &bar_b[t]);
        }
        bool good = tc::mbar_wait(&bar_h, 0, err, &failed);
        const uint32_t idesc = tc::idesc_bf16(128, BN);
        const uint32_t h0 = tc::smem_u32(sHalo);
        for (int t = 0; t < 9 && good; t++) {
            const int buf = t & 1;
            good = tc::mbar_wait(&bar_b[buf], (t >> 1) & 1, err, &failed);
            if (!good) break;
            tc::tc_fence_after();
            const int ky = t / 3, kx = t % 3;
            const uint32_t b0 = tc::smem_u32(sB + buf * wtap);
            for (int k = 0; k < C / 16; k++) {
                uint64_t ad = tc::sdesc(h0 + 2 * k * kHaloPlane + (ky * kHaloW + kx) * 16, kHaloPlane, kHaloW * 16);
                uint64_t bd = tc::sdesc(b0 + 2 * k * BN * 16, BN * 16, 128);
                tc::mma_bf16(tmem, ad, bd, idesc, (t > 0 || k > 0) ? 1u : 0u);
            }
            tc::mma_commit(&bar_m[buf]);
            if (t + 2 < 9) {
                // the buffer is refilled once the MMAs reading it are done
                good = tc::mbar_wait(&bar_m[buf], (t >> 1) & 1, err, &failed);
                if (!good) break;
                tc::mbar_expect_tx(&bar_b[buf], wtap);
                tc::bulk_load(sB + buf * wtap, Wn + (size_t)(t + 2) * C * BN, wtap, &bar_b[buf]);
            }
        }
        if (good) tc::mma_commit(&bar_done);  // arrives when every MMA above is done
    }
    __syncwarp();
    const bool ok = __syncthreads_and(tc::mbar_wait(&bar_done, 0, err, &failed) ? 1 : 0) != 0;
    tc::tc_fence_after();
    if (ok) {
        const int r = threadIdx.x;
        const int y = y0 + r / kConvTX, x = x0 + r % kConvTX;
        const bool valid = y < gh && x < gw;
        const uint32_t ta = lane_addr(tmem);
        const int n0 = nb * BN;
        const long long pos = KIND == CONV_TOKMIX ? (long long)I.row0 + (long long)y * gw + x
                                                  : I.cell0 + (long long)y * gw + x;
        for (int c = 0; c < BN; c += 16) {
            float a[16];
            tc::tmem_ld16(ta + c, a);
            if (!valid) continue;
            if (KIND == CONV_TOKMIX) {
                // the centre of the halo tile is xn at this token
                const uint8_t* centre = sHalo + ((r / kConvTX + 1) * kHaloW + (r % kConvTX + 1)) * 16;
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int ch = n0 + c + i;
                    const float xn = bf2f(*reinterpret_cast<const bf16*>(centre + (size_t)(ch / 8) * kHaloPlane + (ch % 8) * 2));
                    a[i] = xn + gelu_fast(a[i] + bias[ch]);
                }
                store_bf16x16(static_cast<bf16*>(out) + (size_t)pos * N + n0 + c, a);
            } else {
#pragma unroll
                for (int i = 0; i < 16; i++) a[i] = gelu_fast(a[i] + bias[n0 + c + i]);
                float4* o = reinterpret_cast<float4*>(static_cast<float*>(out) + (size_t)pos * N + n0 + c);
#pragma unroll
                for (int i = 0; i < 4; i++) o[i] = make_float4(a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]);
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------
// host

static const bf16* upload_bf16(DeviceArena& a, const std::vector<uint16_t>& v) {
    void* d = a.alloc(v.size() * 2);
    cuda_check(cudaMemcpy(d, v.data(), v.size() * 2, cudaMemcpyHostToDevice), "upload weights", JC_MAP);
    return static_cast<const bf16*>(d);
}

// B[n][k] for n < N, k < K into [N/BN][K/8][BN][8].
static std::vector<uint16_t> blocked(int N, int K, int BN, const std::function<float(int, int)>& f) {
    std::vector<uint16_t> out((size_t)N * K);
    size_t i = 0;
    for (int nb = 0; nb < N / BN; nb++)
        for (int kc = 0; kc < K / 8; kc++)
            for (int n = 0; n < BN; n++)
                for (int e = 0; e < 8; e++) out[i++] = f2bf(f(nb * BN + n, kc * 8 + e));
    return out;
}

static const HostTensor& tget(const TensorMap& t, const std::string& n) {
    auto it = t.find(n);
    if (it == t.end()) throw Error(JC_BAD_CHECKPOINT, "missing tensor `" + n + "`");
    return it->second;
}

template <class K>
static void set_smem(K kernel, size_t bytes) {
    cuda_check(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes),
               "cudaFuncSetAttribute");
}

BF16Path::BF16Path(const Dims& d, const TensorMap& t, DeviceArena& arena) {
    const int D = d.D, F = d.F, HD = d.HD;
    if (D % 32 || D > 256 || 32 % d.heads || F % 64 || HD != 32 || d.C != 3 || d.P != 4 || d.C * d.P * d.P > 64)
        throw Error(JC_LIMIT,
                    "the BF16 path needs dim a multiple of 32 and <= 256, heads dividing 32, a cell-head width of 32, "
                    "3 channels and patch 4");
    nc_mlp = 64;
    n_nc = (D <= 128 && F % 128 == 0) ? 2 : 1;  // nc 128 needs 128 KB of shared memory at dim 128
    bn_qkv = (3 * D) % 128 == 0 ? 128 : 3 * D;
    bn_tm = D <= 128 ? D : 64;
    if (F % nc_mlp) throw Error(JC_LIMIT, "the MLP width must be a multiple of the MLP chunk");
    for (int l = 0; l < d.L; l++) {
        const std::string p = "blocks." + std::to_string(l) + ".";
        const auto &q = tget(t, p + "q.weight").data, &k = tget(t, p + "k.weight").data, &v = tget(t, p + "v.weight").data;
        // B[n][k] = Wqkv[k][n]: q | k | v along n
        wqkv[l] = upload_bf16(arena, blocked(3 * D, D, bn_qkv, [&](int n, int kk) {
                                  const auto& w = n < D ? q : (n < 2 * D ? k : v);
                                  return w[(size_t)kk * D + (n % D)];
                              }));
        const auto& wpr = tget(t, p + "proj.weight").data;
        wp[l] = upload_bf16(arena, blocked(D, D, D, [&](int n, int kk) { return wpr[(size_t)kk * D + n]; }));
        const auto& w1h = tget(t, p + "ff1.weight").data;  // [D, F]
        const auto& w2h = tget(t, p + "ff2.weight").data;  // [F, D]
        for (int v = 0; v < n_nc; v++) {
            const int nc = v == 0 ? 64 : 128;
            w1v[v][l] = upload_bf16(arena, blocked(F, D, nc, [&](int n, int kk) { return w1h[(size_t)kk * F + n]; }));
            // W2 chunk j: B2_j[n][k] = W2[j*nc + k][n] -> [j][nc/8][D][8]
            std::vector<uint16_t> w2b((size_t)F * D);
            size_t i = 0;
            for (int j = 0; j < F / nc; j++)
                for (int kc = 0; kc < nc / 8; kc++)
                    for (int n = 0; n < D; n++)
                        for (int e = 0; e < 8; e++) w2b[i++] = f2bf(w2h[(size_t)(j * nc + kc * 8 + e) * D + n]);
            w2v[v][l] = upload_bf16(arena, w2b);
        }
    }
    {
        // token_mix: per N block of 128 (or D) and tap: [C/8][BN][8] of W[co][ci][ky][kx]
        const auto& w = tget(t, "head.token_mix.weight").data;
        const int BN = bn_tm;
        std::vector<uint16_t> o((size_t)9 * D * D);
        size_t i = 0;
        for (int nb = 0; nb < D / BN; nb++)
            for (int tap = 0; tap < 9; tap++)
                for (int kc = 0; kc < D / 8; kc++)
                    for (int n = 0; n < BN; n++)
                        for (int e = 0; e < 8; e++)
                            o[i++] = f2bf(w[((size_t)(nb * BN + n) * D + kc * 8 + e) * 9 + tap]);
        wtm = upload_bf16(arena, o);
    }
    {
        const auto& w = tget(t, "head.to_cells.weight").data;  // [HD][D]
        wtc = upload_bf16(arena, blocked(HD, D, HD, [&](int n, int kk) { return w[(size_t)n * D + kk]; }));
    }
    {
        // conv1: per tap [48/8][32][8] over the zc channels: z (32), then the
        // state's [hi, lo, hi] parts with weights [W_hi, W_hi, W_lo]
        const auto& w = tget(t, "head.conv1.weight").data;  // [HD][HD+C][3][3]
        const int cin = HD + d.C;
        auto bf_round = [](float v) {
            uint32_t u = (uint32_t)f2bf(v) << 16;
            float r;
            std::memcpy(&r, &u, 4);
            return r;
        };
        std::vector<uint16_t> o((size_t)9 * kZcCh * HD);
        size_t i = 0;
        for (int tap = 0; tap < 9; tap++)
            for (int kc = 0; kc < kZcCh / 8; kc++)
                for (int n = 0; n < HD; n++)
                    for (int e = 0; e < 8; e++) {
                        const int ch = kc * 8 + e;
                        float v = 0.0f;
                        if (ch < HD) {
                            v = w[((size_t)n * cin + ch) * 9 + tap];
                        } else if (ch < kZcState + 9) {
                            const int part = (ch - kZcState) / 3, c = (ch - kZcState) % 3;
                            const float full = w[((size_t)n * cin + HD + c) * 9 + tap];
                            const float hi = bf_round(full);
                            v = part < 2 ? hi : full - hi;
                        }
                        o[i++] = f2bf(v);
                    }
        wc1 = upload_bf16(arena, o);
    }
    cache_key_ = "d" + std::to_string(D) + "_l" + std::to_string(d.L) + "_f" + std::to_string(F) + "_r" +
                 std::to_string(d.radius) + "_k" + std::to_string(d.mask_kind) + "_g" + std::to_string(d.dilation);
    load_cache();
    set_smem(tc_gemm_kernel<EPI_BF16>, 200 * 1024);
    set_smem(tc_gemm_kernel<EPI_F32>, 200 * 1024);
    set_smem(tc_gemm_kernel<EPI_RESID_LN>, 200 * 1024);
    set_smem(tc_mlp_kernel, 200 * 1024);
    set_smem(tc_conv3_kernel<CONV_TOKMIX>, 200 * 1024);
    set_smem(tc_conv3_kernel<CONV_CELL1>, 200 * 1024);
    set_smem(bf_embed_kernel<1>, 100 * 1024);
    set_smem(bf_embed_kernel<4>, 100 * 1024);
    set_smem(bf_embed_kernel<8>, 100 * 1024);
}

static void launch_attention(const Dims& d, const bf16* qkv, const InstDev* inst, int n, int R, bf16* attn,
                             int threads, cudaStream_t s) {
    const int wpb = threads / 32;
    const unsigned blocks = (unsigned)((R + wpb - 1) / wpb);
    const int fpl = d.D / 32;
    const bool r1 = d.mask_kind == 1 && d.radius == 1;
    if (fpl == 1) {
        if (r1) bf_attention_r1_kernel<1><<<blocks, threads, 0, s>>>(d, qkv, inst, n, R, attn);
        else bf_attention_kernel<1><<<blocks, threads, 0, s>>>(d, qkv, inst, n, R, attn);
    } else if (fpl == 4) {
        if (r1) bf_attention_r1_kernel<4><<<blocks, threads, 0, s>>>(d, qkv, inst, n, R, attn);
        else bf_attention_kernel<4><<<blocks, threads, 0, s>>>(d, qkv, inst, n, R, attn);
    } else if (fpl == 8) {
        if (r1) bf_attention_r1_kernel<8><<<blocks, threads, 0, s>>>(d, qkv, inst, n, R, attn);
        else bf_attention_kernel<8><<<blocks, threads, 0, s>>>(d, qkv, inst, n, R, attn);
    } else {
        throw Error(JC_LIMIT, "the BF16 attention supports dim 32, 128 or 256");
    }
}

static int initial_autotune() {
    const char* e = std::getenv("JC_AUTOTUNE");
    return e && std::atoi(e) == 0 ? 0 : 1;
}
std::atomic<int> g_autotune{initial_autotune()};

static int row_bucket(int R) {
    int b = 128;
    while (b < R && b < (1 << 30)) b <<= 1;
    return b;
}

Tuning BF16Path::tuning_for(int rows) const {
    std::lock_guard<std::mutex> lk(tune_mu_);
    if (g_autotune.load()) {
        auto it = tuned_.find(row_bucket(rows));
        if (it != tuned_.end()) return it->second;
    }
    return Tuning{nc_mlp, 256};
}

// Times `launch` with CUDA events: one warm-up, then `reps` launches.
template <class F>
static float time_launches(F&& launch, int reps, cudaStream_t s) {
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    launch();
    cudaEventRecord(a, s);
    for (int i = 0; i < reps; i++) launch();
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / reps;
}

void BF16Path::tune(const Dims& d, const WeightsF32& w, const Pack& p, cudaStream_t s) const {
    if (!g_autotune.load() || p.R == 0) return;
    const int bucket = row_bucket(p.R);
    {
        std::lock_guard<std::mutex> lk(tune_mu_);
        if (tuned_.count(bucket)) return;
    }
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    const int R = p.R, D = d.D;
    bf16* ln = reinterpret_cast<bf16*>(p.bt[0]);
    bf16* qkv = reinterpret_cast<bf16*>(p.bt[1]);
    bf16* attn = reinterpret_cast<bf16*>(p.bt[2]);
    const CUtensorMap m_ln = rows_map(ln, D, R);
    const unsigned gm = (unsigned)((R + 127) / 128);
    Tuning best{nc_mlp, 256};
    // the workspace holds transient values; the timed launches may leave
    // anything in it (every forward rewrites it from the state)
    float best_ms = 1e30f;
    for (int v = 0; v < n_nc; v++) {
        const int NC = v == 0 ? 64 : 128;
        const size_t smem = std::max((size_t)D * 256 + 2 * (size_t)D * NC * 2 + (size_t)NC * 256, (size_t)128 * D * 4);
        const float ms = time_launches(
            [&] {
                tc_mlp_kernel<<<gm, kMlpThreads, smem, s>>>(m_ln, w1v[v][0], w2v[v][0], w.blk[0].b1, w.blk[0].b2, D,
                                                            d.F, NC, R, p.x, w.norm_g, w.norm_b, ln, p.err);
            },
            3, s);
        if (ms < best_ms) {
            best_ms = ms;
            best.nc = NC;
        }
    }
    best_ms = 1e30f;
    for (int threads : {64, 128, 256}) {
        const float ms = time_launches([&] { launch_attention(d, qkv, p.inst, p.n_inst, R, attn, threads, s); }, 3, s);
        if (ms < best_ms) {
            best_ms = ms;
            best.attn_threads = threads;
        }
    }
    cuda_check(cudaGetLastError(), "autotune");
    {
        std::lock_guard<std::mutex> lk(tune_mu_);
        tuned_[bucket] = best;
    }
    save_cache(bucket, best);
}

// Tuned schedules persist in the JSON-lines file named by JC_AUTOTUNE_CACHE,
// one object per tuned row bucket:
//   {"model": "d128_l4_f512_r1_k1_g1", "rows": 65536, "nc": 64, "attn_threads": 128}
// keyed by the model shape (dim, layers, MLP width, mask radius, kind and
// dilation). Lines that do not parse or name another shape are skipped;
// later lines override earlier ones.
void BF16Path::load_cache() {
    const char* path = std::getenv("JC_AUTOTUNE_CACHE");
    if (!path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    char line[512], key[128];
    while (std::fgets(line, sizeof line, f)) {
        int bucket, nc, th;
        if (std::sscanf(line, " {\"model\": \"%127[^\"]\", \"rows\": %d, \"nc\": %d, \"attn_threads\": %d", key,
                        &bucket, &nc, &th) != 4)
            continue;
        if (cache_key_ == key && (nc == 64 || (nc == 128 && n_nc == 2)) && (th == 64 || th == 128 || th == 256))
            tuned_[bucket] = Tuning{nc, th};
    }
    std::fclose(f);
}

void BF16Path::save_cache(int bucket, const Tuning& t) const {
    const char* path = std::getenv("JC_AUTOTUNE_CACHE");
    if (!path) return;
    std::lock_guard<std::mutex> lk(tune_mu_);
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "{\"model\": \"%s\", \"rows\": %d, \"nc\": %d, \"attn_threads\": %d}\n", cache_key_.c_str(), bucket,
                 t.nc, t.attn_threads);
    std::fclose(f);
}

void BF16Path::alloc_workspace(DeviceArena& a, const Dims& d, Pack& p, int rows, long long cells, int max_inst) const {
    const size_t R = (size_t)rows, NC = (size_t)cells;
    const int strides[4] = {d.D * 2, 3 * d.D * 2, d.D * 2, d.D * 2};  // ln, qkv, attn, t1
    for (int i = 0; i < 4; i++) {
        p.bt[i] = static_cast<char*>(a.alloc(R * strides[i] + 256));
        p.bt_stride[i] = strides[i];
    }
    p.bc[0] = static_cast<char*>(a.alloc(NC * kZcCh * 2 + 256));
    p.bc_stride[0] = kZcCh * 2;
    p.bc[1] = static_cast<char*>(a.alloc(NC * d.HD * 4 + 256));  // c1, f32
    p.bc_stride[1] = d.HD * 4;
    p.tmaps = a.alloc((size_t)max_inst * 2 * sizeof(CUtensorMap));
}

void BF16Path::prepare(const Dims& d, const Pack& p, const InstDev* hinst, cudaStream_t s) const {
    std::vector<CUtensorMap> maps((size_t)p.n_inst * 2);
    for (int i = 0; i < p.n_inst; i++) {
        const InstDev& I = hinst[i];
        maps[2 * i + 0] = halo_map(p.bt[0] + (size_t)I.row0 * p.bt_stride[0], d.D, I.tx, I.ty);
        maps[2 * i + 1] = halo_map(p.bc[0] + (size_t)I.cell0 * p.bc_stride[0], kZcCh, I.nx, I.ny);
    }
    // synchronous: the host vector is released on return
    cuda_check(cudaMemcpyAsync(p.tmaps, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice, s),
               "tensor maps", JC_MAP);
    cuda_check(cudaStreamSynchronize(s), "tensor maps", JC_POLL);
}

void BF16Path::forward(const Dims& d, const WeightsF32& w, const Pack& p, int mode, cudaStream_t s) const {
    const int R = p.R, D = d.D, n = p.n_inst;
    if (R == 0) return;
    bf16* ln = reinterpret_cast<bf16*>(p.bt[0]);
    bf16* qkv = reinterpret_cast<bf16*>(p.bt[1]);
    bf16* attn = reinterpret_cast<bf16*>(p.bt[2]);
    bf16* t1 = reinterpret_cast<bf16*>(p.bt[3]);
    bf16* zc = reinterpret_cast<bf16*>(p.bc[0]);
    float* c1 = reinterpret_cast<float*>(p.bc[1]);
    const CUtensorMap m_ln = rows_map(ln, D, R), m_attn = rows_map(attn, D, R), m_t1 = rows_map(t1, D, R);
    const unsigned gm = (unsigned)((R + 127) / 128);
    const Tuning tu = tuning_for(R);
    {
        KScope k("bf_embed", s);
        const unsigned blocks = (unsigned)((R + kEmbedRows - 1) / kEmbedRows);
        const size_t smem = ((size_t)d.C * d.P * d.P * D + (size_t)kEmbedRows * d.C * d.P * d.P) * sizeof(float);
        if (D <= 32) bf_embed_kernel<1><<<blocks, 256, smem, s>>>(d, w.embed_w, w.embed_b, w.meta_w, w.meta_b, w.blk[0].n1g, w.blk[0].n1b, p.inst, n, R, p.x, ln);
        else if (D <= 128) bf_embed_kernel<4><<<blocks, 256, smem, s>>>(d, w.embed_w, w.embed_b, w.meta_w, w.meta_b, w.blk[0].n1g, w.blk[0].n1b, p.inst, n, R, p.x, ln);
        else bf_embed_kernel<8><<<blocks, 256, smem, s>>>(d, w.embed_w, w.embed_b, w.meta_w, w.meta_b, w.blk[0].n1g, w.blk[0].n1b, p.inst, n, R, p.x, ln);
        check_launch("bf_embed");
    }
    for (int l = 0; l < d.L; l++) {
        const auto& B = w.blk[l];
        {
            KScope k("tc_qkv", s);
            const int BN = bn_qkv;
            GemmEpi ep{B.bqkv, qkv, nullptr, nullptr, nullptr, nullptr, 3 * D};
            tc_gemm_kernel<EPI_BF16><<<dim3(gm, 3 * D / BN), 128, (size_t)D * 256 + (size_t)D * BN * 2, s>>>(
                m_ln, wqkv[l], D, BN, R, ep, p.err);
            check_launch("tc_qkv");
        }
        {
            KScope k("bf_attention", s);
            launch_attention(d, qkv, p.inst, n, R, attn, tu.attn_threads, s);
            check_launch("bf_attention");
        }
        {
            KScope k("tc_proj_ln", s);
            GemmEpi ep{B.bp, ln, nullptr, p.x, B.n2g, B.n2b, D};
            const size_t smem = std::max((size_t)D * 256 + (size_t)D * D * 2, (size_t)128 * D * 4);
            tc_gemm_kernel<EPI_RESID_LN><<<dim3(gm, 1), 128, smem, s>>>(
                m_attn, wp[l], D, D, R, ep, p.err);
            check_launch("tc_proj_ln");
        }
        {
            KScope k("tc_mlp", s);
            const int NC = tu.nc, v = NC == 128 ? 1 : 0;
            const float* ng = l + 1 < d.L ? w.blk[l + 1].n1g : w.norm_g;
            const float* nbeta = l + 1 < d.L ? w.blk[l + 1].n1b : w.norm_b;
            const size_t smem = std::max((size_t)D * 256 + 2 * (size_t)D * NC * 2 + (size_t)NC * 256, (size_t)128 * D * 4);
            tc_mlp_kernel<<<gm, kMlpThreads, smem, s>>>(m_ln, w1v[v][l], w2v[v][l], B.b1, B.b2, D, d.F, NC, R, p.x, ng,
                                                        nbeta, ln, p.err);
            check_launch("tc_mlp");
        }
    }
    {
        KScope k("tc_token_mix", s);
        const int BN = bn_tm;
        size_t smem = (size_t)(D / 8) * kHaloPlane + 2 * (size_t)D * BN * 2;
        tc_conv3_kernel<CONV_TOKMIX><<<dim3(p.n_ttiles, D / BN), 128, smem, s>>>(
            reinterpret_cast<const CUtensorMap*>(p.tmaps), 0, wtm, w.tm_b, D, BN, D, p.inst, n, t1, p.err);
        check_launch("tc_token_mix");
    }
    {
        KScope k("tc_to_cells", s);
        GemmEpi ep{w.tc_b, nullptr, p.z0, nullptr, nullptr, nullptr, d.HD};
        tc_gemm_kernel<EPI_F32><<<dim3(gm, 1), 128, (size_t)D * 256 + (size_t)D * d.HD * 2, s>>>(
            m_t1, wtc, D, d.HD, R, ep, p.err);
        check_launch("tc_to_cells");
    }
    const long long NC = p.NC;
    {
        KScope k("bf_upsample", s);
        bf_upsample_kernel<<<(unsigned)((NC + 255) / 256), 256, 0, s>>>(d, p.z0, p.inst, n, NC, zc);
        check_launch("bf_upsample");
    }
    {
        KScope k("tc_conv1", s);
        size_t smem = (size_t)(kZcCh / 8) * kHaloPlane + 2 * (size_t)kZcCh * d.HD * 2;
        tc_conv3_kernel<CONV_CELL1><<<dim3(p.n_ctiles, 1), 128, smem, s>>>(
            reinterpret_cast<const CUtensorMap*>(p.tmaps), 1, wc1, w.c1_b, kZcCh, d.HD, d.HD, p.inst, n, c1, p.err);
        check_launch("tc_conv1");
    }
    conv2_step(d, c1, w, p, mode, "bf_conv2_step", s);
}

}  // namespace jc
