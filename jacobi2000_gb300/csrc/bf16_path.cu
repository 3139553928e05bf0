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
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>

#include "bf16_path.hpp"
#include "launch.hpp"
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

// f32 -> IEEE binary16 bits, round to nearest even (host)
static uint16_t f2h(float f) {
    const __half h = __float2half_rn(f);
    uint16_t u;
    std::memcpy(&u, &h, 2);
    return u;
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

// Tensor of `rank` dims (innermost first), strides in bytes of dims
// 1..rank-1, box dims; bf16 and no swizzle unless given; zero fill out of
// bounds.
static CUtensorMap make_map(const void* base, int rank, const uint64_t* dims, const uint64_t* strides,
                            const uint32_t* box, CUtensorMapDataType type = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                            CUtensorMapSwizzle swz = CU_TENSOR_MAP_SWIZZLE_NONE) {
    CUtensorMap m;
    cuuint64_t gd[5], gs[4];
    cuuint32_t bx[5], es[5];
    for (int i = 0; i < rank; i++) {
        gd[i] = dims[i];
        bx[i] = box[i];
        es[i] = 1;
    }
    for (int i = 0; i < rank - 1; i++) gs[i] = strides[i];
    CUresult r = encode_fn()(&m, type, rank, const_cast<void*>(base), gd, gs, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                             swz,
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

// Output tiles of a [rows, cols] matrix with row pitch `ld` elements (bf16,
// or f32 when f32): boxes of 128 bytes x 128 rows, stored from shared memory
// in the 128-byte swizzled layout (16-byte chunk j of tile row r at chunk
// j ^ (r % 8)).
static CUtensorMap store_map(const void* base, int cols, int rows, int ld, bool f32) {
    const int es = f32 ? 4 : 2;
    uint64_t dims[2] = {(uint64_t)cols, (uint64_t)(rows > 0 ? rows : 1)};
    uint64_t strides[1] = {(uint64_t)ld * es};
    uint32_t box[2] = {(uint32_t)(128 / es), 128};
    return make_map(base, 2, dims, strides, box, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                    CU_TENSOR_MAP_SWIZZLE_128B);
}

// One instance's [ny, nx, C] channel-last grid (bf16, or f32 when f32),
// stored as 128-byte x 8 x 16 boxes (one 8 x 16 conv tile, 128 bytes of
// channels) from 128-byte swizzled shared memory; positions outside the grid
// are not written.
static CUtensorMap tile_store_map(const void* base, int C, int nx, int ny, bool f32) {
    const int es = f32 ? 4 : 2;
    uint64_t dims[3] = {(uint64_t)C, (uint64_t)nx, (uint64_t)ny};
    uint64_t strides[2] = {(uint64_t)C * es, (uint64_t)nx * C * es};
    uint32_t box[3] = {(uint32_t)(128 / es), kConvTX, kConvTY};
    return make_map(base, 3, dims, strides, box, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
                    CU_TENSOR_MAP_SWIZZLE_128B);
}

// One instance's plane-major f16 cell-head grid: `planes` planes of
// [ny][nx][8 channels], `plane` bytes apart, seen as a [planes][ny][nx * 8]
// tensor, so each box row is a run of whole positions (one 16-byte chunk
// each) and a box of a conv tile moves in a few long rows instead of one
// 16-byte row per position. Halo loads: 10 x 18 positions of every plane
// from element (x0 - 1) * 8 (a 16-byte boundary; the fill covers the grid's
// edges), landing as [planes][18][10][8]; tile stores: 8 x 16 positions of
// every plane from [planes][16][8][8] (positions outside the grid are not
// written).
static CUtensorMap cell_plane_map(const void* base, int planes, long long plane, int nx, int ny, bool halo) {
    uint64_t dims[3] = {(uint64_t)nx * 8, (uint64_t)ny, (uint64_t)planes};
    uint64_t strides[2] = {(uint64_t)nx * 16, (uint64_t)plane};
    uint32_t box[3] = {(uint32_t)(halo ? (kConvTX + 2) * 8 : kConvTX * 8), (uint32_t)(halo ? kConvTY + 2 : kConvTY),
                       (uint32_t)planes};
    return make_map(base, 3, dims, strides, box, CU_TENSOR_MAP_DATA_TYPE_FLOAT16);
}

// One instance's qkv rows as a [ty, tx, 3D] grid, loaded as 64-channel boxes
// of side x side tokens in the 128-byte swizzled layout (attention tiles).
static CUtensorMap att_map(const void* base, int D, int tx, int ty, int side) {
    uint64_t dims[3] = {(uint64_t)(3 * D), (uint64_t)tx, (uint64_t)ty};
    uint64_t strides[2] = {(uint64_t)3 * D * 2, (uint64_t)tx * 3 * D * 2};
    uint32_t box[3] = {64, (uint32_t)side, (uint32_t)side};
    return make_map(base, 3, dims, strides, box, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, CU_TENSOR_MAP_SWIZZLE_128B);
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

// Cell-head input channels (f16, conv1's operand type; f16 keeps 3 more
// mantissa bits than bf16 and the values are far inside its range): 32 z,
// then the state split exactly into f16 parts, s = hi + lo: [hi (3), lo (3),
// hi (3)] multiplied by the conv1 weights [W_hi, W_hi, W_lo], so the state
// enters conv1 with ~22-bit precision; the remaining 7 channels are zero.
constexpr int kZcCh = 48;
constexpr int kZcState = 32;
constexpr int kHaloW = kConvTX + 2, kHaloH = kConvTY + 2;
// bytes of one 8-channel plane of a halo tile (2880 used), padded so every
// plane starts on a 128-byte boundary for TMA (token-level halos, one load
// per plane)
constexpr int kHaloPlane = (kHaloW * kHaloH * 16 + 127) / 128 * 128;
// one 8-channel plane of a cell-level halo tile, loaded with every other
// plane by one TMA box (planes packed)
constexpr int kCellPlane = kHaloW * kHaloH * 16;

__device__ __forceinline__ float bf2f(bf16 v) { return __bfloat162float(v); }

// d0 = fma(a0, b0, d0), d1 = fma(a1, b1, d1) in one paired instruction
// (fma.rn.f32x2: each lane rounds like fmaf).
__device__ __forceinline__ void fma2_f32(float& d0, float& d1, float a0, float a1, float b0, float b1) {
    asm("{\n\t.reg .b64 a, b, d;\n\tmov.b64 a, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\tmov.b64 d, {%0, %1};\n\t"
        "fma.rn.f32x2 d, a, b, d;\n\tmov.b64 {%0, %1}, d;\n\t}"
        : "+f"(d0), "+f"(d1)
        : "f"(a0), "f"(a1), "f"(b0), "f"(b1));
}

// Token embedding and the first LayerNorm (cpu.rs:253-280, 289). Persistent
// CTAs walk tiles of 64 token rows: the embed weights [pd][D] are staged in
// shared memory once per CTA, and each tile's patches arrive as 16-byte
// asynchronous copies (one per (row, channel, patch row): 4 cells), double-
// buffered so the next tile's patches are in flight while this one is
// summed. Patches sit as [channel, patch row][row][4] floats. Warp w owns
// rows 8w..8w+7 and lane l owns the CPL = D/32 consecutive outputs
// [CPL l, CPL l + CPL): per group of 4 patch elements it reads 8 patch
// float4s and 4 x CPL weights and does 32 x CPL FMAs. Each output is summed in
// the reference's order (bias, then the patch elements in order, then + pos,
// + the meta linear); x is written f32 and LayerNorm(x) bf16, with vector
// stores. The pos rows of a warp's 8 rows are loaded together before the
// LayerNorms, and the meta linear is kept while the instance stays the same
// (across tiles too).
constexpr int kEmbedRows = 64;
constexpr int kEmbedGroups = 12;  // 3 channels x 4 patch rows, 4 patch columns each

__host__ __device__ constexpr size_t embed_smem(int D) {
    return ((size_t)48 * D + 2 * (size_t)kEmbedGroups * kEmbedRows * 4) * sizeof(float);
}

template <int CPL>
__global__ void __launch_bounds__(256, (CPL <= 4 ? 3 : 1)) bf_embed_kernel(Dims d, const float* __restrict__ We,
                                                       const float* __restrict__ be, const float* __restrict__ Wm,
                                                       const float* __restrict__ bm, const float* __restrict__ g,
                                                       const float* __restrict__ b, const InstDev* inst, int n_inst,
                                                       int R, float* __restrict__ x, bf16* __restrict__ ln) {
    JC_PDL_ENTRY;
    extern __shared__ __align__(16) float esm[];
    constexpr int D = 32 * CPL;
    constexpr int P = 4, pd = 3 * P * P;  // 3 channels, patch 4 (checked when the path is built)
    float* sW = esm;                      // [pd][D]
    float4* sP = reinterpret_cast<float4*>(esm + (size_t)pd * D);  // 2 x [groups][kEmbedRows] float4
    __shared__ int rinst[2][kEmbedRows];
    const int n_tiles = (R + kEmbedRows - 1) / kEmbedRows;
    for (int i = threadIdx.x; i < pd * D / 4; i += blockDim.x)
        cp_async16(reinterpret_cast<float4*>(sW) + i, reinterpret_cast<const float4*>(We) + i, true);
    // the patches of tile t into buffer `buf` (and each row's instance); with
    // 256 threads, a multiple of the tile's rows, a thread copies the patches
    // of one row (threadIdx.x % kEmbedRows), so it finds that row's instance once
    static_assert(256 % kEmbedRows == 0, "embed copy layout");
    auto issue = [&](int t, int buf) {
        const int i = threadIdx.x % kEmbedRows, r = t * kEmbedRows + i;
        // a warp's rows are consecutive: the instance of its first row by a
        // warp-wide search, then at most a step or two per lane
        int ii = warp_find_last_le(n_inst, __shfl_sync(0xffffffffu, r, 0), [&](int k) { return (long long)inst[k].row0; });
        while (ii + 1 < n_inst && inst[ii + 1].row0 <= r) ii++;
        if (r >= R) ii = -1;
        for (int e = threadIdx.x; e < kEmbedRows * kEmbedGroups; e += blockDim.x) {
            const int gq = e / kEmbedRows;  // (channel, patch row)
            if (gq == 0) rinst[buf][i] = ii;
            const float* src = We;
            if (ii >= 0) {
                const InstDev& I = inst[ii];
                const int tk = r - I.row0, c = gq / P, py = gq % P;
                src = I.state + (size_t)c * I.nx * I.ny + ((size_t)(tk / I.tx) * P + py) * I.nx +
                      (size_t)(tk % I.tx) * P;
            }
            cp_async16(sP + ((size_t)buf * kEmbedGroups + gq) * kEmbedRows + i, src, ii >= 0);
        }
        cp_async_commit();
    };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i0 = warp * 8;  // this warp's 8 rows
    const int o0 = CPL * lane;
    int k = 0;
    int m_inst = -1;  // the instance whose meta linear m holds
    float m[CPL];
    if ((int)blockIdx.x < n_tiles) issue(blockIdx.x, 0);
    for (int t = blockIdx.x; t < n_tiles; t += gridDim.x, k++) {
        const int buf = k & 1;
        if (t + (int)gridDim.x < n_tiles) {
            issue(t + gridDim.x, buf ^ 1);
            cp_async_wait_group<1>();
        } else {
            cp_async_wait_group<0>();
        }
        __syncthreads();
        const int r0 = t * kEmbedRows;
        if (r0 + i0 < R) {
            float v[8][CPL];
#pragma unroll
            for (int q = 0; q < 8; q++)
#pragma unroll
                for (int c = 0; c < CPL; c++) v[q][c] = be[o0 + c];
            const float4* pb = sP + (size_t)buf * kEmbedGroups * kEmbedRows + i0;
#pragma unroll 2
            for (int gq = 0; gq < kEmbedGroups; gq++) {
                float4 p4[8];
#pragma unroll
                for (int q = 0; q < 8; q++) p4[q] = pb[gq * kEmbedRows + q];
#pragma unroll
                for (int px = 0; px < 4; px++) {
                    const int f = gq * 4 + px;
                    float wv[CPL];
                    if (CPL % 4 == 0) {
#pragma unroll
                        for (int c = 0; c < CPL; c += 4) {
                            const float4 w4 = *reinterpret_cast<const float4*>(sW + f * D + o0 + c);
                            wv[c] = w4.x; wv[c + 1] = w4.y; wv[c + 2] = w4.z; wv[c + 3] = w4.w;
                        }
                    } else {
#pragma unroll
                        for (int c = 0; c < CPL; c++) wv[c] = sW[f * D + o0 + c];
                    }
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const float pv = px == 0 ? p4[q].x : px == 1 ? p4[q].y : px == 2 ? p4[q].z : p4[q].w;
                        if (CPL % 2 == 0) {
#pragma unroll
                            for (int c = 0; c < CPL; c += 2) fma2_f32(v[q][c], v[q][c + 1], pv, pv, wv[c], wv[c + 1]);
                        } else {
#pragma unroll
                            for (int c = 0; c < CPL; c++) v[q][c] = fmaf(pv, wv[c], v[q][c]);
                        }
                    }
                }
            }
            // + pos for the warp's 8 rows, the loads of all rows in flight together
            int rii[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int r = r0 + i0 + q;
                rii[q] = r < R ? rinst[buf][i0 + q] : -1;
                if (rii[q] >= 0) {
                    const InstDev& I = inst[rii[q]];
                    const float* pos = I.pos + (size_t)(r - I.row0) * D + o0;
                    if (CPL % 4 == 0) {
#pragma unroll
                        for (int c = 0; c < CPL; c += 4) {
                            const float4 p4 = *reinterpret_cast<const float4*>(pos + c);
                            v[q][c] += p4.x; v[q][c + 1] += p4.y; v[q][c + 2] += p4.z; v[q][c + 3] += p4.w;
                        }
                    } else {
#pragma unroll
                        for (int c = 0; c < CPL; c++) v[q][c] += pos[c];
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int r = r0 + i0 + q;
                if (r >= R) continue;  // warp-uniform
                const int ii = rii[q];
                if (ii != m_inst) {
                    // the meta linear depends only on the instance: computed
                    // again only where the instance changes (kept across tiles)
                    const InstDev& I = inst[ii];
                    m_inst = ii;
#pragma unroll
                    for (int c = 0; c < CPL; c++) {
                        m[c] = bm[o0 + c];
                        for (int f = 0; f < d.meta_dim; f++) m[c] = fmaf(I.meta[f], Wm[(size_t)f * D + o0 + c], m[c]);
                    }
                }
                float sum = 0.f;
#pragma unroll
                for (int c = 0; c < CPL; c++) {
                    v[q][c] = v[q][c] + m[c];
                    sum += v[q][c];
                }
                const float mean = warp_sum(sum) / (float)D;
                float sq = 0.f;
#pragma unroll
                for (int c = 0; c < CPL; c++) sq += (v[q][c] - mean) * (v[q][c] - mean);
                const float rstd = rsqrtf(warp_sum(sq) / (float)D + 1e-5f);  // 2 ulp
                float o[CPL];
#pragma unroll
                for (int c = 0; c < CPL; c++) o[c] = (v[q][c] - mean) * rstd * g[o0 + c] + b[o0 + c];
                float* xr = x + (size_t)r * D + o0;
                bf16* lr = ln + (size_t)r * D + o0;
                if (CPL % 4 == 0) {
#pragma unroll
                    for (int c = 0; c < CPL; c += 4) {
                        *reinterpret_cast<float4*>(xr + c) = make_float4(v[q][c], v[q][c + 1], v[q][c + 2], v[q][c + 3]);
                        __nv_bfloat162 lo = __floats2bfloat162_rn(o[c], o[c + 1]);
                        __nv_bfloat162 hi = __floats2bfloat162_rn(o[c + 2], o[c + 3]);
                        uint2 u;
                        u.x = *reinterpret_cast<uint32_t*>(&lo);
                        u.y = *reinterpret_cast<uint32_t*>(&hi);
                        *reinterpret_cast<uint2*>(lr + c) = u;
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < CPL; c++) {
                        xr[c] = v[q][c];
                        lr[c] = __float2bfloat16(o[c]);
                    }
                }
            }
        }
        __syncthreads();  // every warp is done with `buf` before it is refilled
    }
    cp_async_wait_group<0>();
}

// Packed bf16 vectors of 1, 4 or 8 elements <-> f32.
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

// One thread per (token row, head): the head's query stays in registers and
// every dot product and weighted sum runs serially in the thread, so no
// shuffles are needed; the threads of one row read the key and value rows of
// a candidate as consecutive 16-byte pieces. Radius-1 stencil (any dilation):
// scores, max, exp, denominator and the (e / denom)-weighted sum in the
// reference's order (cpu.rs:121-158); a general stencil or the full mask uses
// the online (running max) form.
template <int HD>
__device__ __forceinline__ void load_head(const bf16* p, float* f) {
#pragma unroll
    for (int w = 0; w < HD / 8; w++) {
        const uint4 u = reinterpret_cast<const uint4*>(p)[w];
        const uint32_t a[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            f[8 * w + 2 * i] = __uint_as_float(a[i] << 16);
            f[8 * w + 2 * i + 1] = __uint_as_float(a[i] & 0xffff0000u);
        }
    }
}

template <int HD>
__device__ __forceinline__ float dot_head(const float* q, const bf16* kp) {
    float p0 = 0.f, p1 = 0.f;
#pragma unroll
    for (int w = 0; w < HD / 8; w++) {
        const uint4 u = reinterpret_cast<const uint4*>(kp)[w];
        const uint32_t a[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            p0 = fmaf(q[8 * w + 2 * i], __uint_as_float(a[i] << 16), p0);
            p1 = fmaf(q[8 * w + 2 * i + 1], __uint_as_float(a[i] & 0xffff0000u), p1);
        }
    }
    return p0 + p1;
}

template <int HD>
__device__ __forceinline__ void axpy_head(float wgt, const bf16* vp, float* acc) {
#pragma unroll
    for (int w = 0; w < HD / 8; w++) {
        const uint4 u = reinterpret_cast<const uint4*>(vp)[w];
        const uint32_t a[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            acc[8 * w + 2 * i] = fmaf(wgt, __uint_as_float(a[i] << 16), acc[8 * w + 2 * i]);
            acc[8 * w + 2 * i + 1] = fmaf(wgt, __uint_as_float(a[i] & 0xffff0000u), acc[8 * w + 2 * i + 1]);
        }
    }
}

template <int HD>
__device__ __forceinline__ void store_head(bf16* p, const float* acc) {
#pragma unroll
    for (int w = 0; w < HD / 8; w++) BfVec<8>::store(p + 8 * w, acc + 8 * w);
}

template <int HD>
__global__ void __launch_bounds__(256) bf_attn_head_r1_kernel(Dims d, const bf16* __restrict__ qkv,
                                                              const InstDev* inst, int n_inst, int R,
                                                              bf16* __restrict__ out) {
    JC_PDL_ENTRY;
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = gid / d.heads, h = gid - r * d.heads;
    if (r >= R) return;
    const int D = d.D;
    const size_t D3 = 3 * (size_t)D;
    const InstDev& I = inst[inst_of_row(inst, n_inst, r)];
    const int t = r - I.row0, qy = t / I.tx, qx = t - qy * I.tx, dil = d.dilation;
    const float scale = 1.0f / sqrtf((float)HD);
    float q[HD];
    load_head<HD>(qkv + (size_t)r * D3 + h * HD, q);
    float sc[9];
    int kr[9];
    float smax = -INFINITY;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const int ky = qy + (j / 3 - 1) * dil, kx = qx + (j % 3 - 1) * dil;
        const bool in = ky >= 0 && kx >= 0 && ky < I.ty && kx < I.tx;
        kr[j] = in ? I.row0 + ky * I.tx + kx : -1;
        sc[j] = in ? dot_head<HD>(q, qkv + (size_t)kr[j] * D3 + D + h * HD) * scale : -INFINITY;
        smax = fmaxf(smax, sc[j]);
    }
    float denom = 0.f;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        sc[j] = kr[j] >= 0 ? __expf(sc[j] - smax) : 0.f;
        denom += sc[j];
    }
    const float inv = 1.0f / denom;
    float acc[HD];
#pragma unroll
    for (int i = 0; i < HD; i++) acc[i] = 0.f;
#pragma unroll
    for (int j = 0; j < 9; j++)
        if (kr[j] >= 0) axpy_head<HD>(sc[j] * inv, qkv + (size_t)kr[j] * D3 + 2 * D + h * HD, acc);
    store_head<HD>(out + (size_t)r * D + h * HD, acc);
}

template <int HD>
__global__ void __launch_bounds__(256) bf_attn_head_kernel(Dims d, const bf16* __restrict__ qkv, const InstDev* inst,
                                                           int n_inst, int R, bf16* __restrict__ out) {
    JC_PDL_ENTRY;
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = gid / d.heads, h = gid - r * d.heads;
    if (r >= R) return;
    const int D = d.D;
    const size_t D3 = 3 * (size_t)D;
    const InstDev& I = inst[inst_of_row(inst, n_inst, r)];
    const int t = r - I.row0, qy = t / I.tx, qx = t - qy * I.tx;
    const float scale = 1.0f / sqrtf((float)HD);
    float q[HD], acc[HD];
    load_head<HD>(qkv + (size_t)r * D3 + h * HD, q);
#pragma unroll
    for (int i = 0; i < HD; i++) acc[i] = 0.f;
    const int side = 2 * d.radius + 1;
    const int nc = d.mask_kind == 0 ? I.tx * I.ty : side * side;
    float m = -INFINITY, l = 0.f;
    for (int j = 0; j < nc; j++) {
        int kr;
        if (d.mask_kind == 0) {
            kr = I.row0 + j;
        } else {
            const int ky = qy + (j / side - d.radius) * d.dilation, kx = qx + (j % side - d.radius) * d.dilation;
            if (ky < 0 || kx < 0 || ky >= I.ty || kx >= I.tx) continue;
            kr = I.row0 + ky * I.tx + kx;
        }
        const float s = dot_head<HD>(q, qkv + (size_t)kr * D3 + D + h * HD) * scale;
        const float mn = fmaxf(m, s);
        const float c = __expf(m - mn), e = __expf(s - mn);
        l = l * c + e;
#pragma unroll
        for (int i = 0; i < HD; i++) acc[i] *= c;
        axpy_head<HD>(e, qkv + (size_t)kr * D3 + 2 * D + h * HD, acc);
        m = mn;
    }
    const float inv = 1.0f / l;
#pragma unroll
    for (int i = 0; i < HD; i++) acc[i] *= inv;
    store_head<HD>(out + (size_t)r * D + h * HD, acc);
}

// Radius-1, dilation-1 stencil attention over shared-memory tiles (cpu.rs:
// 97-164, mask.rs:18-30). A CTA takes one 8 x 8 block of an instance's token
// grid (half of an 8 x 16 conv tile) for the heads of one 64-channel box:
// TMA brings the block's queries and the keys and values of its 10 x 10 halo
// for those channels into shared memory as 128-byte swizzled boxes (zero fill
// outside the grid, where the mask excludes the candidates anyway); 34 KB per
// CTA keeps six CTAs on an SM. Thread (token, head) then does the
// arithmetic of bf_attn_head_r1_kernel, in the same order, on shared-memory
// operands: the eight lanes of a quarter warp are eight neighbouring tokens
// of one head, so the swizzle spreads their 16-byte reads over all banks.
constexpr int kAttTile = 8;                        // tokens per side of a CTA's block
constexpr int kAttHalo = kAttTile + 2;             // halo side
constexpr int kAttBoxKV = kAttHalo * kAttHalo * 128;   // one 64-channel halo box: 12800 bytes
constexpr int kAttBoxKVPad = 13 * 1024;                // 1024-aligned slot of one halo box
constexpr int kAttBoxQ = kAttTile * kAttTile * 128;    // one 64-channel query box: 8192 bytes

// 16-byte chunk c (0..7) of row rho of a 128-byte swizzled box
__device__ __forceinline__ const uint4* swz_chunk(const uint8_t* box, int rho, int c) {
    return reinterpret_cast<const uint4*>(box + (size_t)rho * 128 + ((c ^ (rho & 7)) << 4));
}

template <int HD>
__device__ __forceinline__ void axpy_head_s(float wgt, const uint8_t* boxes, int box_stride, int rho, int ch0,
                                            float* acc) {
#pragma unroll
    for (int w = 0; w < HD / 8; w++) {
        const int ch = ch0 + 8 * w;
        const uint4 u = *swz_chunk(boxes + (size_t)(ch >> 6) * box_stride, rho, (ch & 63) >> 3);
        const uint32_t a[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
        for (int i = 0; i < 4; i++) {
            acc[8 * w + 2 * i] = fmaf(wgt, __uint_as_float(a[i] << 16), acc[8 * w + 2 * i]);
            acc[8 * w + 2 * i + 1] = fmaf(wgt, __uint_as_float(a[i] & 0xffff0000u), acc[8 * w + 2 * i + 1]);
        }
    }
}

// lo += a.lo * b.lo, hi += a.hi * b.hi for bf16 pairs a, b with f32
// accumulators, one rounding each (mixed-precision fma.rn.f32.bf16).
__device__ __forceinline__ void fma2_bf16_f32(uint32_t a, uint32_t b, float& lo, float& hi) {
    asm("{\n\t.reg .b16 al, ah, bl, bh;\n\t"
        "mov.b32 {al, ah}, %2;\n\t"
        "mov.b32 {bl, bh}, %3;\n\t"
        "fma.rn.f32.bf16 %0, al, bl, %0;\n\t"
        "fma.rn.f32.bf16 %1, ah, bh, %1;\n\t}"
        : "+f"(lo), "+f"(hi)
        : "r"(a), "r"(b));
}

// One (token, head) of the radius-1 stencil attention from the staged boxes:
// query box sQ (8 x 8 tokens), key and value halo boxes sK, sV (10 x 10; the
// positions outside the grid hold the tensor map's zero fill), token (lx, ly)
// of the block, grid position (qx, qy) in a tx x ty token grid. The nine
// scores are accumulated together, channel chunk outer and key inner, so a
// thread has 18 independent FMA chains in flight; each chain adds its
// channels in the same order as dot_head (even channels in one, odd in the
// other, then the two added), so every attention form gives the same bits.
// Keys outside the grid get score
// -inf and weight 0 (their zero-filled values then add exact zeros).
template <int HD>
__device__ __forceinline__ void attn_stencil_token(const uint8_t* sQ, const uint8_t* sK, const uint8_t* sV, int lx,
                                                   int ly, int qx, int qy, int tx, int ty, int hl, float scale,
                                                   float* acc) {
    // the query stays packed (bf16 pairs); scores use the mixed-precision FMA
    // bf16 x bf16 + f32, whose product is exact in f32, so each step rounds
    // exactly like fmaf on the unpacked values
    uint32_t q[HD / 2];
#pragma unroll
    for (int w = 0; w < HD / 8; w++) {
        const int ch = hl * HD + 8 * w;
        const uint4 u = *swz_chunk(sQ + (size_t)(ch >> 6) * kAttBoxQ, ly * kAttTile + lx, (ch & 63) >> 3);
        q[4 * w] = u.x;
        q[4 * w + 1] = u.y;
        q[4 * w + 2] = u.z;
        q[4 * w + 3] = u.w;
    }
    float p0[9], p1[9];
#pragma unroll
    for (int j = 0; j < 9; j++) p0[j] = p1[j] = 0.f;
#pragma unroll
    for (int w = 0; w < HD / 8; w++) {
        const int ch = hl * HD + 8 * w;
#pragma unroll
        for (int j = 0; j < 9; j++) {
            const int rho = (ly + j / 3) * kAttHalo + (lx + j % 3);
            const uint4 u = *swz_chunk(sK + (size_t)(ch >> 6) * kAttBoxKVPad, rho, (ch & 63) >> 3);
            const uint32_t a[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int i = 0; i < 4; i++) fma2_bf16_f32(q[4 * w + i], a[i], p0[j], p1[j]);
        }
    }
    float sc[9];
    bool in[9];
    float smax = -INFINITY;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const int ky = qy + j / 3 - 1, kx = qx + j % 3 - 1;
        in[j] = ky >= 0 && kx >= 0 && ky < ty && kx < tx;
        sc[j] = in[j] ? (p0[j] + p1[j]) * scale : -INFINITY;
        smax = fmaxf(smax, sc[j]);
    }
    float denom = 0.f;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        sc[j] = in[j] ? __expf(sc[j] - smax) : 0.f;
        denom += sc[j];
    }
    const float inv = 1.0f / denom;
#pragma unroll
    for (int i = 0; i < HD; i++) acc[i] = 0.f;
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const int rho = (ly + j / 3) * kAttHalo + (lx + j % 3);
        axpy_head_s<HD>(sc[j] * inv, sV, kAttBoxKVPad, rho, hl * HD, acc);
    }
}

// Maps of an instance used here: slot kv_slot = halo boxes (64 ch x 10 x 10)
// over its qkv rows, slot q_slot = query boxes (64 ch x 8 x 8) over the same
// rows. D = 64 * (boxes per vector); threads = 64 tokens x heads.
template <int HD>
__global__ void __launch_bounds__(64 * (64 / HD), 5) bf_attn_tile_kernel(Dims d, const CUtensorMap* __restrict__ maps, int kv_slot,
                                                           int q_slot, const InstDev* inst, int n_inst,
                                                           bf16* __restrict__ out, int* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const int D = d.D;
    constexpr int HPB = 64 / HD;                  // heads per 64-channel box
    const int bx = blockIdx.z;                    // this CTA's box: heads bx HPB ..
    uint8_t* sK = smem;                           // the halo box of the keys
    uint8_t* sV = sK + (size_t)kAttBoxKVPad;      // the halo box of the values
    uint8_t* sQ = sV + (size_t)kAttBoxKVPad;      // the query box
    __shared__ uint64_t bar;
    __shared__ volatile int failed;
    const int tile = blockIdx.x, half = blockIdx.y;
    const int lo = warp_find_last_le(n_inst, tile, [&](int i) { return (long long)inst[i].tt0; });
    // the instance's fields in registers (no reloads after the barriers)
    const int Itx = inst[lo].tx, Ity = inst[lo].ty, Itt0 = inst[lo].tt0, Irow0 = inst[lo].row0;
    const int tiles_x = (Itx + kConvTX - 1) / kConvTX;
    const int tl = tile - Itt0;
    const int x0 = (tl % tiles_x) * kConvTX, y0 = (tl / tiles_x) * kConvTY + half * kAttTile;
    const CUtensorMap* mkv = maps + kMapsPerInst * lo + kv_slot;
    const CUtensorMap* mq = maps + kMapsPerInst * lo + q_slot;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_barrier_init();
        failed = 0;
        if (tc::smem_u32(smem) & 1023u) {
            failed = 1;
            atomicExch(err, 2);
        }
    }
    __syncthreads();
    JC_PDL_ENTRY;
    if (y0 >= Ity) return;  // the lower half of a tile that overhangs the grid (uniform per CTA)
    if (threadIdx.x == 0 && !failed) {
        tc::tensormap_acquire(mkv);
        tc::tensormap_acquire(mq);
        tc::mbar_expect_tx(&bar, (uint32_t)(2 * kAttBoxKV + kAttBoxQ));
        tc::tma_load_3d(sK, mkv, D + 64 * bx, x0 - 1, y0 - 1, &bar);
        tc::tma_load_3d(sV, mkv, 2 * D + 64 * bx, x0 - 1, y0 - 1, &bar);
        tc::tma_load_3d(sQ, mq, 64 * bx, x0, y0, &bar);
    }
    const bool ok = __syncthreads_and(tc::mbar_wait(&bar, 0, err, &failed) ? 1 : 0) != 0;
    if (!ok) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int hl = warp % HPB;                   // head within the box
    const int h = bx * HPB + hl;
    const int tok = (warp / HPB) * 32 + lane;    // 0..63 within the block
    if (tok >= kAttTile * kAttTile) return;
    const int lx = tok & 7, ly = tok >> 3;
    const int qx = x0 + lx, qy = y0 + ly;
    if (qx >= Itx || qy >= Ity) return;
    const float scale = 1.0f / sqrtf((float)HD);
    float acc[HD];
    attn_stencil_token<HD>(sQ, sK, sV, lx, ly, qx, qy, Itx, Ity, hl, scale, acc);
    store_head<HD>(out + ((size_t)Irow0 + (size_t)qy * Itx + qx) * D + h * HD, acc);
}

// to_cells' output (f32 [rows, HD]) -> the cell-head input zc (f16, 48
// channels, conv1's operand type, plane-major: [6][cells][8], `zc_plane`
// elements between planes): upsample along y then x (cpu.rs:211-245;
// weights (i + 1/2) / P, the far neighbour clamped to the grid), the state
// appended split exactly into f16 parts (cpu.rs:339-342), zero padding. One CTA per 8 x 16 cell tile
// (the conv tiles): the 5 x 3 tokens it reads are staged in shared memory
// (row pitch HD + 4 floats against bank conflicts), thread r makes cell
// (y0 + r / 8, x0 + r % 8).
constexpr int kUpTokY = kConvTY / 4 + 1, kUpTokX = kConvTX / 4 + 1, kUpPitch = 36;

template <int HD, int C>
__global__ void __launch_bounds__(128) bf_upsample_kernel(Dims d, const float* __restrict__ z0, const InstDev* inst,
                                                          int n_inst, __half* __restrict__ zc, long long zc_plane) {
    static_assert(kZcState == HD && kZcState + 3 * C <= kZcCh && HD + 4 <= kUpPitch, "zc layout");
    constexpr int P = 4;  // patch (the BF16 path is built for 4); (i + 1/2) / 4 is exact as a product
    __shared__ __align__(16) float win[kUpTokY * kUpTokX * kUpPitch];
    const int tile = blockIdx.x;
    // the instance descriptors are written before the forward's first kernel
    const int lo = warp_find_last_le(n_inst, tile, [&](int i) { return (long long)inst[i].ct0; });
    const InstDev I = inst[lo];
    JC_PDL_ENTRY;
    const int tiles_x = (I.nx + kConvTX - 1) / kConvTX;
    const int tl = tile - I.ct0;
    const int x0 = (tl % tiles_x) * kConvTX, y0 = (tl / tiles_x) * kConvTY;
    const int ty0 = y0 / P, tx0 = x0 / P;
    for (int e = threadIdx.x; e < kUpTokY * kUpTokX * (HD / 4); e += blockDim.x) {
        const int q = e % (HD / 4), t = e / (HD / 4), ty = ty0 + t / kUpTokX, tx = tx0 + t % kUpTokX;
        const bool in = ty < I.ty && tx < I.tx;
        cp_async16(win + t * kUpPitch + 4 * q, in ? z0 + (size_t)(I.row0 + ty * I.tx + tx) * HD + 4 * q : z0, in);
    }
    cp_async_wait_all();
    __syncthreads();
    const int r = threadIdx.x;
    const int y = y0 + r / kConvTX, x = x0 + r % kConvTX;
    if (y >= I.ny || x >= I.nx) return;
    const int yt = y / P, iy = y % P, xt = x / P, ix = x % P;
    const int yt2 = min(yt + 1, I.ty - 1), xt2 = min(xt + 1, I.tx - 1);
    const float wy = ((float)iy + 0.5f) * (1.0f / P), wx = ((float)ix + 0.5f) * (1.0f / P);
    auto tok = [&](int ty, int tx) {
        return reinterpret_cast<const float4*>(win + ((ty - ty0) * kUpTokX + (tx - tx0)) * kUpPitch);
    };
    const float4 *a = tok(yt, xt), *b = tok(yt, xt2), *c = tok(yt2, xt), *e = tok(yt2, xt2);
    const float uy = 1.0f - wy, ux = 1.0f - wx;
    float vals[kZcCh];
#pragma unroll
    for (int i = 0; i < kZcCh; i++) vals[i] = 0.f;
#pragma unroll
    for (int q = 0; q < HD / 4; q++) {
        float4 A = a[q], B = b[q], Cc = c[q], E = e[q];
        vals[4 * q + 0] = (A.x * uy + Cc.x * wy) * ux + (B.x * uy + E.x * wy) * wx;
        vals[4 * q + 1] = (A.y * uy + Cc.y * wy) * ux + (B.y * uy + E.y * wy) * wx;
        vals[4 * q + 2] = (A.z * uy + Cc.z * wy) * ux + (B.z * uy + E.z * wy) * wx;
        vals[4 * q + 3] = (A.w * uy + Cc.w * wy) * ux + (B.w * uy + E.w * wy) * wx;
    }
    const size_t plane = (size_t)I.nx * I.ny, cl = (size_t)y * I.nx + x;
#pragma unroll
    for (int ch = 0; ch < C; ch++) {
        const float sv = I.state[ch * plane + cl];
        const float hi = __half2float(__float2half_rn(sv));
        vals[kZcState + ch] = hi;
        vals[kZcState + 3 + ch] = sv - hi;  // exact in f32; rounded to f16 below
        vals[kZcState + 6 + ch] = hi;
    }
    __half* o = zc + ((size_t)I.cell0 + cl) * 8;
#pragma unroll
    for (int q = 0; q < kZcCh / 8; q++) {
        uint32_t w[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            __half2 h = __floats2half2_rn(vals[8 * q + 2 * i], vals[8 * q + 2 * i + 1]);
            w[i] = *reinterpret_cast<uint32_t*>(&h);
        }
        *reinterpret_cast<uint4*>(o + q * zc_plane) = make_uint4(w[0], w[1], w[2], w[3]);
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

// GELU, x Phi(x) (cpu.rs:67-74), as x * sigmoid(2 u) with the odd
// polynomial u = x (c1 + c3 x^2 + c5 x^4): the tanh form of Hendrycks &
// Gimpel (2016) with its coefficients refitted (minimax of the absolute GELU
// error on |x| <= 9; |x| is clamped to 9, where Phi is 0 or 1 to f32
// precision). Maximum absolute error 2.6e-5 against the exact erf form, far
// below the bf16 rounding of the values it feeds. Two MUFU operations
// (ex2, rcp) and seven FMA-pipe instructions.
__device__ __forceinline__ float gelu_fast(float x) {
    // coefficients of u, times -2 log2(e), so sigmoid(2u) = 1 / (1 + 2^t)
    constexpr float k1 = -2.0f * 1.4426950408889634f * 7.97506042e-01f;
    constexpr float k3 = -2.0f * 1.4426950408889634f * 3.70071725e-02f;
    constexpr float k5 = -2.0f * 1.4426950408889634f * -3.51557324e-04f;
    const float xc = fminf(fmaxf(x, -9.0f), 9.0f);
    const float x2 = xc * xc;
    const float t = xc * fmaf(x2, fmaf(x2, k5, k3), k1);
    float e, r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(t));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(1.0f + e));
    return x * r;
}

// gelu_fast(v + b) of two values with the adds, multiplies and multiply-adds
// paired (add/mul/fma.rn.f32x2: each lane is the scalar operation with the
// same rounding), so both results are gelu_fast's bits in fewer instructions.
__device__ __forceinline__ void gelu_fast_pair(float& v0, float& v1, float b0, float b1) {
    constexpr float k1 = -2.0f * 1.4426950408889634f * 7.97506042e-01f;
    constexpr float k3 = -2.0f * 1.4426950408889634f * 3.70071725e-02f;
    constexpr float k5 = -2.0f * 1.4426950408889634f * -3.51557324e-04f;
    float x0, x1, e0, e1, r0, r1;
    asm("{\n\t.reg .b64 v, b;\n\tmov.b64 v, {%2, %3};\n\tmov.b64 b, {%4, %5};\n\t"
        "add.rn.f32x2 v, v, b;\n\tmov.b64 {%0, %1}, v;\n\t}"
        : "=f"(x0), "=f"(x1)
        : "f"(v0), "f"(v1), "f"(b0), "f"(b1));
    const float c0 = fminf(fmaxf(x0, -9.0f), 9.0f), c1 = fminf(fmaxf(x1, -9.0f), 9.0f);
    float t0, t1;
    asm("{\n\t.reg .b64 c, q, p, kk1, kk3, kk5;\n\tmov.b64 c, {%2, %3};\n\t"
        "mov.b64 kk1, {%4, %4};\n\tmov.b64 kk3, {%5, %5};\n\tmov.b64 kk5, {%6, %6};\n\t"
        "mul.rn.f32x2 q, c, c;\n\tfma.rn.f32x2 p, q, kk5, kk3;\n\tfma.rn.f32x2 p, q, p, kk1;\n\t"
        "mul.rn.f32x2 p, c, p;\n\tmov.b64 {%0, %1}, p;\n\t}"
        : "=f"(t0), "=f"(t1)
        : "f"(c0), "f"(c1), "f"(k1), "f"(k3), "f"(k5));
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e0) : "f"(t0));
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e1) : "f"(t1));
    float d0, d1;
    asm("{\n\t.reg .b64 e, one;\n\tmov.b64 e, {%2, %3};\n\tmov.b64 one, {%4, %4};\n\t"
        "add.rn.f32x2 e, one, e;\n\tmov.b64 {%0, %1}, e;\n\t}"
        : "=f"(d0), "=f"(d1)
        : "f"(e0), "f"(e1), "f"(1.0f));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(d0));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(d1));
    asm("{\n\t.reg .b64 x, r;\n\tmov.b64 x, {%2, %3};\n\tmov.b64 r, {%4, %5};\n\t"
        "mul.rn.f32x2 x, x, r;\n\tmov.b64 {%0, %1}, x;\n\t}"
        : "=f"(v0), "=f"(v1)
        : "f"(x0), "f"(x1), "f"(r0), "f"(r1));
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

// Residual + LayerNorm rows (two-pass mean and biased variance, eps 1e-5),
// in one fixed arithmetic shared by every kernel that produces them, so the
// MLP forms give the same bits: every operation is an explicitly rounded
// one (no compiler contraction), element v = x + (acc + bias); each
// 4-element slot contributes ((v0 + v1) + (v2 + v3)) and, for the variance,
// fma(e0, e0, e1 e1) + fma(e2, e2, e3 e3); slot q belongs to lane q % 32, a
// lane sums its slots in order starting from 0, and the 32 lane partials are
// added in the xor-butterfly order of warp_sum; rstd = ln_rstd(sum of
// squared deviations); out = fma((v - mean) rstd, g, b).
__device__ __forceinline__ float4 resid4(float4 x, float4 a, float4 bias) {
    return make_float4(__fadd_rn(x.x, __fadd_rn(a.x, bias.x)), __fadd_rn(x.y, __fadd_rn(a.y, bias.y)),
                       __fadd_rn(x.z, __fadd_rn(a.z, bias.z)), __fadd_rn(x.w, __fadd_rn(a.w, bias.w)));
}
__device__ __forceinline__ float sum4(float4 v) { return __fadd_rn(__fadd_rn(v.x, v.y), __fadd_rn(v.z, v.w)); }
__device__ __forceinline__ float sqdev4(float4 v, float m) {
    const float e0 = __fsub_rn(v.x, m), e1 = __fsub_rn(v.y, m), e2 = __fsub_rn(v.z, m), e3 = __fsub_rn(v.w, m);
    return __fadd_rn(__fmaf_rn(e0, e0, __fmul_rn(e1, e1)), __fmaf_rn(e2, e2, __fmul_rn(e3, e3)));
}
// 1 / sqrt(variance + eps) of the residual + LayerNorm rows: the hardware
// reciprocal square root (rsqrtf, 2 ulp), not a rounded square root and a
// rounded division (which cost the MLP kernel 7% of its time). Every kernel
// that forms these rows calls this, so they keep giving the same bits.
__device__ __forceinline__ float ln_rstd(float sq_sum, int D) { return rsqrtf(sq_sum / (float)D + 1e-5f); }

__device__ __forceinline__ float ln1(float v, float m, float rstd, float g, float b) {
    return __fmaf_rn(__fmul_rn(__fsub_rn(v, m), rstd), g, b);
}
// warp_sum of N independent values at once: the butterfly steps of all N are
// interleaved, so their shuffle latencies overlap; each value is added in
// warp_sum's order and gets warp_sum's bits.
template <int N>
__device__ __forceinline__ void warp_sum_n(float (&v)[N]) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < N; k++) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
}

// The 32 lane partials in the order warp_sum adds them.
__device__ __forceinline__ float tree32(float* a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int i = 0; i < o; i++) a[i] = __fadd_rn(a[i], a[i + o]);
    return a[0];
}

// One warp per tile row over the staged accumulator tile (float4 slot q of
// row r at q ^ slot_swz(r, D)); x and ln are read and written coalesced, G
// rows in flight per warp. Rows [0, nrows) of the tile (a multiple of G),
// tile row r -> global row m0 + r. SPL = slots per lane (1: D <= 128, 2: 256).
// PRE: load every row group's residual rows up front (four groups at most).
// A warp's residual rows for rows_resid_ln_t at D = 128 (lane l's slot of
// each of its up to 16 rows), loaded ahead of the epilogue by load_xrows so
// the loads overlap an MMA wait.
struct XRows {
    float4 v[4][4];
};
__device__ __forceinline__ void load_xrows(const float* __restrict__ x, int m0, int R, int warp, int nwarps,
                                           int nrows, XRows& xr) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int r0 = warp * 4 + i * nwarps * 4;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int row = m0 + r0 + k;
            xr.v[i][k] = r0 < nrows && row < R ? reinterpret_cast<const float4*>(x + (size_t)row * 128)[lane]
                                               : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
}

template <int SPL, bool FULL, bool PRE = false, bool LNS = false>  // FULL: every lane owns SPL slots (D = 128 SPL)
__device__ __forceinline__ void rows_resid_ln_t(const float* tile, int D, int m0, int R, const float* __restrict__ bias,
                                float* __restrict__ x, const float* __restrict__ g, const float* __restrict__ b,
                                bf16* __restrict__ ln, int warp, int nwarps, int nrows, const XRows* xin = nullptr) {
    const int lane = threadIdx.x & 31;
    const int nq = D / 4;
    const int swz = D >= 128 ? 31 : nq - 1;  // slot_swz mask
    constexpr int G = 4;
    auto on = [&](int j) { return FULL || lane + 32 * j < nq; };
    float4 bb[SPL], gg[SPL], be[SPL];
#pragma unroll
    for (int j = 0; j < SPL; j++) {
        const int q = on(j) ? lane + 32 * j : 0;
        bb[j] = reinterpret_cast<const float4*>(bias)[q];
        gg[j] = reinterpret_cast<const float4*>(g)[q];
        be[j] = reinterpret_cast<const float4*>(b)[q];
    }
    // at most four row groups per warp (D <= 128): every group's residual
    // rows are loaded up front, so their latencies overlap instead of
    // adding up group after group
    constexpr int PF = 4;
    float4 xpre[SPL == 1 && PRE ? PF : 1][G];
    const bool prefetched = PRE && SPL == 1 && nrows <= PF * nwarps * G;
    if (SPL == 1 && prefetched && xin) {
#pragma unroll
        for (int i = 0; i < PF; i++)
#pragma unroll
            for (int k = 0; k < G; k++) xpre[SPL == 1 && PRE ? i : 0][k] = xin->v[i][k];
    } else if (SPL == 1 && prefetched) {
#pragma unroll
        for (int i = 0; i < PF; i++) {
            const int r0 = warp * G + i * nwarps * G;
#pragma unroll
            for (int k = 0; k < G; k++) {
                const int row = m0 + r0 + k;
                const int q = on(0) ? lane : 0;
                xpre[SPL == 1 && PRE ? i : 0][k] = r0 < nrows && row < R
                                                ? reinterpret_cast<const float4*>(x + (size_t)row * D)[q]
                                                : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
    }
    int grp = 0;
    for (int r0 = warp * G; r0 < nrows; r0 += nwarps * G, grp++) {
        float4 a[G][SPL], xv[G][SPL];
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int r = r0 + k, row = m0 + r;
#pragma unroll
            for (int j = 0; j < SPL; j++) {
                const int q = on(j) ? lane + 32 * j : 0;
                a[k][j] = reinterpret_cast<const float4*>(tile + (size_t)r * D)[q ^ (r & swz)];
                if (SPL == 1 && prefetched) {
                    float4 t = xpre[0][k];
#pragma unroll
                    for (int i = 1; i < PF; i++)
                        if (grp == i) t = xpre[SPL == 1 && PRE ? i : 0][k];
                    xv[k][j] = t;
                } else {
                    xv[k][j] = row < R ? reinterpret_cast<const float4*>(x + (size_t)row * D)[q]
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
        }
        // the G rows' reductions run interleaved (warp_sum_n): the same
        // order and bits per row as one warp_sum after another
        float4 v[G][SPL];
        float mean[G], q2[G];
#pragma unroll
        for (int k = 0; k < G; k++) {
            float s = 0.f;
#pragma unroll
            for (int j = 0; j < SPL; j++) {
                v[k][j] = resid4(xv[k][j], a[k][j], bb[j]);
                if (on(j)) s = __fadd_rn(s, sum4(v[k][j]));
            }
            mean[k] = s;
        }
        warp_sum_n(mean);
#pragma unroll
        for (int k = 0; k < G; k++) {
            mean[k] = mean[k] / (float)D;
            float t = 0.f;
#pragma unroll
            for (int j = 0; j < SPL; j++)
                if (on(j)) t = __fadd_rn(t, sqdev4(v[k][j], mean[k]));
            q2[k] = t;
        }
        warp_sum_n(q2);
#pragma unroll
        for (int k = 0; k < G; k++) {
            const int row = m0 + r0 + k;
            if (row >= R) break;  // warp-uniform
            const float rstd = ln_rstd(q2[k], D);
#pragma unroll
            for (int j = 0; j < SPL; j++) {
                if (!on(j)) continue;
                const int q = lane + 32 * j;
                reinterpret_cast<float4*>(x + (size_t)row * D)[q] = v[k][j];
                float o[4] = {ln1(v[k][j].x, mean[k], rstd, gg[j].x, be[j].x),
                              ln1(v[k][j].y, mean[k], rstd, gg[j].y, be[j].y),
                              ln1(v[k][j].z, mean[k], rstd, gg[j].z, be[j].z),
                              ln1(v[k][j].w, mean[k], rstd, gg[j].w, be[j].w)};
                if (LNS)  // the MMA A tile in shared memory: [D/8][128][8] core matrices
                    BfVec<4>::store(reinterpret_cast<bf16*>(reinterpret_cast<uint8_t*>(ln) + (size_t)(q >> 1) * 2048 +
                                                            (size_t)(r0 + k) * 16 + (q & 1) * 8), o);
                else
                    BfVec<4>::store(ln + (size_t)row * D + 4 * q, o);
            }
        }
    }
}

// LNS: `ln` is the shared-memory A tile of an MMA (D = 128 only).
template <bool PRE = false, bool LNS = false>
__device__ __forceinline__ void rows_resid_ln_any(const float* tile, int D, int m0, int R, const float* bias, float* x,
                                  const float* g, const float* b, bf16* ln, int warp, int nwarps, int nrows = 128,
                                  const XRows* xin = nullptr) {
    if (LNS) {
        if (D == 128) rows_resid_ln_t<1, true, PRE, true>(tile, D, m0, R, bias, x, g, b, ln, warp, nwarps, nrows, xin);
        return;
    }
    if (D == 256) rows_resid_ln_t<2, true>(tile, D, m0, R, bias, x, g, b, ln, warp, nwarps, nrows);
    else if (D == 128) rows_resid_ln_t<1, true, PRE>(tile, D, m0, R, bias, x, g, b, ln, warp, nwarps, nrows, xin);
    else if (D > 128) rows_resid_ln_t<2, false>(tile, D, m0, R, bias, x, g, b, ln, warp, nwarps, nrows);
    else rows_resid_ln_t<1, false, PRE>(tile, D, m0, R, bias, x, g, b, ln, warp, nwarps, nrows);
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
                                                      const __grid_constant__ CUtensorMap tmO,
                                                      const bf16* __restrict__ Bblk, int K, int BN, int R,
                                                      GemmEpi ep, int* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;                       // [K/8][128][8]
    uint8_t* sB = smem + (size_t)K * 256;     // [K/8][BN][8]
    __shared__ __align__(16) float sbias[256];
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
    if (EPI != EPI_RESID_LN)
        for (int i = threadIdx.x; i < BN; i += blockDim.x) sbias[i] = ep.bias[nb * BN + i];
    tc::tc_fence_before();
    __syncthreads();
    JC_PDL_ENTRY;
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
            // stage the tile (bias added) in 128-byte swizzled boxes of 128
            // rows in the operand shared memory, then store it with TMA
            constexpr int EB = EPI == EPI_BF16 ? 2 : 4;  // bytes per element
            constexpr int PB = 128 / EB;                 // elements per box row
            const int r = threadIdx.x;
            for (int c = 0; c < BN; c += 16) {
                float a[16];
                tc::tmem_ld16(ta + c, a);  // collective: every lane of the warp loads
#pragma unroll
                for (int i = 0; i < 16; i += 4) {
                    const float4 bv = *reinterpret_cast<const float4*>(sbias + c + i);
                    a[i] += bv.x;
                    a[i + 1] += bv.y;
                    a[i + 2] += bv.z;
                    a[i + 3] += bv.w;
                }
                uint8_t* box = smem + (size_t)(c / PB) * 16384 + (size_t)r * 128;
                const int j0 = (c % PB) * EB / 16;  // first 16-byte chunk of these 16 columns
                if (EPI == EPI_BF16) {
                    BfVec<8>::store(reinterpret_cast<bf16*>(box + ((j0 ^ (r & 7)) << 4)), a);
                    BfVec<8>::store(reinterpret_cast<bf16*>(box + (((j0 + 1) ^ (r & 7)) << 4)), a + 8);
                } else {
#pragma unroll
                    for (int q = 0; q < 4; q++)
                        *reinterpret_cast<float4*>(box + (((j0 + q) ^ (r & 7)) << 4)) =
                            make_float4(a[4 * q], a[4 * q + 1], a[4 * q + 2], a[4 * q + 3]);
                }
            }
            tc::fence_async_shared();
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int c = 0; c < BN; c += PB) tc::tma_store_2d(&tmO, smem + (size_t)(c / PB) * 16384, n0 + c, m0);
                tc::bulk_commit();
                tc::bulk_wait_read();
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// Residual + LayerNorm of tile row r by the thread that owns it (TMEM lane
// r): v = x + (acc + bias) in place in the f32 row of sX (128-byte swizzled
// boxes of 32 columns x 128 rows: 16-byte chunk q of row r at box q / 8,
// chunk (q % 8) ^ (r % 8)), then mean and biased variance over the row (two
// passes) and LayerNorm(v) as bf16: into swizzled staging boxes of 64
// columns (sLn) or straight to the global row (lnrow).
__device__ __forceinline__ float4* xrow_chunk(uint8_t* sX, int r, int q) {
    return reinterpret_cast<float4*>(sX + (size_t)(q >> 3) * 16384 + (size_t)r * 128 + (((q & 7) ^ (r & 7)) << 4));
}

// DT > 0: the width as a compile-time constant (every loop unrolled, so the
// shared-memory reads of a pass are all in flight at once); DT = 0: D.
template <int DT>
__device__ void row_resid_ln_t(uint32_t ta, int r, int D_, uint8_t* sX, const float* sbias, const float* sg,
                               const float* sb, uint8_t* sLn, bf16* lnrow) {
    const int D = DT > 0 ? DT : D_;
    // D <= 128: slot q is lane q's only slot, so lane partial q = 0 + sum4
    const int nq = D / 4;
#pragma unroll
    for (int c = 0; c < D; c += 16) {
        float a[16];
        tc::tmem_ld16(ta + c, a);
#pragma unroll
        for (int i = 0; i < 4; i++) {
            float4* p = xrow_chunk(sX, r, (c >> 2) + i);
            const int o = c + 4 * i;
            *p = resid4(*p, make_float4(a[4 * i], a[4 * i + 1], a[4 * i + 2], a[4 * i + 3]),
                        make_float4(sbias[o], sbias[o + 1], sbias[o + 2], sbias[o + 3]));
        }
    }
    float part[32];
#pragma unroll
    for (int l = 0; l < 32; l++) part[l] = l < nq ? __fadd_rn(0.f, sum4(*xrow_chunk(sX, r, l))) : 0.f;
    const float mean = tree32(part) / (float)D;
#pragma unroll
    for (int l = 0; l < 32; l++) part[l] = l < nq ? __fadd_rn(0.f, sqdev4(*xrow_chunk(sX, r, l), mean)) : 0.f;
    const float rstd = ln_rstd(tree32(part), D);
#pragma unroll
    for (int c = 0; c < D; c += 8) {
        const float4 v0 = *xrow_chunk(sX, r, c >> 2), v1 = *xrow_chunk(sX, r, (c >> 2) + 1);
        const float in[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
        float o[8];
#pragma unroll
        for (int i = 0; i < 8; i++) o[i] = ln1(in[i], mean, rstd, sg[c + i], sb[c + i]);
        if (sLn) {
            const int j = (c & 63) >> 3;
            BfVec<8>::store(reinterpret_cast<bf16*>(sLn + (size_t)(c >> 6) * 16384 + (size_t)r * 128 + ((j ^ (r & 7)) << 4)), o);
        } else if (lnrow) {
            BfVec<8>::store(lnrow + c, o);
        }
    }
}

__device__ __forceinline__ void row_resid_ln(uint32_t ta, int r, int D, uint8_t* sX, const float* sbias,
                                             const float* sg, const float* sb, uint8_t* sLn, bf16* lnrow) {
    if (D == 128) row_resid_ln_t<128>(ta, r, D, sX, sbias, sg, sb, sLn, lnrow);
    else row_resid_ln_t<0>(ta, r, D, sX, sbias, sg, sb, sLn, lnrow);
}

constexpr int kLnMaxD = 128;  // widest row the row-per-thread LayerNorm serves

// Fused MLP: x += gelu(LN2(x) @ W1 + b1) @ W2 + b2, then LayerNorm of the new
// x (the next block's norm1, or the final norm) into `ln`. Per chunk of NC
// hidden columns, one after the other, S = A @ W1_chunk (TMEM), h = gelu(S +
// b1) written to shared memory as bf16 by all 8 warps (two per TMEM lane
// quarter, one column half each), O += h @ W2_chunk (TMEM); the hidden
// activations never leave the SM. Every summation order is fixed by
// NC-independent K slices of 16, so every chunk width gives the same bits.
// The residual + LayerNorm epilogue stages O through shared memory and runs
// one warp per row.
//
// PROJ: the block's output projection first (cpu.rs:300-305: x += attn @ Wp
// + bp, then LayerNorm2): the tile's attention rows (TMA, tmP) and Wp (one
// bulk copy into the weight buffers, which need D * D * 2 bytes: dim 128
// with 64-column chunks) give P in the O accumulator; its residual +
// LayerNorm epilogue is the one above (the arithmetic every residual +
// LayerNorm here shares, so the result equals the separate projection
// kernel's bit for bit), with P staged behind sA and the LN2 rows written
// straight into sA as the MLP's A operand (no global round trip). The
// tile's rows of x and ln are only touched by this CTA.
constexpr int kMlpSerialThreads = 256;

template <bool PROJ>
__global__ void __launch_bounds__(kMlpSerialThreads, 2) tc_mlp_serial_kernel(const __grid_constant__ CUtensorMap tmA,
                                                             const bf16* __restrict__ W1, const bf16* __restrict__ W2,
                                                             const float* __restrict__ b1,
                                                             const float* __restrict__ b2, int D, int F, int NC, int R,
                                                             float* __restrict__ x, const float* __restrict__ g,
                                                             const float* __restrict__ b, bf16* __restrict__ ln,
                                                             int* err, const __grid_constant__ CUtensorMap tmP,
                                                             const bf16* __restrict__ Wp, const float* __restrict__ bp,
                                                             const float* __restrict__ g2, const float* __restrict__ be2) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sA = smem;                           // [D/8][128][8]
    uint8_t* sB1 = sA + (size_t)D * 256;          // [D/8][NC][8]
    uint8_t* sB2 = sB1 + (size_t)D * NC * 2;      // [NC/8][D][8]
    uint8_t* sH = sB2 + (size_t)D * NC * 2;       // [NC/8][128][8]
    __shared__ __align__(16) float sb1[1024];
    __shared__ uint64_t bar_a, bar_w1, bar_w2, bar_s, bar_o, bar_p, bar_pm;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int quarter = warp & 3, half = warp >> 2;
    const int m0 = blockIdx.x * 128;
    const uint32_t ncols = D <= 128 ? 256 : 512;
    const uint32_t s_col = D <= 128 ? 128 : 256;  // O in [0, D), S in [s_col, s_col + NC)
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar_p, 1);
        tc::mbar_init(&bar_pm, 1);
        tc::mbar_init(&bar_a, 1);
        tc::mbar_init(&bar_w1, 1);
        tc::mbar_init(&bar_w2, 1);
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
    JC_PDL_ENTRY;
    tc::tc_fence_after();
    const uint32_t tO = tmem_base, tS = tmem_base + s_col;
    const uint32_t a0 = tc::smem_u32(sA), w1s = tc::smem_u32(sB1), w2s = tc::smem_u32(sB2), hs = tc::smem_u32(sH);
    if constexpr (PROJ) {
        // P = attn @ Wp into the O accumulator, then x += P + bp, ln = LN2(x)
        if (threadIdx.x == 0 && !failed) {
            tc::mbar_expect_tx(&bar_p, (uint32_t)D * 256 + (uint32_t)D * D * 2);
            for (int kc = 0; kc < D / 8; kc++) tc::tma_load_2d(sA + kc * 2048, &tmP, kc * 8, m0, &bar_p);
            tc::bulk_load(sB1, Wp, (uint32_t)D * D * 2, &bar_p);
            if (tc::mbar_wait(&bar_p, 0, err, &failed)) {
                tc::tc_fence_after();
                const uint32_t idesc = tc::idesc_bf16(128, D);
                for (int k = 0; k < D / 16; k++)
                    tc::mma_bf16(tO, tc::sdesc(a0 + k * 4096, 2048, 128), tc::sdesc(w1s + k * 2 * D * 16, D * 16, 128),
                                 idesc, k > 0 ? 1u : 0u);
                tc::mma_commit(&bar_pm);
            }
        }
        __syncwarp();
        XRows xr;  // the residual rows, loaded while P is computed
        if (D == 128) load_xrows(x, m0, R, warp, kMlpSerialThreads / 32, 128, xr);
        const bool pok = __syncthreads_and(tc::mbar_wait(&bar_pm, 0, err, &failed) ? 1 : 0) != 0;
        tc::tc_fence_after();
        if (pok) {
            // Wp is consumed: the f32 P tile is staged behind sA, and the LN2
            // rows go straight into sA as the MLP's A operand
            float* tile = reinterpret_cast<float*>(smem + (size_t)D * 256);
            stage_rows(lane_addr(tO), quarter * 32 + lane, D, half * (D / 2), (half + 1) * (D / 2), tile);
            __syncthreads();
            rows_resid_ln_any<true, true>(tile, D, m0, R, bp, x, g2, be2, reinterpret_cast<bf16*>(sA), warp,
                                          kMlpSerialThreads / 32, 128, &xr);
        }
        // the A tile written above is read by the MMAs (async proxy)
        tc::fence_async_shared();
        tc::tc_fence_before();
        __syncthreads();
        tc::tc_fence_after();
    }
    const int nchunks = F / NC;
    const uint32_t wbytes = (uint32_t)D * NC * 2;
    auto issue_s = [&]() {  // S = A @ W1_chunk into tS
        const uint32_t idesc = tc::idesc_bf16(128, NC);
        for (int k = 0; k < D / 16; k++)
            tc::mma_bf16(tS, tc::sdesc(a0 + k * 4096, 2048, 128), tc::sdesc(w1s + k * 2 * NC * 16, NC * 16, 128), idesc,
                         k > 0 ? 1u : 0u);
        tc::mma_commit(&bar_s);
    };
    // Chunk j's critical path is GELU_j then S_{j+1}: W1_{j+1} is loaded as
    // soon as S_j has read W1_j, W2_j once O_{j-1} has read W2_{j-1}, and
    // S_{j+1} is issued right after GELU_j, ahead of O_j. The MMAs and their
    // accumulation order are those of one chunk after another.
    if (threadIdx.x == 0 && !failed) {
        if (!PROJ) {
            tc::mbar_expect_tx(&bar_a, (uint32_t)D * 256);
            for (int kc = 0; kc < D / 8; kc++) tc::tma_load_2d(sA + kc * 2048, &tmA, kc * 8, m0, &bar_a);
        }
        tc::mbar_expect_tx(&bar_w1, wbytes);
        tc::bulk_load(sB1, W1, wbytes, &bar_w1);
        tc::mbar_expect_tx(&bar_w2, wbytes);
        tc::bulk_load(sB2, W2, wbytes, &bar_w2);
        if ((PROJ || tc::mbar_wait(&bar_a, 0, err, &failed)) && tc::mbar_wait(&bar_w1, 0, err, &failed)) {
            tc::tc_fence_after();
            issue_s();
        }
    }
    __syncwarp();
    bool ok = true;
    for (int j = 0; j < nchunks && ok; j++) {
        ok = __syncthreads_and(tc::mbar_wait(&bar_s, j & 1, err, &failed) ? 1 : 0) != 0;
        tc::tc_fence_after();
        if (!ok) break;
        if (threadIdx.x == 0 && !failed && j + 1 < nchunks) {  // S_j has read W1_j
            tc::mbar_expect_tx(&bar_w1, wbytes);
            tc::bulk_load(sB1, W1 + (size_t)(j + 1) * D * NC, wbytes, &bar_w1);
        }
        if (j > 0) {  // O_{j-1} has read h_{j-1} and W2_{j-1}
            ok = __syncthreads_and(tc::mbar_wait(&bar_o, (j - 1) & 1, err, &failed) ? 1 : 0) != 0;
            tc::tc_fence_after();
            if (!ok) break;
            if (threadIdx.x == 0 && !failed) {
                tc::mbar_expect_tx(&bar_w2, wbytes);
                tc::bulk_load(sB2, W2 + (size_t)j * D * NC, wbytes, &bar_w2);
            }
        }
        {
            // h = gelu(S + b1) -> bf16 -> shared memory in the core-matrix layout
            const int r = quarter * 32 + lane;
            const uint32_t ta = lane_addr(tS);
            const int c0 = half * (NC / 2), c1 = c0 + NC / 2;
            for (int c = c0; c < c1; c += 16) {
                float a[16];
                tc::tmem_ld16(ta + c, a);
#pragma unroll
                for (int i = 0; i < 16; i += 2) gelu_fast_pair(a[i], a[i + 1], sb1[j * NC + c + i], sb1[j * NC + c + i + 1]);
                BfVec<8>::store(reinterpret_cast<bf16*>(sH + (size_t)(c / 8) * 2048 + r * 16), a);
                BfVec<8>::store(reinterpret_cast<bf16*>(sH + (size_t)(c / 8 + 1) * 2048 + r * 16), a + 8);
            }
        }
        tc::fence_async_shared();
        tc::tc_fence_before();
        __syncthreads();
        tc::tc_fence_after();
        if (threadIdx.x == 0 && !failed) {
            // S_{j+1} first (tS was read by every GELU thread), then O_j
            if (j + 1 < nchunks && tc::mbar_wait(&bar_w1, (j + 1) & 1, err, &failed)) {
                tc::tc_fence_after();
                issue_s();
            }
            if (!failed && tc::mbar_wait(&bar_w2, j & 1, err, &failed)) {
                tc::tc_fence_after();
                const uint32_t idesc = tc::idesc_bf16(128, D);
                for (int k = 0; k < NC / 16; k++)
                    tc::mma_bf16(tO, tc::sdesc(hs + k * 4096, 2048, 128), tc::sdesc(w2s + k * 2 * D * 16, D * 16, 128),
                                 idesc, (j > 0 || k > 0) ? 1u : 0u);
                tc::mma_commit(&bar_o);
            }
        }
        __syncwarp();
    }
    XRows xr2;  // the residual rows (this CTA wrote them above, or an earlier kernel), loaded while the last O runs
    if (D == 128) load_xrows(x, m0, R, warp, kMlpSerialThreads / 32, 128, xr2);
    if (ok) {  // the last O
        ok = __syncthreads_and(tc::mbar_wait(&bar_o, (nchunks - 1) & 1, err, &failed) ? 1 : 0) != 0;
        tc::tc_fence_after();
    }
    if (ok) {
        // every MMA is complete: reuse the operand shared memory for the f32 O tile
        float* tile = reinterpret_cast<float*>(smem);
        stage_rows(lane_addr(tO), quarter * 32 + lane, D, half * (D / 2), (half + 1) * (D / 2), tile);
        __syncthreads();
        rows_resid_ln_any<true>(tile, D, m0, R, b2, x, g, b, ln, warp, kMlpSerialThreads / 32, 128,
                                D == 128 ? &xr2 : nullptr);
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem_base, ncols);
}

// One decision for the `n` threads (whole warps) that meet at named barrier `bar`.
__device__ __forceinline__ bool all_of(bool v, int bar, int n) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbarrier.red.and.pred p, %2, %3, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"(v ? 1u : 0u), "r"(bar), "r"(n)
        : "memory");
    return r != 0;
}


// Persistent output projection + residual + LayerNorm (cpu.rs:300-313) for
// dims up to 128: x += attn @ Wp + bp, ln = LayerNorm2(x). One CTA per SM
// walks row tiles with its stages on separate warps:
//   warp 0     (one lane) TMA-loads each tile's attention rows and f32
//              residual rows (128-byte swizzled boxes) into one of two slots;
//   warp 1     (one lane) loads Wp once and issues each tile's MMAs into one
//              of two TMEM accumulators;
//   warps 2-5  thread r owns tile row r: the residual update in place in the
//              slot's x rows, the LayerNorm (row_resid_ln, the shared
//              arithmetic), ln rows straight to global, the new x rows back
//              with a TMA store.
constexpr int kPLThreads = 6 * 32;

struct PLSmem {
    size_t b, a, x, total;
    __host__ __device__ explicit PLSmem(int D) {
        b = 0;                                             // Wp [D/8][D][8]
        a = (size_t)D * D * 2;                             // 2 x [D/8][128][8]
        x = (a + 2 * (size_t)D * 256 + 1023) / 1024 * 1024;  // 2 x D/32 boxes of 32 f32 x 128 rows
        total = x + 2 * (size_t)D * 512;
    }
};

__global__ void __launch_bounds__(kPLThreads, 1) tc_projln_persistent_kernel(
    const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmX, const bf16* __restrict__ Wp,
    const float* __restrict__ bias, const float* __restrict__ gam, const float* __restrict__ bet,
    bf16* __restrict__ ln, int D, int R, int* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const PLSmem L(D);
    uint8_t* sB = smem + L.b;
    uint8_t* sA = smem + L.a;
    uint8_t* sX = smem + L.x;
    __shared__ uint64_t b_full, in_full[2], in_empty[2], acc_full[2], acc_empty[2];
    __shared__ __align__(16) float sbias[kLnMaxD], sg[kLnMaxD], sb[kLnMaxD];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n_tiles = (R + 127) / 128;
    const int my_tiles = (int)blockIdx.x < n_tiles ? (n_tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const uint32_t ncols = D <= 32 ? 64 : (D <= 64 ? 128 : 256);  // two accumulators
    if (threadIdx.x == 0) {
        tc::mbar_init(&b_full, 1);
        for (int i = 0; i < 2; i++) {
            tc::mbar_init(&in_full[i], 1);
            tc::mbar_init(&in_empty[i], 2);  // the MMAs have read A, the epilogue's store has read x
            tc::mbar_init(&acc_full[i], 1);
            tc::mbar_init(&acc_empty[i], 4 * 32);
        }
        tc::fence_barrier_init();
        failed = 0;
        if ((tc::smem_u32(smem) & 1023u) || D > kLnMaxD || D % 32) {
            failed = 1;
            atomicExch(err, 2);
        }
    }
    for (int i = threadIdx.x; i < D; i += blockDim.x) {
        sbias[i] = bias[i];
        sg[i] = gam[i];
        sb[i] = bet[i];
    }
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    tc::tc_fence_before();
    __syncthreads();
    JC_PDL_ENTRY;
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    const size_t a_bytes = (size_t)D * 256, x_bytes = (size_t)D * 512;
    if (warp == 0) {
        if (lane == 0 && !failed) {
            for (int it = 0; it < my_tiles; it++) {
                const int s = it & 1;
                if (it >= 2 && !tc::mbar_wait(&in_empty[s], (uint32_t)((it - 2) >> 1) & 1u, err, &failed)) break;
                const int m0 = ((int)blockIdx.x + it * (int)gridDim.x) * 128;
                tc::mbar_expect_tx(&in_full[s], (uint32_t)(a_bytes + x_bytes));
                for (int kc = 0; kc < D / 8; kc++)
                    tc::tma_load_2d(sA + s * a_bytes + kc * 2048, &tmA, kc * 8, m0, &in_full[s]);
                for (int bx = 0; bx < D / 32; bx++)
                    tc::tma_load_2d(sX + s * x_bytes + bx * 16384, &tmX, bx * 32, m0, &in_full[s]);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0 && !failed) {
            tc::mbar_expect_tx(&b_full, (uint32_t)D * D * 2);
            tc::bulk_load(sB, Wp, (uint32_t)D * D * 2, &b_full);
            bool good = tc::mbar_wait(&b_full, 0, err, &failed);
            const uint32_t idesc = tc::idesc_bf16(128, D);
            const uint32_t b0 = tc::smem_u32(sB);
            for (int it = 0; it < my_tiles && good; it++) {
                const int s = it & 1;
                good = tc::mbar_wait(&in_full[s], (uint32_t)(it >> 1) & 1u, err, &failed) &&
                       (it < 2 || tc::mbar_wait(&acc_empty[s], (uint32_t)((it - 2) >> 1) & 1u, err, &failed));
                if (!good) break;
                tc::tc_fence_after();
                const uint32_t a0 = tc::smem_u32(sA + s * a_bytes);
                const uint32_t acc = tmem + (uint32_t)s * D;
                for (int k = 0; k < D / 16; k++)
                    tc::mma_bf16(acc, tc::sdesc(a0 + k * 4096, 2048, 128), tc::sdesc(b0 + k * 2 * D * 16, D * 16, 128),
                                 idesc, k > 0 ? 1u : 0u);
                tc::mma_commit(&in_empty[s]);
                tc::mma_commit(&acc_full[s]);
            }
        }
        __syncwarp();
    } else {
        const int r = (warp & 3) * 32 + lane;
        const bool leader = warp == 2 && lane == 0;
        for (int it = 0; it < my_tiles; it++) {
            const int s = it & 1;
            const bool ready = tc::mbar_wait(&acc_full[s], (uint32_t)(it >> 1) & 1u, err, &failed) &&
                               tc::mbar_wait(&in_full[s], (uint32_t)(it >> 1) & 1u, err, &failed);
            if (!all_of(ready, 1, 128)) break;
            tc::tc_fence_after();
            const int m0 = ((int)blockIdx.x + it * (int)gridDim.x) * 128;
            const int row = m0 + r;
            row_resid_ln(lane_addr(tmem + (uint32_t)s * D), r, D, sX + s * x_bytes, sbias, sg, sb, nullptr,
                         row < R ? ln + (size_t)row * D : nullptr);
            tc::tc_fence_before();
            tc::mbar_arrive(&acc_empty[s]);
            tc::fence_async_shared();
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (leader) {
                for (int bx = 0; bx < D / 32; bx++) tc::tma_store_2d(&tmX, sX + s * x_bytes + bx * 16384, bx * 32, m0);
                tc::bulk_commit();
                tc::bulk_wait_read();
                tc::mbar_arrive(&in_empty[s]);
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// Persistent q/k/v projection (cpu.rs:291-297, the three linears as one GEMM
// over the concatenated weights): one CTA per SM walks row tiles; the whole
// weight matrix stays in shared memory. Items are (tile, N block):
//   warp 0     (one lane) TMA-loads each tile's LayerNorm rows into one of two
//              slots;
//   warp 1     (one lane) loads the weights once and issues each item's MMAs
//              into one of two TMEM accumulators;
//   warps 2-5  add the bias, round to bf16 into one of two 128-byte swizzled
//              staging areas and store the item with TMA.
constexpr int kQKVPThreads = 6 * 32;

struct QKVPSmem {
    size_t b, a, stage, total;
    __host__ __device__ QKVPSmem(int D, int BN) {
        b = 0;                                            // [3D/BN][D/8][BN][8]
        a = (size_t)3 * D * D * 2;                        // 2 x [D/8][128][8]
        stage = (a + 2 * (size_t)D * 256 + 1023) / 1024 * 1024;  // 2 x ceil(BN/64) boxes of 16 KB
        total = stage + 2 * (size_t)((BN + 63) / 64) * 16384;
    }
};

__global__ void __launch_bounds__(kQKVPThreads, 1) tc_qkv_persistent_kernel(
    const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmO, const bf16* __restrict__ W,
    const float* __restrict__ bias, int D, int BN, int R, int* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    const QKVPSmem L(D, BN);
    uint8_t* sB = smem + L.b;
    uint8_t* sA = smem + L.a;
    uint8_t* sStage = smem + L.stage;
    __shared__ uint64_t b_full, a_full[2], a_empty[2], acc_full[2], acc_empty[2];
    __shared__ __align__(16) float sbias[3 * 128];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int NB = 3 * D / BN;
    const int n_tiles = (R + 127) / 128;
    const int my_tiles = (int)blockIdx.x < n_tiles ? (n_tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int total = my_tiles * NB;
    uint32_t ncols = 32;
    while (ncols < 2u * BN) ncols <<= 1;
    const size_t a_bytes = (size_t)D * 256, st_bytes = (size_t)((BN + 63) / 64) * 16384;
    if (threadIdx.x == 0) {
        tc::mbar_init(&b_full, 1);
        for (int i = 0; i < 2; i++) {
            tc::mbar_init(&a_full[i], 1);
            tc::mbar_init(&a_empty[i], 1);
            tc::mbar_init(&acc_full[i], 1);
            tc::mbar_init(&acc_empty[i], 4 * 32);
        }
        tc::fence_barrier_init();
        failed = 0;
        if ((tc::smem_u32(smem) & 1023u) || D > 128 || 3 * D % BN || ncols > 512) {
            failed = 1;
            atomicExch(err, 2);
        }
    }
    for (int i = threadIdx.x; i < 3 * D && i < 3 * 128; i += blockDim.x) sbias[i] = bias[i];
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    tc::tc_fence_before();
    __syncthreads();
    JC_PDL_ENTRY;
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    if (warp == 0) {
        if (lane == 0 && !failed) {
            for (int it = 0; it < my_tiles; it++) {
                const int s = it & 1;
                if (it >= 2 && !tc::mbar_wait(&a_empty[s], (uint32_t)((it - 2) >> 1) & 1u, err, &failed)) break;
                const int m0 = ((int)blockIdx.x + it * (int)gridDim.x) * 128;
                tc::mbar_expect_tx(&a_full[s], (uint32_t)a_bytes);
                for (int kc = 0; kc < D / 8; kc++)
                    tc::tma_load_2d(sA + s * a_bytes + kc * 2048, &tmA, kc * 8, m0, &a_full[s]);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0 && !failed) {
            tc::mbar_expect_tx(&b_full, (uint32_t)3 * D * D * 2);
            tc::bulk_load(sB, W, (uint32_t)3 * D * D * 2, &b_full);
            bool good = tc::mbar_wait(&b_full, 0, err, &failed);
            const uint32_t idesc = tc::idesc_bf16(128, BN);
            const uint32_t b0 = tc::smem_u32(sB);
            for (int g = 0; g < total && good; g++) {
                const int it = g / NB, nb = g % NB, s = it & 1;
                if (nb == 0) good = tc::mbar_wait(&a_full[s], (uint32_t)(it >> 1) & 1u, err, &failed);
                if (good && g >= 2) good = tc::mbar_wait(&acc_empty[g & 1], (uint32_t)((g - 2) >> 1) & 1u, err, &failed);
                if (!good) break;
                tc::tc_fence_after();
                const uint32_t a0 = tc::smem_u32(sA + s * a_bytes);
                const uint32_t bb = b0 + (uint32_t)nb * D * BN * 2;
                const uint32_t acc = tmem + (uint32_t)(g & 1) * BN;
                for (int k = 0; k < D / 16; k++)
                    tc::mma_bf16(acc, tc::sdesc(a0 + k * 4096, 2048, 128), tc::sdesc(bb + k * 2 * BN * 16, BN * 16, 128),
                                 idesc, k > 0 ? 1u : 0u);
                tc::mma_commit(&acc_full[g & 1]);
                if (nb == NB - 1) tc::mma_commit(&a_empty[s]);  // the tile's last read of A
            }
        }
        __syncwarp();
    } else {
        const int r = (warp & 3) * 32 + lane;
        const bool leader = warp == 2 && lane == 0;
        for (int g = 0; g < total; g++) {
            const int it = g / NB, nb = g % NB;
            const bool ready = tc::mbar_wait(&acc_full[g & 1], (uint32_t)(g >> 1) & 1u, err, &failed);
            if (!all_of(ready, 1, 128)) break;
            tc::tc_fence_after();
            // the staging area used two items ago must have been read by its store
            if (leader && g >= 2) tc::bulk_wait_read_1();
            asm volatile("bar.sync 1, 128;" ::: "memory");
            uint8_t* st = sStage + (size_t)(g & 1) * st_bytes;
            const uint32_t ta = lane_addr(tmem + (uint32_t)(g & 1) * BN);
            // 32 columns per TMEM round trip (BN is a multiple of 32)
            for (int c = 0; c < BN; c += 32) {
                float a[32];
                tc::tmem_ld32(ta + c, a);
#pragma unroll
                for (int i = 0; i < 32; i += 4) {
                    const float4 bv = *reinterpret_cast<const float4*>(sbias + nb * BN + c + i);
                    a[i] += bv.x;
                    a[i + 1] += bv.y;
                    a[i + 2] += bv.z;
                    a[i + 3] += bv.w;
                }
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int cc = c + 16 * h;
                    uint8_t* box = st + (size_t)(cc / 64) * 16384 + (size_t)r * 128;
                    const int j0 = (cc % 64) / 8;
                    BfVec<8>::store(reinterpret_cast<bf16*>(box + ((j0 ^ (r & 7)) << 4)), a + 16 * h);
                    BfVec<8>::store(reinterpret_cast<bf16*>(box + (((j0 + 1) ^ (r & 7)) << 4)), a + 16 * h + 8);
                }
            }
            tc::tc_fence_before();
            tc::mbar_arrive(&acc_empty[g & 1]);
            tc::fence_async_shared();
            asm volatile("bar.sync 1, 128;" ::: "memory");
            if (leader) {
                const int m0 = ((int)blockIdx.x + it * (int)gridDim.x) * 128;
                for (int c = 0; c < BN; c += 64) tc::tma_store_2d(&tmO, st + (size_t)(c / 64) * 16384, nb * BN + c, m0);
                tc::bulk_commit();
            }
        }
        if (leader) tc::bulk_wait_read();
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// 3x3 zero-padded convolution over each instance's grid as an implicit GEMM
// (cpu.rs:171-205): tile = 8 x 16 positions (M = 128, row r <-> position
// (y0 + r/8, x0 + r%8)); the halo tile [C/8 planes][18][10][8] is loaded by
// TMA (zero fill outside the grid); tap (ky, kx) is the halo addressed from
// offset (ky*10 + kx)*16 bytes. B per tap: [C/8][BN][8] (the N block `nb`).
// Epilogue (token_mix): out = xn + gelu(acc + b) (cpu.rs:326-328), bf16. The
// cell-head convolutions have their own persistent kernel (tc_cellconv_kernel).
enum { CONV_TOKMIX = 0 };

// Shared memory of tc_conv3_kernel: the halo planes, then NS tap weight
// blocks; with NS = 9 every tap is resident and loaded once.
static __host__ __device__ size_t conv3_smem(int C, int BN, int NS) {
    return (size_t)(C / 8) * kHaloPlane + (size_t)NS * C * BN * 2;
}
// Where the epilogue stages its output boxes: after the halo (1024-aligned,
// for the 128-byte swizzle) when the halo is still read (token mix), else at
// the start.
static __host__ __device__ size_t conv3_stage_offset(int C, bool after_halo) {
    return after_halo ? ((size_t)(C / 8) * kHaloPlane + 1023) / 1024 * 1024 : 0;
}
// Dynamic shared memory of a launch: operands, or the staged output boxes
// (128 bytes of channels each, eb bytes per element) if those need more.
static size_t conv3_launch_smem(int C, int BN, int NS, int eb) {
    const size_t boxes = (size_t)((BN * eb + 127) / 128);
    return std::max(conv3_smem(C, BN, NS), conv3_stage_offset(C, eb == 2) + boxes * 16384);
}

template <int KIND>
__global__ void __launch_bounds__(128) tc_conv3_kernel(const CUtensorMap* __restrict__ maps, int map_slot,
                                                       int store_slot, const bf16* __restrict__ Wt,
                                                       const float* __restrict__ bias, int C, int BN, int NS,
                                                       const InstDev* inst, int n_inst, int* err) {
    static_assert(KIND == CONV_TOKMIX, "token_mix only");
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sHalo = smem;                                   // [C/8][18][10][8]
    uint8_t* sB = smem + (size_t)(C / 8) * kHaloPlane;       // NS x [C/8][BN][8]
    constexpr int kMaxNS = 9;
    __shared__ uint64_t bar_h, bar_b[kMaxNS], bar_m[kMaxNS], bar_done;
    __shared__ __align__(16) float sbias[256];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    const int warp = threadIdx.x >> 5;
    // tile -> instance
    const int tile = blockIdx.x, nb = blockIdx.y;
    const int lo = warp_find_last_le(n_inst, tile, [&](int i) {
        return (long long)inst[i].tt0;
    });
    const InstDev I = inst[lo];
    const int gw = I.tx;
    const int tiles_x = (gw + kConvTX - 1) / kConvTX;
    const int tl = tile - I.tt0;
    const int x0 = (tl % tiles_x) * kConvTX, y0 = (tl / tiles_x) * kConvTY;
    const CUtensorMap* map = maps + kMapsPerInst * lo + map_slot;
    const CUtensorMap* omap = maps + kMapsPerInst * lo + store_slot;
    const uint32_t ncols = BN <= 32 ? 32 : (BN <= 64 ? 64 : (BN <= 128 ? 128 : 256));
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar_h, 1);
        tc::mbar_init(&bar_done, 1);
        for (int i = 0; i < kMaxNS; i++) {
            tc::mbar_init(&bar_b[i], 1);
            tc::mbar_init(&bar_m[i], 1);
        }
        tc::fence_barrier_init();
        failed = 0;
        if ((tc::smem_u32(smem) & 1023u) || NS < 2 || NS > kMaxNS) {  // aligned operand tiles
            failed = 1;
            atomicExch(err, 2);
        }
    }
    for (int i = threadIdx.x; i < BN; i += blockDim.x) sbias[i] = bias[nb * BN + i];
    if (warp == 0) tc::tmem_alloc(&tmem_base, ncols);
    tc::tc_fence_before();
    __syncthreads();
    JC_PDL_ENTRY;
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t wtap = (uint32_t)C * BN * 2;  // bytes of one tap's B block
    const bf16* Wn = Wt + (size_t)nb * 9 * C * BN;
    if (threadIdx.x == 0 && !failed) {
        tc::tensormap_acquire(map);
        tc::tensormap_acquire(omap);
        tc::mbar_expect_tx(&bar_h, (uint32_t)(C / 8) * (kHaloW * kHaloH * 16));
        for (int kc = 0; kc < C / 8; kc++)
            tc::tma_load_3d(sHalo + kc * kHaloPlane, map, kc * 8, x0 - 1, y0 - 1, &bar_h);
        for (int t = 0; t < NS && t < 9; t++) {
            tc::mbar_expect_tx(&bar_b[t], wtap);
            tc::bulk_load(sB + t * wtap, Wn + (size_t)t * C * BN, wtap, &bar_b[t]);
        }
        bool good = tc::mbar_wait(&bar_h, 0, err, &failed);
        const uint32_t idesc = tc::idesc_bf16(128, BN);
        const uint32_t h0 = tc::smem_u32(sHalo);
        for (int t = 0; t < 9 && good; t++) {
            const int buf = t % NS;
            good = tc::mbar_wait(&bar_b[buf], (uint32_t)(t / NS) & 1u, err, &failed);
            if (!good) break;
            tc::tc_fence_after();
            const int ky = t / 3, kx = t % 3;
            const uint32_t b0 = tc::smem_u32(sB + buf * wtap);
            for (int k = 0; k < C / 16; k++) {
                uint64_t ad = tc::sdesc(h0 + 2 * k * kHaloPlane + (ky * kHaloW + kx) * 16, kHaloPlane, kHaloW * 16);
                uint64_t bd = tc::sdesc(b0 + 2 * k * BN * 16, BN * 16, 128);
                tc::mma_bf16(tmem, ad, bd, idesc, (t > 0 || k > 0) ? 1u : 0u);
            }
            if (t + NS < 9) {
                // the stage is refilled once the MMAs reading it are done
                tc::mma_commit(&bar_m[buf]);
                good = tc::mbar_wait(&bar_m[buf], (uint32_t)(t / NS) & 1u, err, &failed);
                if (!good) break;
                tc::mbar_expect_tx(&bar_b[buf], wtap);
                tc::bulk_load(sB + buf * wtap, Wn + (size_t)(t + NS) * C * BN, wtap, &bar_b[buf]);
            }
        }
        if (good) tc::mma_commit(&bar_done);  // arrives when every MMA above is done
    }
    __syncwarp();
    const bool ok = __syncthreads_and(tc::mbar_wait(&bar_done, 0, err, &failed) ? 1 : 0) != 0;
    tc::tc_fence_after();
    if (ok) {
        // epilogue into 128-byte swizzled boxes of the 128 tile positions
        // (row r = position (y0 + r / 8, x0 + r % 8)), stored with TMA;
        // positions outside the grid are clipped by the store
        const int r = threadIdx.x;
        const uint32_t ta = lane_addr(tmem);
        constexpr int EB = 2;        // bytes per output element (bf16)
        constexpr int PB = 128 / EB;  // elements per box row
        // the epilogue still reads the halo centre, so it stages after the halo
        uint8_t* stage = smem + conv3_stage_offset(C, true);
        for (int c = 0; c < BN; c += 16) {
            float a[16];
            tc::tmem_ld16(ta + c, a);
            // the centre of the halo tile is xn at this token
            const uint8_t* centre = sHalo + ((r / kConvTX + 1) * kHaloW + (r % kConvTX + 1)) * 16;
            const int n0 = nb * BN;
#pragma unroll
            for (int i = 0; i < 16; i += 2) gelu_fast_pair(a[i], a[i + 1], sbias[c + i], sbias[c + i + 1]);
#pragma unroll
            for (int i = 0; i < 16; i++) {
                const int ch = n0 + c + i;
                const float xn = bf2f(*reinterpret_cast<const bf16*>(centre + (size_t)(ch / 8) * kHaloPlane + (ch % 8) * 2));
                a[i] = xn + a[i];
            }
            uint8_t* box = stage + (size_t)(c / PB) * 16384 + (size_t)r * 128;
            const int j0 = (c % PB) * EB / 16;
            BfVec<8>::store(reinterpret_cast<bf16*>(box + ((j0 ^ (r & 7)) << 4)), a);
            BfVec<8>::store(reinterpret_cast<bf16*>(box + (((j0 + 1) ^ (r & 7)) << 4)), a + 8);
        }
        tc::fence_async_shared();
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int c = 0; c < BN; c += PB)
                tc::tma_store_3d(omap, stage + (size_t)(c / PB) * 16384, nb * BN + c, x0, y0);
            tc::bulk_commit();
            tc::bulk_wait_read();
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// Persistent cell-head convolutions on the tensor cores, one CTA walking
// cell tiles tile = blockIdx.x + k gridDim.x with its stages on separate
// warps, so the halo loads, the MMAs and the epilogue of consecutive tiles
// overlap:
//   warp 0     (one lane) TMA-loads each tile's halo into one of two slots;
//   warp 1     (one lane) issues a tile's MMAs into one of two TMEM
//              accumulators (the weights stay resident);
//   warps 2-5  (one TMEM lane quarter each) run the epilogue.
// kCellConv1, conv1 (cpu.rs:343-346): the 3x3 conv of the cell-head input zc
// (48 f16 channels) to 32 channels as 9 taps x 3 MMAs (tap (ky, kx) is the
// halo tile addressed from position (ky, kx)), + bias, GELU, stored as f16
// (c1) through one staged box (the next tile's epilogue waits until the
// store has read it) and a TMA store; the MMA order and the epilogue
// arithmetic are those of tc_conv3_kernel.
// kCellConv2, conv2 and the step (cpu.rs:347-348, 84-88): 32 -> 3 channels.
// With 3 outputs the per-tap form would re-read the whole halo tile from
// shared memory for 9 tiny MMAs; instead one GEMM gives every halo position
// p its 27 tap contributions Z[p][(ky, kx), co] = c1[p] . W[co][.][ky][kx]
// (M = the 180 halo positions in two 128-row MMAs, N = 32 with 5 zero
// columns, K = 32 f16 channels, f32 sums), the epilogue stages Z in shared
// memory and each output cell adds its nine neighbours' contributions in
// tap order, + bias, + the state when the tick writes the next state, into
// the instance's planar output. Its f16 operands and sum order make it the
// BF16 form's own conv2 (the FP32 path keeps the reference's f32 order).
constexpr int kC1PThreads = 6 * 32;
constexpr int kCellConv1 = 0, kCellConv2 = 1;

// halo tiles in flight per CTA: two, so that three conv1 CTAs (four conv2
// CTAs) fit on an SM, which measured faster than three stages at two (three)
constexpr int kC1PHaloStages = 2;
constexpr int kHaloPos = kHaloW * kHaloH;  // 180 halo positions
constexpr int kZPitch = 33;                // f32 per staged Z row (bank-conflict-free column reads)

// TMEM columns per accumulator, weight bytes and staged bytes of each kind.
__host__ __device__ constexpr int cellconv_bn(int kind) { return kind == kCellConv1 ? 32 : 64; }
__host__ __device__ constexpr size_t cellconv_wbytes(int kind, int C) {
    return kind == kCellConv1 ? (size_t)9 * C * 32 * 2 : (size_t)C * 32 * 2;
}
__host__ __device__ constexpr size_t cellconv_stage(int kind) {
    return kind == kCellConv1 ? (size_t)128 * 32 * 2 : (size_t)kHaloPos * kZPitch * 4;
}

struct C1PSmem {
    size_t halo, w, stage, total;
    __host__ __device__ C1PSmem(int kind, int C) {
        halo = 0;                                                          // stages x [C/8][18][10][8]
        w = halo + (size_t)kC1PHaloStages * (C / 8) * kCellPlane;          // the weight blocks
        stage = (w + cellconv_wbytes(kind, C) + 1023) / 1024 * 1024;       // staged output
        total = stage + cellconv_stage(kind);
    }
};

template <int KIND>
__global__ void __launch_bounds__(kC1PThreads) tc_cellconv_kernel(const CUtensorMap* __restrict__ maps,
                                                                   const bf16* __restrict__ Wt,
                                                                   const float* __restrict__ bias, int C,
                                                                   int n_tiles, const InstDev* inst, int n_inst,
                                                                   int mode, int* err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr int BN = cellconv_bn(KIND);
    constexpr int kInSlot = KIND == kCellConv1 ? 1 : 6;  // zc halo | c1 halo
    const C1PSmem L(KIND, C);
    uint8_t* sHalo = smem + L.halo;
    uint8_t* sW = smem + L.w;
    uint8_t* sStage = smem + L.stage;
    const size_t halo_bytes = (size_t)(C / 8) * kCellPlane;
    const uint32_t wbytes = (uint32_t)cellconv_wbytes(KIND, C);
    constexpr int HS = kC1PHaloStages;
    constexpr int kBias = KIND == kCellConv1 ? 32 : 3;
    __shared__ uint64_t w_full, h_full[HS], h_empty[HS], a_full[2], a_empty[2];
    __shared__ __align__(16) float sbias[32];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int my_tiles = (int)blockIdx.x < n_tiles ? (n_tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (threadIdx.x == 0) {
        tc::mbar_init(&w_full, 1);
        for (int i = 0; i < HS; i++) {
            tc::mbar_init(&h_full[i], 1);
            tc::mbar_init(&h_empty[i], 1);
        }
        for (int i = 0; i < 2; i++) {
            tc::mbar_init(&a_full[i], 1);
            tc::mbar_init(&a_empty[i], 4 * 32);
        }
        tc::fence_barrier_init();
        failed = 0;
        if (tc::smem_u32(smem) & 1023u) {
            failed = 1;
            atomicExch(err, 2);
        }
    }
    if (threadIdx.x < 32) sbias[threadIdx.x] = (int)threadIdx.x < kBias ? bias[threadIdx.x] : 0.f;
    if (warp == 0) tc::tmem_alloc(&tmem_base, 2 * BN);
    tc::tc_fence_before();
    __syncthreads();
    JC_PDL_ENTRY;
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    // tile -> (instance, origin)
    auto locate = [&](int tile, int& ii, int& x0, int& y0) {
        int lo = 0, hi = n_inst - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (inst[mid].ct0 <= tile) lo = mid; else hi = mid - 1;
        }
        ii = lo;
        const InstDev& I = inst[lo];
        const int tiles_x = (I.nx + kConvTX - 1) / kConvTX;
        const int tl = tile - I.ct0;
        x0 = (tl % tiles_x) * kConvTX;
        y0 = (tl / tiles_x) * kConvTY;
    };
    if (warp == 0) {
        if (lane == 0 && !failed) {
            // halo producer
            for (int it = 0; it < my_tiles; it++) {
                const int hb = it % HS;
                if (it >= HS && !tc::mbar_wait(&h_empty[hb], (uint32_t)((it - HS) / HS) & 1u, err, &failed)) break;
                int ii, x0, y0;
                locate((int)blockIdx.x + it * (int)gridDim.x, ii, x0, y0);
                const CUtensorMap* map = maps + kMapsPerInst * ii + kInSlot;
                tc::tensormap_acquire(map);
                tc::mbar_expect_tx(&h_full[hb], (uint32_t)halo_bytes);
                tc::tma_load_3d(sHalo + hb * halo_bytes, map, (x0 - 1) * 8, y0 - 1, 0, &h_full[hb]);
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        if (lane == 0 && !failed) {
            // MMA issuer: the weights once, then every tile
            tc::mbar_expect_tx(&w_full, wbytes);
            tc::bulk_load(sW, Wt, wbytes, &w_full);
            bool good = tc::mbar_wait(&w_full, 0, err, &failed);
            const uint32_t idesc = tc::idesc_f16(128, 32);  // f16 input and weights, N = 32
            const uint32_t w0 = tc::smem_u32(sW);
            for (int it = 0; it < my_tiles && good; it++) {
                const int b = it & 1, hb = it % HS;
                good = tc::mbar_wait(&h_full[hb], (uint32_t)(it / HS) & 1u, err, &failed) &&
                       (it < 2 || tc::mbar_wait(&a_empty[b], (uint32_t)((it - 2) >> 1) & 1u, err, &failed));
                if (!good) break;
                tc::tc_fence_after();
                const uint32_t h0 = tc::smem_u32(sHalo + hb * halo_bytes);
                const uint32_t acc = tmem + (uint32_t)b * BN;
                if constexpr (KIND == kCellConv1) {
                    // rows = the 8 x 16 output positions (8-row groups 10 positions apart)
                    for (int t = 0; t < 9; t++) {
                        const int ky = t / 3, kx = t % 3;
                        const uint32_t b0 = w0 + (uint32_t)t * C * 32 * 2;
                        for (int k = 0; k < C / 16; k++) {
                            uint64_t ad = tc::sdesc(h0 + 2 * k * kCellPlane + (ky * kHaloW + kx) * 16, kCellPlane,
                                                    kHaloW * 16);
                            uint64_t bd = tc::sdesc(b0 + 2 * k * 32 * 16, 32 * 16, 128);
                            tc::mma_bf16(acc, ad, bd, idesc, (t > 0 || k > 0) ? 1u : 0u);
                        }
                    }
                } else {
                    // rows = halo positions 0..127 and 128..255 (those past 179,
                    // read past the plane, are never used)
                    for (int m = 0; m < 2; m++)
                        for (int k = 0; k < C / 16; k++) {
                            uint64_t ad = tc::sdesc(h0 + 2 * k * kCellPlane + m * 128 * 16, kCellPlane, 128);
                            uint64_t bd = tc::sdesc(w0 + 2 * k * 32 * 16, 32 * 16, 128);
                            tc::mma_bf16(acc + (uint32_t)m * 32, ad, bd, idesc, k > 0 ? 1u : 0u);
                        }
                }
                tc::mma_commit(&h_empty[hb]);
                tc::mma_commit(&a_full[b]);
            }
        }
        __syncwarp();
    } else {
        // epilogue: thread r = TMEM lane r
        const int r = (warp & 3) * 32 + lane;
        const bool leader = warp == 2 && lane == 0;
        for (int it = 0; it < my_tiles; it++) {
            const int b = it & 1;
            // the tile's instance, origin and (conv2) state, fetched before
            // the wait so their latency overlaps the MMAs
            const int tile = (int)blockIdx.x + it * (int)gridDim.x;
            const int ii = warp_find_last_le(n_inst, tile, [&](int i) { return (long long)inst[i].ct0; });
            const InstDev I = inst[ii];
            const int tiles_x = (I.nx + kConvTX - 1) / kConvTX;
            const int x0 = ((tile - I.ct0) % tiles_x) * kConvTX, y0 = ((tile - I.ct0) / tiles_x) * kConvTY;
            const int x = x0 + (r & 7), y = y0 + (r >> 3);
            const bool inside = x < I.nx && y < I.ny;
            const size_t plane = (size_t)I.nx * I.ny, cl = inside ? (size_t)y * I.nx + x : 0;
            float st[3] = {0.f, 0.f, 0.f};
            if (KIND == kCellConv2 && inside && mode == kWriteNextState) {
#pragma unroll
                for (int co = 0; co < 3; co++) st[co] = I.state[co * plane + cl];
            }
            const bool ready = tc::mbar_wait(&a_full[b], (uint32_t)(it >> 1) & 1u, err, &failed);
            uint32_t all_ready;
            asm volatile(
                "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbarrier.red.and.pred p, 1, 128, q;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(all_ready)
                : "r"(ready ? 1u : 0u)
                : "memory");
            if (!all_ready) break;
            tc::tc_fence_after();
            const uint32_t ta = lane_addr(tmem + (uint32_t)b * BN);
            if constexpr (KIND == kCellConv2) {
                // Z rows r and 128 + r -> shared memory, then output cell r
                float* Z = reinterpret_cast<float*>(sStage);
#pragma unroll
                for (int m = 0; m < 2; m++) {
                    float a[32];
                    tc::tmem_ld32(ta + m * 32, a);
                    const int pos = m * 128 + r;
                    if (pos < kHaloPos) {
#pragma unroll
                        for (int c = 0; c < 27; c++) Z[pos * kZPitch + c] = a[c];
                    }
                }
                tc::tc_fence_before();
                tc::mbar_arrive(&a_empty[b]);
                asm volatile("bar.sync 1, 128;" ::: "memory");
                const int lx = r & 7, ly = r >> 3;
                float v[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int t = 0; t < 9; t++) {
                    const float* zr = Z + ((ly + t / 3) * kHaloW + lx + t % 3) * kZPitch + 3 * t;
#pragma unroll
                    for (int co = 0; co < 3; co++) v[co] += zr[co];
                }
                if (inside) {
#pragma unroll
                    for (int co = 0; co < 3; co++) {
                        float o = v[co] + sbias[co];
                        if (mode == kWriteNextState) o = o + st[co];
                        I.out[co * plane + cl] = o;
                    }
                }
                asm volatile("bar.sync 1, 128;" ::: "memory");  // Z is rewritten by the next tile
            } else {
                // the staging box used two tiles ago must have been read by its store
                if (leader && it >= 1) tc::bulk_wait_read();
                asm volatile("bar.sync 1, 128;" ::: "memory");
                uint8_t* box = sStage + (size_t)r * 16;  // [4 planes][128][8] f16
                for (int c = 0; c < BN; c += 16) {
                    float a[16];
                    tc::tmem_ld16(ta + c, a);
#pragma unroll
                    for (int i = 0; i < 16; i += 2) gelu_fast_pair(a[i], a[i + 1], sbias[c + i], sbias[c + i + 1]);
                    uint32_t w[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        __half2 h = __floats2half2_rn(a[2 * i], a[2 * i + 1]);
                        w[i] = *reinterpret_cast<uint32_t*>(&h);
                    }
                    *reinterpret_cast<uint4*>(box + (c / 8) * 2048) = make_uint4(w[0], w[1], w[2], w[3]);
                    *reinterpret_cast<uint4*>(box + (c / 8 + 1) * 2048) = make_uint4(w[4], w[5], w[6], w[7]);
                }
                tc::tc_fence_before();
                tc::mbar_arrive(&a_empty[b]);
                tc::fence_async_shared();
                asm volatile("bar.sync 1, 128;" ::: "memory");
                if (leader) {
                    const CUtensorMap* omap = maps + kMapsPerInst * ii + 3;
                    tc::tensormap_acquire(omap);
                    tc::tma_store_3d(omap, sStage, x0 * 8, y0, 0);
                    tc::bulk_commit();
                }
            }
        }
        if (KIND == kCellConv1 && leader) tc::bulk_wait_read();
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 2 * BN);
}

// Whether the shared-memory attention tiles apply (radius-1, dilation-1
// stencil; 64-channel boxes; at most 4 heads of width 32 or 64).
static bool attn_tile_ok(const Dims& d) {
    return d.mask_kind == 1 && d.radius == 1 && d.dilation == 1 && d.D % 64 == 0 && d.heads <= 4 &&
           (d.D / d.heads == 32 || d.D / d.heads == 64);
}
static size_t attn_tile_smem(const Dims&) { return (size_t)2 * kAttBoxKVPad + kAttBoxQ; }

// ---------------------------------------------------------------------------
// host

static const bf16* upload_bf16(DeviceArena& a, const std::vector<uint16_t>& v) {
    return static_cast<const bf16*>(a.upload_bytes(v.data(), v.size() * 2));
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

void BF16Path::weight_slots(std::vector<const void**>& out) const {
    auto add = [&](const bf16* const& p) { out.push_back(reinterpret_cast<const void**>(const_cast<const bf16**>(&p))); };
    for (int l = 0; l < dims_.L; l++) {
        add(wqkv[l]);
        add(wp[l]);
    }
    for (int v = 0; v < n_nc; v++)
        for (int l = 0; l < dims_.L; l++) {
            add(w1v[v][l]);
            add(w2v[v][l]);
        }
    add(wtm);
    add(wtc);
    add(wc1);
    add(wc2);
}

BF16Path::BF16Path(const Dims& d, const TensorMap* tp, DeviceArena* ap) {
    const int D = d.D, F = d.F, HD = d.HD;
    dims_D_ = D;
    dims_F_ = F;
    dims_ = d;
    if (D % 32 || D > 256 || 32 % d.heads || F % 64 || HD != 32 || d.C != 3 || d.P != 4 || d.C * d.P * d.P > 64)
        throw Error(JC_LIMIT,
                    "the BF16 path needs dim a multiple of 32 and <= 256, heads dividing 32, a cell-head width of 32, "
                    "3 channels and patch 4");
    n_nc = 2;  // MLP weights arranged for chunk widths 32 and 64
    bn_qkv = (3 * D) % 128 == 0 ? 128 : 3 * D;
    bn_tm = D <= 128 ? D : 64;
    if (F > 1024) throw Error(JC_LIMIT, "the BF16 MLP supports a hidden width of at most 1024");
    {
        int dev = 0;
        cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
        cuda_check(cudaDeviceGetAttribute(&n_sms_, cudaDevAttrMultiProcessorCount, dev), "SM count");
    }
    // default: the serial kernel, 64 columns (fits every supported width)
    def_tuning_ = Tuning{64, 256};
    if (!mlp_fits(64)) def_tuning_.nc = 32;
    if (!mlp_fits(def_tuning_.nc)) throw Error(JC_LIMIT, "the BF16 MLP does not fit in shared memory at this width");
    if (attn_tile_ok(d)) def_tuning_.attn_threads = 0;  // shared-memory attention tiles
    for (int l = 0; l < kMaxLayers; l++) {
        wqkv[l] = wp[l] = nullptr;
        w1v[0][l] = w1v[1][l] = w2v[0][l] = w2v[1][l] = nullptr;
    }
    wtm = wtc = wc1 = nullptr;
    if (tp) upload_weights(d, *tp, *ap);
    cache_key_ = "d" + std::to_string(D) + "_l" + std::to_string(d.L) + "_f" + std::to_string(F) + "_r" +
                 std::to_string(d.radius) + "_k" + std::to_string(d.mask_kind) + "_g" + std::to_string(d.dilation);
    load_cache();
    set_kernel_attributes();
}

void BF16Path::upload_weights(const Dims& d, const TensorMap& t, DeviceArena& arena) {
    const int D = d.D, F = d.F, HD = d.HD;
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
            const int nc = v == 0 ? 32 : 64;
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
        // conv1 (f16 operands): per tap [48/8][32][8] over the zc channels: z
        // (32), then the state's [hi, lo, hi] parts with weights [W_hi, W_hi, W_lo]
        const auto& w = tget(t, "head.conv1.weight").data;  // [HD][HD+C][3][3]
        const int cin = HD + d.C;
        auto h_round = [](float v) { return __half2float(__float2half_rn(v)); };
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
                            const float hi = h_round(full);
                            v = part < 2 ? hi : full - hi;
                        }
                        o[i++] = f2h(v);
                    }
        wc1 = upload_bf16(arena, o);  // f16 bits
    }
    {
        // conv2 (f16 operands): [32/8][32][8] over the c1 channels, column
        // n = 3 tap + co for tap = 3 ky + kx, columns 27..31 zero
        const auto& w = tget(t, "head.conv2.weight").data;  // [C][HD][3][3]
        std::vector<uint16_t> o((size_t)HD * 32);
        size_t i = 0;
        for (int kc = 0; kc < HD / 8; kc++)
            for (int n = 0; n < 32; n++)
                for (int e = 0; e < 8; e++)
                    o[i++] = f2h(n < 9 * d.C ? w[((size_t)(n % 3) * HD + kc * 8 + e) * 9 + n / 3] : 0.0f);
        wc2 = upload_bf16(arena, o);  // f16 bits
    }
}

void BF16Path::set_kernel_attributes() {
    set_smem(tc_gemm_kernel<EPI_BF16>, 200 * 1024);
    set_smem(tc_gemm_kernel<EPI_F32>, 200 * 1024);
    set_smem(tc_gemm_kernel<EPI_RESID_LN>, 200 * 1024);
    set_smem(tc_mlp_serial_kernel<false>, kMlpSmemMax);
    set_smem(tc_mlp_serial_kernel<true>, kMlpSmemMax);
    set_smem(tc_projln_persistent_kernel, 225 * 1024);  // 227 KB per CTA less the static shared memory
    set_smem(tc_qkv_persistent_kernel, 225 * 1024);
    set_smem(tc_cellconv_kernel<kCellConv1>, 200 * 1024);
    set_smem(tc_cellconv_kernel<kCellConv2>, 200 * 1024);
    set_smem(bf_attn_tile_kernel<32>, 200 * 1024);
    set_smem(bf_attn_tile_kernel<64>, 200 * 1024);
    set_smem(tc_conv3_kernel<CONV_TOKMIX>, 200 * 1024);
    set_smem(bf_embed_kernel<1>, 100 * 1024);
    set_smem(bf_embed_kernel<2>, 100 * 1024);
    set_smem(bf_embed_kernel<3>, 100 * 1024);
    set_smem(bf_embed_kernel<4>, 100 * 1024);
    set_smem(bf_embed_kernel<5>, 100 * 1024);
    set_smem(bf_embed_kernel<6>, 100 * 1024);
    set_smem(bf_embed_kernel<7>, 100 * 1024);
    set_smem(bf_embed_kernel<8>, 100 * 1024);
}

// One thread per (token row, head) in CTAs of `threads` threads (64, 128 or
// 256; the arithmetic of a thread does not depend on it).

static void launch_attention(const Dims& d, const bf16* qkv, const InstDev* inst, int n, int R, bf16* attn,
                             int threads, cudaStream_t s, const Pack* p = nullptr) {
    if (threads == 0) {
        // shared-memory tiles: grid (8 x 16 token tiles, their two 8 x 8 halves)
        const CUtensorMap* maps = reinterpret_cast<const CUtensorMap*>(p->tmaps);
        // one CTA per (token tile, 8 x 8 half, 64-channel box of heads)
        const dim3 grid((unsigned)p->n_ttiles, 2, (unsigned)(d.D / 64));
        if (d.D / d.heads == 32)
            cuda_check(launch_pdl(bf_attn_tile_kernel<32>, grid, 64 * 2, attn_tile_smem(d), s, 1u, d, maps, 4, 5, inst,
                                  n, attn, p->err),
                       "launch");
        else
            cuda_check(launch_pdl(bf_attn_tile_kernel<64>, grid, 64, attn_tile_smem(d), s, 1u, d, maps, 4, 5, inst, n,
                                  attn, p->err),
                       "launch");
        return;
    }
    const bool r1 = d.mask_kind == 1 && d.radius == 1;
    const int hd = d.D / d.heads;
    const unsigned blocks = (unsigned)(((long long)R * d.heads + threads - 1) / threads);
#define JC_ATTN_HEAD(H)                                                                          \
    if (hd == H) {                                                                               \
        if (r1) cuda_check(launch_pdl(bf_attn_head_r1_kernel<H>, blocks, threads, 0, s, 1u, d, qkv, inst, n, R, attn), "launch"); \
        else cuda_check(launch_pdl(bf_attn_head_kernel<H>, blocks, threads, 0, s, 1u, d, qkv, inst, n, R, attn), "launch");       \
        return;                                                                                  \
    }
    JC_ATTN_HEAD(8)
    JC_ATTN_HEAD(16)
    JC_ATTN_HEAD(32)
    JC_ATTN_HEAD(64)
#undef JC_ATTN_HEAD
    throw Error(JC_LIMIT, "the BF16 attention supports head widths 8, 16, 32 and 64");
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
    return def_tuning_;
}

// Shared memory of the MLP kernel (one stage, one h buffer; with the fused
// projection, the f32 P tile behind the A tile).
static size_t mlp_serial_smem(int D, int NC, bool proj = false) {
    return std::max({(size_t)D * 256 + 2 * (size_t)D * NC * 2 + (size_t)NC * 256, (size_t)128 * D * 4,
                     proj ? (size_t)D * 256 + (size_t)128 * D * 4 : (size_t)0});
}

bool BF16Path::mlp_fits(int nc) const {
    return (nc == 32 || nc == 64) && dims_F_ % nc == 0 && mlp_serial_smem(dims_D_, nc) <= kMlpSmemMax;
}

bool BF16Path::proj_fuses(const Tuning& tu) const { return dims_D_ == 128 && tu.nc == 64; }

void BF16Path::launch_mlp(const Dims& d, const WeightsF32& w, int l, const Tuning& tu, const CUtensorMap& m_ln,
                          const Pack& p, cudaStream_t s, const CUtensorMap* m_attn) const {
    const int D = d.D, R = p.R;
    const int v = tu.nc == 64 ? 1 : 0;
    const float* ng = l + 1 < d.L ? w.blk[l + 1].n1g : w.norm_g;
    const float* nbeta = l + 1 < d.L ? w.blk[l + 1].n1b : w.norm_b;
    const auto& B = w.blk[l];
    bf16* ln = reinterpret_cast<bf16*>(p.bt[0]);
    if (m_attn) {
        if (!proj_fuses(tu)) throw Error(JC_LIMIT, "the fused projection needs dim 128 and 64-column MLP chunks");
        cuda_check(launch_pdl(tc_mlp_serial_kernel<true>, (unsigned)((R + 127) / 128), kMlpSerialThreads,
                              mlp_serial_smem(D, tu.nc, true), s, 1u, m_ln, w1v[v][l], w2v[v][l], B.b1, B.b2, D, d.F, tu.nc, R,
                              p.x, ng, nbeta, ln, p.err, *m_attn, wp[l], B.bp, B.n2g, B.n2b),
                   "launch");
        return;
    }
    cuda_check(launch_pdl(tc_mlp_serial_kernel<false>, (unsigned)((R + 127) / 128), kMlpSerialThreads,
                          mlp_serial_smem(D, tu.nc), s, 1u, m_ln, w1v[v][l], w2v[v][l], B.b1, B.b2, D, d.F, tu.nc, R,
                          p.x, ng, nbeta, ln, p.err, m_ln, wp[l], B.bp, B.n2g, B.n2b),
               "launch");
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
    Tuning best = def_tuning_;
    // the workspace holds transient values; the timed launches may leave
    // anything in it (every forward rewrites it from the state)
    std::string log;
    // A candidate replaces the default only when it is clearly faster (by
    // kTuneMargin): a bucket's choice also serves other mixes of instance
    // sizes with that row count, and single timings vary by a few percent.
    constexpr float kTuneMargin = 0.95f;
    constexpr int kTuneReps = 8;
    float def_ms = 0.f, best_ms = 1e30f;
    for (int nc : {def_tuning_.nc, 96 - def_tuning_.nc}) {  // the default width first, then the other
        // where the default width carries the fused output projection, the
        // MLP alone is not the comparison: keep it
        if (!mlp_fits(nc) || (nc != def_tuning_.nc && proj_fuses(def_tuning_))) continue;
        Tuning t = best;
        t.nc = nc;
        const float ms = time_launches([&] { launch_mlp(d, w, 0, t, m_ln, p, s); }, kTuneReps, s);
        log += (log.empty() ? "" : ", ") + std::string("\"mlp_nc") + std::to_string(nc) + "_ms\": " + std::to_string(ms);
        if (nc == def_tuning_.nc) {
            def_ms = best_ms = ms;
        } else if (ms < kTuneMargin * def_ms && ms < best_ms) {
            best_ms = ms;
            best.nc = nc;
        }
    }
    const int def_attn = def_tuning_.attn_threads;
    std::vector<int> forms = {def_attn};
    for (int threads : {0, 64, 128, 256})
        if (threads != def_attn && (threads != 0 || attn_tile_ok(d))) forms.push_back(threads);
    for (int threads : forms) {
        const float ms = time_launches([&] { launch_attention(d, qkv, p.inst, p.n_inst, R, attn, threads, s, &p); },
                                       kTuneReps, s);
        log += ", \"attn_" + std::to_string(threads) + "_ms\": " + std::to_string(ms);
        if (threads == def_attn) {
            def_ms = best_ms = ms;
        } else if (ms < kTuneMargin * def_ms && ms < best_ms) {
            best_ms = ms;
            best.attn_threads = threads;
        }
    }
    cuda_check(cudaGetLastError(), "autotune");
    {
        std::lock_guard<std::mutex> lk(tune_mu_);
        tuned_[bucket] = best;
    }
    save_cache(bucket, best, log);
}

// Tuned schedules persist in the JSON-lines file named by JC_AUTOTUNE_CACHE,
// one object per tuned row bucket:
//   {"model": "d128_l4_f512_r1_k1_g1", "rows": 65536, "nc": 64, "attn_threads": 0}
// keyed by the model shape (dim, layers, MLP width, mask radius, kind and
// dilation), followed by the candidates' measured times. Lines that do not
// parse or name another shape are skipped; later lines override earlier ones.
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
        if (cache_key_ == key && mlp_fits(nc) && (th == 64 || th == 128 || th == 256 || (th == 0 && attn_tile_ok(dims_))))
            tuned_[bucket] = Tuning{nc, th};
    }
    std::fclose(f);
}

void BF16Path::save_cache(int bucket, const Tuning& t, const std::string& timings) const {
    const char* path = std::getenv("JC_AUTOTUNE_CACHE");
    if (!path) return;
    std::lock_guard<std::mutex> lk(tune_mu_);
    FILE* f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "{\"model\": \"%s\", \"rows\": %d, \"nc\": %d, \"attn_threads\": %d%s%s}\n", cache_key_.c_str(),
                 bucket, t.nc, t.attn_threads, timings.empty() ? "" : ", ", timings.c_str());
    std::fclose(f);
}

void BF16Path::alloc_workspace(DeviceArena& a, const Dims& d, Pack& p, int rows, long long cells, int max_inst) const {
    const size_t R = (size_t)rows, NC = (size_t)cells;
    const int strides[4] = {d.D * 2, 3 * d.D * 2, d.D * 2, d.D * 2};  // ln, qkv, attn, t1
    for (int i = 0; i < 4; i++) {
        p.bt[i] = static_cast<char*>(a.alloc(R * strides[i] + 256));
        p.bt_stride[i] = strides[i];
    }
    // zc and c1, f16, plane-major: [channels / 8][cells][8]
    const int planes[2] = {kZcCh / 8, d.HD / 8};
    for (int i = 0; i < 2; i++) {
        p.bc[i] = static_cast<char*>(a.alloc(NC * planes[i] * 16 + 256));
        p.bc_stride[i] = 16;
        p.bc_plane[i] = (long long)NC * 16;
    }
    p.tmaps = a.alloc((size_t)max_inst * kMapsPerInst * sizeof(CUtensorMap));
}

void BF16Path::prepare(const Dims& d, const Pack& p, const InstDev* hinst, cudaStream_t s, CUtensorMap* hstage) const {
    std::vector<CUtensorMap> tmp(hstage ? 0 : (size_t)p.n_inst * kMapsPerInst);
    CUtensorMap* maps = hstage ? hstage : tmp.data();
    for (int i = 0; i < p.n_inst; i++) {
        const InstDev& I = hinst[i];
        CUtensorMap* m = &maps[(size_t)kMapsPerInst * i];
        m[0] = halo_map(p.bt[0] + (size_t)I.row0 * p.bt_stride[0], d.D, I.tx, I.ty);
        m[1] = cell_plane_map(p.bc[0] + (size_t)I.cell0 * 16, kZcCh / 8, p.bc_plane[0], I.nx, I.ny, true);
        m[2] = tile_store_map(p.bt[3] + (size_t)I.row0 * p.bt_stride[3], d.D, I.tx, I.ty, false);
        m[3] = cell_plane_map(p.bc[1] + (size_t)I.cell0 * 16, d.HD / 8, p.bc_plane[1], I.nx, I.ny, false);
        m[6] = cell_plane_map(p.bc[1] + (size_t)I.cell0 * 16, d.HD / 8, p.bc_plane[1], I.nx, I.ny, true);
        if (attn_tile_ok(d)) {
            m[4] = att_map(p.bt[1] + (size_t)I.row0 * p.bt_stride[1], d.D, I.tx, I.ty, kAttHalo);
            m[5] = att_map(p.bt[1] + (size_t)I.row0 * p.bt_stride[1], d.D, I.tx, I.ty, kAttTile);
        }
    }
    cuda_check(cudaMemcpyAsync(p.tmaps, maps, (size_t)p.n_inst * kMapsPerInst * sizeof(CUtensorMap),
                               cudaMemcpyHostToDevice, s),
               "tensor maps", JC_MAP);
    // a temporary host array is released on return: wait for the copy
    if (!hstage) cuda_check(cudaStreamSynchronize(s), "tensor maps", JC_POLL);
}

void BF16Path::forward(const Dims& d, const WeightsF32& w, const Pack& p, int mode, cudaStream_t s) const {
    const int R = p.R, D = d.D, n = p.n_inst;
    if (R == 0) return;
    bf16* ln = reinterpret_cast<bf16*>(p.bt[0]);
    bf16* qkv = reinterpret_cast<bf16*>(p.bt[1]);
    bf16* attn = reinterpret_cast<bf16*>(p.bt[2]);
    bf16* t1 = reinterpret_cast<bf16*>(p.bt[3]);
    const CUtensorMap m_ln = rows_map(ln, D, R), m_attn = rows_map(attn, D, R), m_t1 = rows_map(t1, D, R);
    const CUtensorMap m_qkv_out = store_map(qkv, 3 * D, R, 3 * D, false), m_z0_out = store_map(p.z0, d.HD, R, d.HD, true);
    const CUtensorMap m_x = store_map(p.x, D, R, D, true);
    const unsigned gm = (unsigned)((R + 127) / 128);
    const Tuning tu = tuning_for(R);
    {
        KScope k("bf_embed", s);
        const int tiles = (R + kEmbedRows - 1) / kEmbedRows;
        const size_t smem = embed_smem(D);
        // persistent: as many CTAs as fit on the SMs at once
        static int occupancy[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // CTAs per SM, per D / 32
        auto grid_for = [&](auto kernel) {
            int& per_sm = occupancy[D / 32];
            if (per_sm == 0)
                cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, smem), "occupancy");
            return (unsigned)std::min(tiles, std::max(1, per_sm) * n_sms_);
        };
#define JC_EMBED(CPL)                                                                                            \
    case CPL:                                                                                                    \
        cuda_check(launch_pdl(bf_embed_kernel<CPL>, grid_for(bf_embed_kernel<CPL>), 256, smem, s, 1u, d, w.embed_w, \
                              w.embed_b, w.meta_w, w.meta_b, w.blk[0].n1g, w.blk[0].n1b, p.inst, n, R, p.x, ln),     \
                   "launch");                                                                                    \
        break;
        switch (D / 32) {
            JC_EMBED(1) JC_EMBED(2) JC_EMBED(3) JC_EMBED(4) JC_EMBED(5) JC_EMBED(6) JC_EMBED(7) JC_EMBED(8)
            default: throw Error(JC_LIMIT, "the BF16 embed supports dim 32..256 in steps of 32");
        }
#undef JC_EMBED
        check_launch("bf_embed");
    }
    for (int l = 0; l < d.L; l++) {
        const auto& B = w.blk[l];
        {
            KScope k("tc_qkv", s);
            const int BN = bn_qkv;
            if (D <= 128) {
                const unsigned grid = (unsigned)std::min((int)gm, n_sms_);
                cuda_check(launch_pdl(tc_qkv_persistent_kernel, grid, kQKVPThreads, QKVPSmem(D, BN).total, s, 1u, m_ln, m_qkv_out, wqkv[l],
                                                                                         B.bqkv, D, BN, R, p.err), "launch");
            } else {
                GemmEpi ep{B.bqkv, qkv, nullptr, nullptr, nullptr, nullptr, 3 * D};
                const size_t smem = std::max((size_t)D * 256 + (size_t)D * BN * 2, (size_t)((BN + 63) / 64) * 16384);
                cuda_check(launch_pdl(tc_gemm_kernel<EPI_BF16>, dim3(gm, 3 * D / BN), 128, smem, s, 1u, m_ln, m_qkv_out, wqkv[l], D, BN, R, ep,
                                                                             p.err), "launch");
            }
            check_launch("tc_qkv");
        }
        {
            KScope k("bf_attention", s);
            launch_attention(d, qkv, p.inst, n, R, attn, tu.attn_threads, s, &p);
            check_launch("bf_attention");
        }
        if (proj_fuses(tu)) {
            // output projection + LayerNorm2 inside the MLP kernel
            KScope k("tc_proj_mlp", s);
            launch_mlp(d, w, l, tu, m_ln, p, s, &m_attn);
            check_launch("tc_proj_mlp");
            continue;
        }
        {
            KScope k("tc_proj_ln", s);
            if (D <= kLnMaxD) {
                const unsigned grid = (unsigned)std::min((int)gm, n_sms_);
                cuda_check(launch_pdl(tc_projln_persistent_kernel, grid, kPLThreads, PLSmem(D).total, s, 1u, m_attn, m_x, wp[l], B.bp, B.n2g,
                                                                                    B.n2b, ln, D, R, p.err), "launch");
            } else {
                GemmEpi ep{B.bp, ln, nullptr, p.x, B.n2g, B.n2b, D};
                const size_t smem = std::max((size_t)D * 256 + (size_t)D * D * 2, (size_t)128 * D * 4);
                cuda_check(launch_pdl(tc_gemm_kernel<EPI_RESID_LN>, dim3(gm, 1), 128, smem, s, 1u, m_attn, m_attn, wp[l], D, D, R, ep,
                                                                            p.err), "launch");
            }
            check_launch("tc_proj_ln");
        }
        {
            KScope k("tc_mlp", s);
            launch_mlp(d, w, l, tu, m_ln, p, s);
            check_launch("tc_mlp");
        }
    }
    {
        KScope k("tc_token_mix", s);
        const int BN = bn_tm;
        const int NS = conv3_smem(D, BN, 9) <= 100 * 1024 ? 9 : 2;
        cuda_check(launch_pdl(tc_conv3_kernel<CONV_TOKMIX>, dim3(p.n_ttiles, D / BN), 128, conv3_launch_smem(D, BN, NS, 2), s, 1u, 
            reinterpret_cast<const CUtensorMap*>(p.tmaps), 0, 2, wtm, w.tm_b, D, BN, NS, p.inst, n, p.err), "launch");
        check_launch("tc_token_mix");
    }
    {
        KScope k("tc_to_cells", s);
        GemmEpi ep{w.tc_b, nullptr, p.z0, nullptr, nullptr, nullptr, d.HD};
        const size_t smem = std::max((size_t)D * 256 + (size_t)D * d.HD * 2, (size_t)((d.HD + 31) / 32) * 16384);
        cuda_check(launch_pdl(tc_gemm_kernel<EPI_F32>, dim3(gm, 1), 128, smem, s, 1u, m_t1, m_z0_out, wtc, D, d.HD, R, ep, p.err), "launch");
        check_launch("tc_to_cells");
    }
    {
        KScope k("bf_upsample", s);
        cuda_check(launch_pdl(bf_upsample_kernel<32, 3>, (unsigned)p.n_ctiles, 128, 0, s, 1u, d, p.z0, p.inst, n,
                                                                       reinterpret_cast<__half*>(p.bc[0]), p.bc_plane[0] / 2), "launch");
        check_launch("bf_upsample");
    }
    {
        KScope k("tc_conv1", s);
        const unsigned grid = (unsigned)std::min(p.n_ctiles, 3 * n_sms_);
        cuda_check(launch_pdl(tc_cellconv_kernel<kCellConv1>, grid, kC1PThreads,
                              C1PSmem(kCellConv1, kZcCh).total, s, 1u,
                              reinterpret_cast<const CUtensorMap*>(p.tmaps), wc1, w.c1_b, kZcCh, p.n_ctiles, p.inst, n,
                              mode, p.err),
                   "launch");
        check_launch("tc_conv1");
    }
    {
        KScope k("tc_conv2", s);
        const unsigned grid = (unsigned)std::min(p.n_ctiles, 4 * n_sms_);
        cuda_check(launch_pdl(tc_cellconv_kernel<kCellConv2>, grid, kC1PThreads, C1PSmem(kCellConv2, d.HD).total, s, 1u,
                              reinterpret_cast<const CUtensorMap*>(p.tmaps), wc2, w.c2_b, d.HD, p.n_ctiles, p.inst, n,
                              mode, p.err),
                   "launch");
        check_launch("tc_conv2");
    }
}

}  // namespace jc
