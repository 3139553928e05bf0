// FP32 forward path and the tick projection. The kernel sequence restates
// crates/engine/src/cpu.rs:249-352 (forward) and project.rs:22-54
// (projections) on CUDA cores; operation order within a row follows the
// reference (bias first, sequential reductions in key order for the
// attention softmax), so results agree with the reference's f32 CPU path to
// rounding.
#include <stdexcept>
#include <string>

#include "engine.hpp"
#include "fp32_kernels.cuh"

namespace jc {

thread_local KernelTimer* g_ktimer = nullptr;

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

// head.conv2 (3x3, HD -> C, cpu.rs:348-349) then the step's residual
// (cpu.rs:84-88). One CTA per 16x16 cell tile: the tile's c1 values plus a
// one-cell halo are staged in shared memory; one thread per cell.
__global__ void __launch_bounds__(256)
conv2_step_kernel(Dims d, const float* __restrict__ c1, const float* __restrict__ w2, const float* __restrict__ b2,
                  const InstDev* inst, int n_inst, int mode) {
    extern __shared__ __align__(16) float sm[];
    constexpr int S = kCellTile + 2;
    const int HD = d.HD;
    float* tile = sm;                  // [S][S][HD]
    float* ws = sm + S * S * HD;       // [C][HD][9]
    // instance and tile of this CTA
    int lo = 0, hi = n_inst - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (inst[mid].tile0 <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    const InstDev& I = inst[lo];
    const int tiles_x = (I.nx + kCellTile - 1) / kCellTile;
    const int tl = blockIdx.x - I.tile0;
    const int y0 = (tl / tiles_x) * kCellTile, x0 = (tl % tiles_x) * kCellTile;
    for (int i = threadIdx.x; i < d.C * HD * 9; i += blockDim.x) ws[i] = w2[i];
    const int q4 = HD / 4;
    for (int e = threadIdx.x; e < S * S * q4; e += blockDim.x) {
        int q = e % q4, p = e / q4, sy = p / S, sx = p % S;
        int y = y0 + sy - 1, x = x0 + sx - 1;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (y >= 0 && x >= 0 && y < I.ny && x < I.nx)
            v = reinterpret_cast<const float4*>(c1 + ((size_t)I.cell0 + (size_t)y * I.nx + x) * HD)[q];
        reinterpret_cast<float4*>(tile + (size_t)p * HD)[q] = v;
    }
    __syncthreads();
    const int ty = threadIdx.x / kCellTile, tx = threadIdx.x % kCellTile;
    const int y = y0 + ty, x = x0 + tx;
    if (y >= I.ny || x >= I.nx) return;
    float acc[4];
    for (int co = 0; co < d.C; co++) acc[co] = b2[co];
    for (int ci = 0; ci < HD; ci++) {
#pragma unroll
        for (int ky = 0; ky < 3; ky++) {
            if (y + ky - 1 < 0 || y + ky - 1 >= I.ny) continue;
#pragma unroll
            for (int kx = 0; kx < 3; kx++) {
                if (x + kx - 1 < 0 || x + kx - 1 >= I.nx) continue;
                float a = tile[((ty + ky) * S + tx + kx) * HD + ci];
                for (int co = 0; co < d.C; co++) acc[co] = fmaf(a, ws[(co * HD + ci) * 9 + ky * 3 + kx], acc[co]);
            }
        }
    }
    const size_t plane = (size_t)I.nx * I.ny, cl = (size_t)y * I.nx + x;
    for (int co = 0; co < d.C; co++) {
        float v = acc[co];
        if (mode == kWriteNextState) v = v + I.state[co * plane + cl];
        I.out[co * plane + cl] = v;
    }
}

// Block-wide f64 sum (fixed order, deterministic). `red` holds 32 doubles.
__device__ double block_sum_d(double v, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum_d(v);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (warp == 0) {
        t = lane < nw ? red[lane] : 0.0;
        t = warp_sum_d(t);
        if (lane == 0) red[0] = t;
    }
    __syncthreads();
    double r = red[0];
    __syncthreads();
    return r;
}

// Potential and kinetic energy sums (project.rs:9-19), per-cell terms in f64
// from the stored f32 values, Neumaier-compensated per thread.
__device__ void energy_terms(const Dims& d, const float* s, long long n, double* P, double* K, double* red) {
    Neu p, k;
    p.init();
    k.init();
    const double hoff = (double)d.norm_mean[0] + (double)d.norm_depth;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        double h = (double)s[i] * d.norm_std[0] + hoff;
        double u = (double)s[n + i] * d.norm_std[1] + d.norm_mean[1];
        double v = (double)s[2 * n + i] * d.norm_std[2] + d.norm_mean[2];
        p.add(0.5 * (double)d.g * h * h);
        k.add(0.5 * h * (u * u + v * v));
    }
    *P = block_sum_d(p.val(), red);
    *K = block_sum_d(k.val(), red);
}

// Mass then energy projection (eval.rs:148-153 order; project.rs:33-54) of
// one instance per CTA, with f64 compensated sums; the shift and scale are
// rounded to f32 and applied with the reference's f32 update.
__global__ void __launch_bounds__(512) projection_kernel(Dims d, const InstDev* inst, ProjSlot* slots, int init) {
    __shared__ double red[32];
    const InstDev& I = inst[blockIdx.x];
    ProjSlot& S = slots[blockIdx.x];
    float* s = I.state;
    const unsigned flags = I.flags;
    const long long n = (long long)I.nx * I.ny;
    if (init) {
        Neu m;
        m.init();
        for (long long i = threadIdx.x; i < n; i += blockDim.x) m.add((double)s[i]);
        double M = block_sum_d(m.val(), red) / (double)n;
        double P, K;
        energy_terms(d, s, n, &P, &K, red);
        if (threadIdx.x == 0) {
            S.mass0 = M;
            S.energy = P + K;
            S.max_viol = 0.0;
            S.last_scale = 1.0;
        }
        return;
    }
    const double prev = S.energy;
    if (flags & 1u) {
        Neu m;
        m.init();
        for (long long i = threadIdx.x; i < n; i += blockDim.x) m.add((double)s[i]);
        double M = block_sum_d(m.val(), red) / (double)n;
        float delta = (float)(S.mass0 - M);
        for (long long i = threadIdx.x; i < n; i += blockDim.x) s[i] = __fadd_rn(s[i], delta);
        __syncthreads();
    }
    double P, K;
    if (flags & 2u) {
        energy_terms(d, s, n, &P, &K, red);
        double bound = prev * (double)d.energy_r_max;
        double budget = bound - P;
        if (!(budget > 0.0)) budget = 0.0;
        double sc = sqrt(budget / (K > 1e-12 ? K : 1e-12));
        sc = sc < 0.0 ? 0.0 : (sc > 1.0 ? 1.0 : sc);
        float s32 = (float)sc;
        for (long long i = threadIdx.x; i < n; i += blockDim.x) {
            float u = __fadd_rn(__fmul_rn(s[n + i], d.norm_std[1]), d.norm_mean[1]);
            float v = __fadd_rn(__fmul_rn(s[2 * n + i], d.norm_std[2]), d.norm_mean[2]);
            s[n + i] = __fdiv_rn(__fsub_rn(__fmul_rn(u, s32), d.norm_mean[1]), d.norm_std[1]);
            s[2 * n + i] = __fdiv_rn(__fsub_rn(__fmul_rn(v, s32), d.norm_mean[2]), d.norm_std[2]);
        }
        if (threadIdx.x == 0) S.last_scale = sc;
        __syncthreads();
    }
    energy_terms(d, s, n, &P, &K, red);
    if (threadIdx.x == 0) {
        double E = P + K;
        double viol = (E - prev * (double)d.energy_r_max) / prev;
        if (viol > S.max_viol) S.max_viol = viol;
        S.energy = E;
    }
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
    {
        KScope k("f32_conv2_step", s);
        constexpr int S = kCellTile + 2;
        size_t smem = ((size_t)S * S * d.HD + (size_t)d.C * d.HD * 9) * sizeof(float);
        conv2_step_kernel<<<p.n_tiles, kCellTile * kCellTile, smem, s>>>(d, p.c1, w.c2_w, w.c2_b, p.inst, n, mode);
        check_launch("conv2_step");
    }
}

void projection(const Dims& d, const Pack& p, int init, cudaStream_t s) {
    KScope k("projection", s);
    f32k::projection_kernel<<<p.n_inst, 512, 0, s>>>(d, p.inst, p.proj, init);
    check_launch("projection");
}

}  // namespace jc
