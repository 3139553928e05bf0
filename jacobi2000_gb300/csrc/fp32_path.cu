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

static void check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

namespace f32k {

// Patchify + embed + pos + meta (cpu.rs:253-280). One CTA per TOK rows;
// threads stride over the D outputs. Token t = ty*tx + tx, feature
// c*P*P + py*P + px.
constexpr int kEmbedTok = 16;

__global__ void embed_kernel(Dims d, const float* __restrict__ We, const float* __restrict__ be,
                             const float* __restrict__ Wm, const float* __restrict__ bm, const InstDev* inst,
                             const int* row_inst, int R, float* __restrict__ x) {
    extern __shared__ float patch[];  // [kEmbedTok][C*P*P]
    const int pd = d.C * d.P * d.P;
    const int r0 = blockIdx.x * kEmbedTok;
    for (int e = threadIdx.x; e < kEmbedTok * pd; e += blockDim.x) {
        int i = e / pd, f = e % pd, r = r0 + i;
        float v = 0.f;
        if (r < R) {
            const InstDev& I = inst[row_inst[r]];
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
        const InstDev& I = inst[row_inst[r]];
        float acc = be[o];
        const float* p = patch + i * pd;
        for (int f = 0; f < pd; f++) acc = fmaf(p[f], We[(size_t)f * d.D + o], acc);
        float m = bm[o];
        for (int f = 0; f < d.meta_dim; f++) m = fmaf(I.meta[f], Wm[(size_t)f * d.D + o], m);
        x[(size_t)r * d.D + o] = (acc + I.pos[(size_t)(r - I.row0) * d.D + o]) + m;
    }
}

// Stencil-masked multi-head attention (cpu.rs:97-164, mask.rs:18-30). One
// warp per (row, head); lanes over the head's features. Candidate keys are
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

__global__ void attention_kernel(Dims d, const float* __restrict__ qkv, const InstDev* inst, const int* row_inst,
                                 int R, float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int wg = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int row = wg / d.heads, head = wg % d.heads;
    if (row >= R) return;
    const int hd = d.D / d.heads, D3 = 3 * d.D;
    const InstDev& I = inst[row_inst[row]];
    const int t = row - I.row0, qy = t / I.tx, qx = t % I.tx;
    const float scale = 1.0f / sqrtf((float)hd);
    const float* q = qkv + (size_t)row * D3 + head * hd;
    float qv0 = lane < hd ? q[lane] : 0.f;
    float qv1 = lane + 32 < hd ? q[lane + 32] : 0.f;
    const int nc = n_candidates(d, I);

    auto score = [&](int kr) {
        const float* k = qkv + (size_t)kr * D3 + d.D + head * hd;
        float p = (lane < hd ? qv0 * k[lane] : 0.f) + (lane + 32 < hd ? qv1 * k[lane + 32] : 0.f);
        for (int e = lane + 64; e < hd; e += 32) p += q[e] * k[e];
        return warp_sum(p) * scale;
    };
    float smax = -INFINITY;
    for (int j = 0; j < nc; j++) {
        int kr = candidate_row(d, I, qy, qx, j);
        if (kr >= 0) smax = fmaxf(smax, score(kr));
    }
    float denom = 0.f;
    for (int j = 0; j < nc; j++) {
        int kr = candidate_row(d, I, qy, qx, j);
        if (kr >= 0) denom += expf(score(kr) - smax);
    }
    float o0 = 0.f, o1 = 0.f;
    for (int j = 0; j < nc; j++) {
        int kr = candidate_row(d, I, qy, qx, j);
        if (kr < 0) continue;
        float e = expf(score(kr) - smax);
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
__global__ void upsample_concat_kernel(Dims d, const float* __restrict__ z0, const InstDev* inst,
                                       const int* cell_inst, long long NC, float* __restrict__ zc) {
    long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= NC) return;
    const InstDev& I = inst[cell_inst[cell]];
    long long cl = cell - I.cell0;
    int y = (int)(cl / I.nx), x = (int)(cl % I.nx);
    int yt = y / d.P, iy = y % d.P, xt = x / d.P, ix = x % d.P;
    int yt2 = min(yt + 1, I.ty - 1), xt2 = min(xt + 1, I.tx - 1);
    float wy = ((float)iy + 0.5f) / (float)d.P, wx = ((float)ix + 0.5f) / (float)d.P;
    const float* a = z0 + (size_t)(I.row0 + yt * I.tx + xt) * d.HD;
    const float* b = z0 + (size_t)(I.row0 + yt * I.tx + xt2) * d.HD;
    const float* c = z0 + (size_t)(I.row0 + yt2 * I.tx + xt) * d.HD;
    const float* e = z0 + (size_t)(I.row0 + yt2 * I.tx + xt2) * d.HD;
    float* o = zc + (size_t)cell * kZcStride;
    for (int ch = 0; ch < d.HD; ch++) {
        float z1a = a[ch] * (1.0f - wy) + c[ch] * wy;  // upsample_y at column xt
        float z1b = b[ch] * (1.0f - wy) + e[ch] * wy;  // upsample_y at column xt2
        o[ch] = z1a * (1.0f - wx) + z1b * wx;          // upsample_x
    }
    size_t plane = (size_t)I.nx * I.ny;
    for (int ch = 0; ch < d.C; ch++) o[d.HD + ch] = I.state[ch * plane + cl];
    for (int ch = d.HD + d.C; ch < kZcStride; ch++) o[ch] = 0.f;
}

// head.conv2 (3x3, HD -> C, cpu.rs:348-349) then the step's residual
// (cpu.rs:84-88), one thread per cell. c1 is [cells, HD].
__global__ void conv2_step_kernel(Dims d, const float* __restrict__ c1, const float* __restrict__ w2,
                                  const float* __restrict__ b2, const InstDev* inst, const int* cell_inst,
                                  long long NC, int mode) {
    extern __shared__ float ws[];  // [C][HD][9]
    for (int i = threadIdx.x; i < d.C * d.HD * 9; i += blockDim.x) ws[i] = w2[i];
    __syncthreads();
    long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= NC) return;
    const InstDev& I = inst[cell_inst[cell]];
    long long cl = cell - I.cell0;
    int y = (int)(cl / I.nx), x = (int)(cl % I.nx);
    float acc[4];
    for (int co = 0; co < d.C; co++) acc[co] = b2[co];
    for (int ci = 0; ci < d.HD; ci++) {
        for (int ky = 0; ky < 3; ky++) {
            int iy = y + ky - 1;
            if (iy < 0 || iy >= I.ny) continue;
            for (int kx = 0; kx < 3; kx++) {
                int ix = x + kx - 1;
                if (ix < 0 || ix >= I.nx) continue;
                float a = c1[(size_t)(I.cell0 + (long long)iy * I.nx + ix) * d.HD + ci];
                for (int co = 0; co < d.C; co++) acc[co] = fmaf(a, ws[(co * d.HD + ci) * 9 + ky * 3 + kx], acc[co]);
            }
        }
    }
    size_t plane = (size_t)I.nx * I.ny;
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
__global__ void projection_kernel(Dims d, const InstDev* inst, ProjSlot* slots, uint32_t flags, int init) {
    __shared__ double red[32];
    const InstDev& I = inst[blockIdx.x];
    ProjSlot& S = slots[I.proj];
    float* s = I.state;
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

template <int BM, int BN, int TM, int TN, class AL, class EP>
static void gemm(const AL& a, const float* W, const float* b, int R, int N, int K, const EP& e, cudaStream_t s) {
    dim3 grid((N + BN - 1) / BN, (R + BM - 1) / BM);
    f32k::gemm_kernel<BM, BN, 16, TM, TN, AL, EP><<<grid, (BM / TM) * (BN / TN), 0, s>>>(a, W, b, R, N, K, e);
    check_launch("gemm_f32");
}

void forward_f32(const Dims& d, const WeightsF32& w, const Pack& p, int mode, cudaStream_t s) {
    using namespace f32k;
    const int R = p.R, D = d.D;
    {
        int pd = d.C * d.P * d.P;
        embed_kernel<<<(R + kEmbedTok - 1) / kEmbedTok, 128, kEmbedTok * pd * sizeof(float), s>>>(
            d, w.embed_w, w.embed_b, w.meta_w, w.meta_b, p.inst, p.row_inst, R, p.x);
        check_launch("embed");
    }
    for (int l = 0; l < d.L; l++) {
        const auto& B = w.blk[l];
        gemm<64, 64, 4, 4>(ALayerNorm{p.x, B.n1g, B.n1b, R, D}, B.wqkv, B.bqkv, R, 3 * D, D,
                           EStore{p.qkv, 3 * D}, s);
        {
            long long warps = (long long)R * d.heads;
            attention_kernel<<<(unsigned)((warps + 3) / 4), 128, 0, s>>>(d, p.qkv, p.inst, p.row_inst, R, p.attn);
            check_launch("attention");
        }
        gemm<64, 64, 4, 4>(APlain{p.attn, D, R, D}, B.wp, B.bp, R, D, D, EResid{p.x, D}, s);
        gemm<64, 64, 4, 4>(ALayerNorm{p.x, B.n2g, B.n2b, R, D}, B.w1, B.b1, R, d.F, D, EGelu{p.ff1, d.F}, s);
        gemm<64, 64, 4, 4>(APlain{p.ff1, d.F, R, d.F}, B.w2, B.b2, R, D, d.F, EResid{p.x, D}, s);
    }
    layernorm_kernel<<<(R + 7) / 8, 256, 0, s>>>(p.x, w.norm_g, w.norm_b, R, D, p.xn);
    check_launch("layernorm");
    gemm<64, 64, 4, 4>(ATokConv3{p.xn, p.row_inst, p.inst, R, D}, w.tm_w, w.tm_b, R, D, 9 * D,
                       EGeluResidFrom{p.xn, p.t1, D}, s);
    gemm<64, 32, 4, 2>(APlain{p.t1, D, R, D}, w.tc_w, w.tc_b, R, d.HD, D, EStore{p.z0, d.HD}, s);
    const long long NC = p.NC;
    upsample_concat_kernel<<<(unsigned)((NC + 255) / 256), 256, 0, s>>>(d, p.z0, p.inst, p.cell_inst, NC, p.zc);
    check_launch("upsample_concat");
    {
        int Rc = (int)NC;
        gemm<64, 32, 4, 2>(ACellConv3{p.zc, p.cell_inst, p.inst, Rc, kZcStride, d.HD + d.C}, w.c1_w, w.c1_b, Rc,
                           d.HD, 9 * kZcStride, EGelu{p.c1, d.HD}, s);
    }
    conv2_step_kernel<<<(unsigned)((NC + 127) / 128), 128, d.C * d.HD * 9 * sizeof(float), s>>>(
        d, p.c1, w.c2_w, w.c2_b, p.inst, p.cell_inst, NC, mode);
    check_launch("conv2_step");
}

void projection(const Dims& d, const Pack& p, uint32_t flags, int init, cudaStream_t s) {
    f32k::projection_kernel<<<p.n_inst, 1024, 0, s>>>(d, p.inst, p.proj, flags, init);
    check_launch("projection");
}

}  // namespace jc
