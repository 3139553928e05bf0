// The eval-metrics path on the device (crates/engine-cli/src/eval.rs:126-176):
// the reference shallow-water solver as a batched stencil kernel, the scores
// of crates/engine/src/metrics.rs with one CTA per scored state, and an
// evaluator that advances solver and model side by side inside the model's
// captured rollout graph and scores every trajectory at each horizon.
//
// Arithmetic: the solver and every score but the correlations repeat the
// reference's f32 operations one by one (explicitly rounded intrinsics, so no
// multiply-add is fused) and its summation order, so they give the
// reference's bits. The correlations' f64 sums are tree-ordered.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "evaluate.hpp"

namespace jc {
namespace ev {

// ---- solver: shallow_water.rs:149-238 ---------------------------------------

constexpr int kSwTX = 64, kSwTY = 32;     // output tile
constexpr int kSwThreads = 512;           // 4 cells per thread
constexpr int kSwPX = kSwTX + 4, kSwPY = kSwTY + 4;  // inputs with a 2-cell apron
constexpr int kSwNX = kSwTX + 2, kSwNY = kSwTY + 2;  // new depth with a 1-cell apron

struct SwDev {
    int nx, ny;
    float r, dt, g, nu, inv2dx, invdx2;
};

SwDev sw_dev(const jc_sw_params& p) {
    SwDev d;
    d.nx = p.nx;
    d.ny = p.ny;
    d.r = p.dt / p.dx;                     // shallow_water.rs:175
    d.dt = p.dt;
    d.g = p.g;
    d.nu = p.nu;
    d.inv2dx = 1.0f / (2.0f * p.dx);       // :186
    d.invdx2 = 1.0f / (p.dx * p.dx);       // :187
    return d;
}

// Face flux 0.5 (h_a + h_b) 0.5 (q_a + q_b), rounded step by step in the
// order shallow_water.rs:160,169 evaluates it.
__device__ __forceinline__ float face_flux(float ha, float hb, float qa, float qb) {
    return __fmul_rn(__fmul_rn(__fmul_rn(0.5f, __fadd_rn(ha, hb)), 0.5f), __fadd_rn(qa, qb));
}

struct SwSmem {
    float h[kSwPY][kSwPX + 1], u[kSwPY][kSwPX + 1], v[kSwPY][kSwPX + 1];
    float hn[kSwNY][kSwNX + 1];
};

// One forward-backward step of every state: continuity in flux form (zero
// flux through the walls), then momentum on the new surface with mirrored
// ghost cells (h even, normal velocity odd, tangential velocity even).
// grid (x tiles, y tiles, states); src and dst are [states][3][ny][nx]. A
// 64x32 tile per CTA keeps enough loads in flight per SM to cover the DRAM
// latency (the step is a pure stream: 12 bytes read and 12 written per cell).
__global__ void __launch_bounds__(kSwThreads)
sw_step_kernel(SwDev p, const float* __restrict__ src, float* __restrict__ dst) {
    __shared__ SwSmem sm;
    const int nx = p.nx, ny = p.ny;
    const long long n = (long long)nx * ny;
    const float* H = src + (long long)blockIdx.z * 3 * n;
    const float* U = H + n;
    const float* V = U + n;
    const int x0 = blockIdx.x * kSwTX, y0 = blockIdx.y * kSwTY;
    const int tid = threadIdx.x;
    // inputs on [y0-2, y0+TY+2) x [x0-2, x0+TX+2); apron positions outside
    // the grid hold a clamped neighbour and are never read below. Thread t
    // keeps column t % kSwPX and walks rows t / kSwPX, + kLoadRows, ...
    constexpr int kLoadRows = kSwThreads / kSwPX;  // 7 rows per pass
    if (tid < kLoadRows * kSwPX) {
        const int lx = tid % kSwPX;
        const int gx = min(max(x0 - 2 + lx, 0), nx - 1);
#pragma unroll
        for (int ly = tid / kSwPX; ly < kSwPY; ly += kLoadRows) {
            const int gy = min(max(y0 - 2 + ly, 0), ny - 1);
            const long long o = (long long)gy * nx + gx;
            sm.h[ly][lx] = __ldg(H + o);
            sm.u[ly][lx] = __ldg(U + o);
            sm.v[ly][lx] = __ldg(V + o);
        }
    }
    __syncthreads();
    // continuity on the tile and its 1-cell apron (cells inside the grid);
    // thread t keeps column t % kSwNX
    constexpr int kContRows = kSwThreads / kSwNX;  // 7 rows per pass
    if (tid < kContRows * kSwNX) {
        const int lx = tid % kSwNX;
        const int gx = x0 - 1 + lx;
        const bool xin = gx >= 0 && gx < nx;
        const bool wl = gx == 0, wr = gx == nx - 1;
        const int sx = lx + 1;
        for (int ly = tid / kSwNX; ly < kSwNY; ly += kContRows) {
            const int gy = y0 - 1 + ly;
            if (!xin || gy < 0 || gy >= ny) continue;
            const int sy = ly + 1;
            const float h = sm.h[sy][sx];
            const float fxl = wl ? 0.f : face_flux(sm.h[sy][sx - 1], h, sm.u[sy][sx - 1], sm.u[sy][sx]);
            const float fxr = wr ? 0.f : face_flux(h, sm.h[sy][sx + 1], sm.u[sy][sx], sm.u[sy][sx + 1]);
            const float fyl = gy == 0 ? 0.f : face_flux(sm.h[sy - 1][sx], h, sm.v[sy - 1][sx], sm.v[sy][sx]);
            const float fyr = gy == ny - 1 ? 0.f : face_flux(h, sm.h[sy + 1][sx], sm.v[sy][sx], sm.v[sy + 1][sx]);
            sm.hn[ly][lx] = __fsub_rn(h, __fmul_rn(p.r, __fadd_rn(__fsub_rn(fxr, fxl), __fsub_rn(fyr, fyl))));
        }
    }
    __syncthreads();
    float* D = dst + (long long)blockIdx.z * 3 * n;
    // momentum, centred differences on the new surface (:188-232); thread t
    // keeps column t % kSwTX and takes rows t / kSwTX, + 8, ...
    const int tx = tid % kSwTX;
    const int gx = x0 + tx;
    const int sx = tx + 2, qx = tx + 1;  // in h, u, v / in hn
    const int dxm = gx == 0 ? 0 : -1, dxp = gx == nx - 1 ? 0 : 1;
    const float sxm = gx == 0 ? -1.f : 1.f, sxp = gx == nx - 1 ? -1.f : 1.f;
#pragma unroll
    for (int c = 0; c < (kSwTX * kSwTY) / kSwThreads; c++) {
        const int ty = tid / kSwTX + c * (kSwThreads / kSwTX);
        const int gy = y0 + ty;
        if (gx >= nx || gy >= ny) continue;
        const int sy = ty + 2, qy = ty + 1;
        const int dym = gy == 0 ? 0 : -1, dyp = gy == ny - 1 ? 0 : 1;
        const float sym = gy == 0 ? -1.f : 1.f, syp = gy == ny - 1 ? -1.f : 1.f;
        const float hl = sm.hn[qy][qx + dxm], hr = sm.hn[qy][qx + dxp];
        const float hd = sm.hn[qy + dym][qx], hu = sm.hn[qy + dyp][qx];
        const float ul = __fmul_rn(sxm, sm.u[sy][sx + dxm]), ur = __fmul_rn(sxp, sm.u[sy][sx + dxp]);
        const float ud = sm.u[sy + dym][sx], uu = sm.u[sy + dyp][sx];
        const float vl = sm.v[sy][sx + dxm], vr = sm.v[sy][sx + dxp];
        const float vd = __fmul_rn(sym, sm.v[sy + dym][sx]), vu = __fmul_rn(syp, sm.v[sy + dyp][sx]);
        const float u0 = sm.u[sy][sx], v0 = sm.v[sy][sx];
        const float dudx = __fmul_rn(__fsub_rn(ur, ul), p.inv2dx), dudy = __fmul_rn(__fsub_rn(uu, ud), p.inv2dx);
        const float dvdx = __fmul_rn(__fsub_rn(vr, vl), p.inv2dx), dvdy = __fmul_rn(__fsub_rn(vu, vd), p.inv2dx);
        const float dhdx = __fmul_rn(__fsub_rn(hr, hl), p.inv2dx), dhdy = __fmul_rn(__fsub_rn(hu, hd), p.inv2dx);
        const float lap_u =
            __fmul_rn(__fsub_rn(__fadd_rn(__fadd_rn(__fadd_rn(ul, ur), ud), uu), __fmul_rn(4.0f, u0)), p.invdx2);
        const float lap_v =
            __fmul_rn(__fsub_rn(__fadd_rn(__fadd_rn(__fadd_rn(vl, vr), vd), vu), __fmul_rn(4.0f, v0)), p.invdx2);
        const float tu = __fadd_rn(
            __fsub_rn(__fsub_rn(__fmul_rn(-u0, dudx), __fmul_rn(v0, dudy)), __fmul_rn(p.g, dhdx)),
            __fmul_rn(p.nu, lap_u));
        const float tv = __fadd_rn(
            __fsub_rn(__fsub_rn(__fmul_rn(-u0, dvdx), __fmul_rn(v0, dvdy)), __fmul_rn(p.g, dhdy)),
            __fmul_rn(p.nu, lap_v));
        const long long o = (long long)gy * nx + gx;
        D[o] = sm.hn[qy][qx];
        D[n + o] = __fadd_rn(u0, __fmul_rn(p.dt, tu));
        D[2 * n + o] = __fadd_rn(v0, __fmul_rn(p.dt, tv));
    }
}

void sw_step(const SwDev& p, const float* src, float* dst, int count, cudaStream_t s) {
    KScope k("sw_step", s);
    const int gx = (p.nx + kSwTX - 1) / kSwTX, gy = (p.ny + kSwTY - 1) / kSwTY;
    const long long stride = 3LL * p.nx * p.ny;
    for (int c0 = 0; c0 < count; c0 += 65535) {
        const int c = std::min(65535, count - c0);
        sw_step_kernel<<<dim3(gx, gy, c), kSwThreads, 0, s>>>(p, src + c0 * stride, dst + c0 * stride);
    }
    cuda_check(cudaGetLastError(), "sw_step launch");
}

void check_params(const jc_sw_params& p) {
    if (p.nx < 1 || p.ny < 1 || (long long)p.nx * p.ny > (1LL << 30))
        throw Error(JC_BAD_SHAPE, "solver grid must be at least 1 x 1 and at most 2^30 cells");
    if (!(p.dx > 0.0f) || !std::isfinite(p.dt) || !std::isfinite(p.g) || !std::isfinite(p.nu) ||
        !std::isfinite(p.depth))
        throw Error(JC_BAD_ARGUMENT, "solver parameters must be finite with dx > 0");
}

// steps ticks of `count` states in place; `scratch` holds as many floats as
// the states (ping-pong partner).
void sw_run(const SwDev& d, float* states, float* scratch, int count, int steps, cudaStream_t s) {
    float* a = states;
    float* b = scratch;
    for (int t = 0; t < steps; t++) {
        sw_step(d, a, b, count, s);
        std::swap(a, b);
    }
    if (a != states)
        cuda_check(cudaMemcpyAsync(states, a, 3LL * d.nx * d.ny * count * sizeof(float), cudaMemcpyDeviceToDevice, s),
                   "solver result");
}

// State::add_drop (shallow_water.rs:102-111), host.
void add_drop(int nx, int ny, float* h, float cx, float cy, float amp, float sigma) {
    const float inv = 1.0f / (2.0f * sigma * sigma);
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            const float dx = (float)x - cx, dy = (float)y - cy;
            h[(size_t)y * nx + x] += amp * expf(-(dx * dx + dy * dy) * inv);
        }
}

// ---- scores: metrics.rs -------------------------------------------------------

constexpr int kScThreads = 512;
constexpr int kScChunk = 4096;  // cells staged per step of the sequential f32 sums

struct ScoreArgs {
    int nx, ny;
    float mean[3], std[3], depth;
    int cap;  // doubles per radial profile
};

struct ScoreRec {
    double sab, saa, sbb;        // correlation sums over (h, u, v)
    double sab_h, saa_h, sbb_h;  // over h
    float peak_m, peak_t;        // max |h| of model and solver (decoded)
    float mean_m, mean_t, std_t; // f32 sequential mean / std of the decoded h fields
    int len;                     // radial profile length rmax + 1
};

ScoreArgs score_args(const jc_config& c, int cap) {
    ScoreArgs a;
    a.nx = c.nx;
    a.ny = c.ny;
    for (int i = 0; i < 3; i++) {
        a.mean[i] = c.norm_mean[i];
        a.std[i] = c.norm_std[i];
    }
    a.depth = c.norm_depth;
    a.cap = cap;
    return a;
}

int profile_cap(int nx, int ny) { return std::min(nx, ny) / 2 + 3; }

// Normalizer::encode of one value of channel ch (norm.rs:30-32).
__device__ __forceinline__ float encode1(const ScoreArgs& a, int ch, float v) {
    if (ch == 0) v = __fsub_rn(v, a.depth);
    return __fdiv_rn(__fsub_rn(v, a.mean[ch]), a.std[ch]);
}

// decode_h (metrics.rs:105-107)
__device__ __forceinline__ float decode_h(const ScoreArgs& a, float x) {
    return __fadd_rn(__fmul_rn(x, a.std[0]), a.mean[0]);
}

template <int N>
__device__ void block_sum(double (&v)[N], double* red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < N; k++) v[k] = warp_sum_d(v[k]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; k++) red[k * 32 + w] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < N; k++) {
        double t = lane < nw ? red[k * 32 + lane] : 0.0;
        v[k] = warp_sum_d(t);
    }
    __syncthreads();
}

__device__ float block_max(float v, float* red) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();
    if (lane == 0) red[w] = v;
    __syncthreads();
    float t = lane < nw ? red[lane] : 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = fmaxf(t, __shfl_xor_sync(0xffffffffu, t, o));
    __syncthreads();
    return t;
}

// Radius bin of a cell (metrics.rs:51-53), f32 as the reference.
__device__ __forceinline__ int radius_bin(int x, int y, float cx, float cy) {
    const float dx = __fsub_rn((float)x, cx), dy = __fsub_rn((float)y, cy);
    const float r = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    return (int)__fadd_rn(r, 0.5f);
}

// One CTA scores state k: model x = xs[k] (normalized [3][n]) against the
// solver state truth + k * truth_stride (physical [3][n]). Writes the sums
// the host turns into a row, and both radial profiles (model, then solver)
// at profs + k * 2 * cap.
__global__ void __launch_bounds__(kScThreads)
score_kernel(ScoreArgs a, const float* const* xs, const float* truth, long long truth_stride, const float* centres,
             ScoreRec* recs, double* profs) {
    __shared__ double red[6 * 32];
    __shared__ float fred[32];
    __shared__ float sp[kScChunk], stg[kScChunk];
    __shared__ float means[2];
    const int k = blockIdx.x, tid = threadIdx.x;
    const int n = a.nx * a.ny;
    const float* x = xs[k];
    const float* T = truth + (long long)k * truth_stride;
    const float cx = centres[2 * k], cy = centres[2 * k + 1];
    auto target = [&](int i) {
        const int ch = i / n;
        return encode1(a, ch, T[i]);
    };
    // pass 1: means of x and of the encoded solver state, peaks of |h|
    double s1[4] = {0.0, 0.0, 0.0, 0.0};
    float pm = 0.f, pt = 0.f;
    for (int i = tid; i < 3 * n; i += kScThreads) {
        const float xv = x[i], tv = target(i);
        s1[0] += (double)xv;
        s1[1] += (double)tv;
        if (i < n) {
            s1[2] += (double)xv;
            s1[3] += (double)tv;
            pm = fmaxf(pm, fabsf(decode_h(a, xv)));
            pt = fmaxf(pt, fabsf(decode_h(a, tv)));
        }
    }
    block_sum(s1, red);
    pm = block_max(pm, fred);
    pt = block_max(pt, fred);
    const double ma = s1[0] / (double)(3 * n), mb = s1[1] / (double)(3 * n);
    const double mah = s1[2] / (double)n, mbh = s1[3] / (double)n;
    // pass 2: correlation sums (metrics.rs:12-18)
    double s2[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = tid; i < 3 * n; i += kScThreads) {
        const double xv = (double)x[i], tv = (double)target(i);
        const double dx = __dsub_rn(xv, ma), dy = __dsub_rn(tv, mb);
        s2[0] = __dadd_rn(s2[0], __dmul_rn(dx, dy));
        s2[1] = __dadd_rn(s2[1], __dmul_rn(dx, dx));
        s2[2] = __dadd_rn(s2[2], __dmul_rn(dy, dy));
        if (i < n) {
            const double ex = __dsub_rn(xv, mah), ey = __dsub_rn(tv, mbh);
            s2[3] = __dadd_rn(s2[3], __dmul_rn(ex, ey));
            s2[4] = __dadd_rn(s2[4], __dmul_rn(ex, ex));
            s2[5] = __dadd_rn(s2[5], __dmul_rn(ey, ey));
        }
    }
    block_sum(s2, red);
    // pass 3: f32 means of the decoded h fields, added in cell order by one
    // thread each (metrics.rs:29-31), through shared-memory chunks
    float acc = 0.f;
    for (int c0 = 0; c0 < n; c0 += kScChunk) {
        const int m = min(kScChunk, n - c0);
        for (int j = tid; j < m; j += kScThreads) {
            sp[j] = decode_h(a, x[c0 + j]);
            stg[j] = decode_h(a, encode1(a, 0, T[c0 + j]));
        }
        __syncthreads();
        if (tid == 0)
            for (int j = 0; j < m; j++) acc = __fadd_rn(acc, sp[j]);
        else if (tid == 32)
            for (int j = 0; j < m; j++) acc = __fadd_rn(acc, stg[j]);
        __syncthreads();
    }
    if (tid == 0) means[0] = __fdiv_rn(acc, (float)n);
    if (tid == 32) means[1] = __fdiv_rn(acc, (float)n);
    __syncthreads();
    // pass 4: f32 standard deviation of the solver's decoded h (metrics.rs:33-36)
    const float mt = means[1];
    acc = 0.f;
    for (int c0 = 0; c0 < n; c0 += kScChunk) {
        const int m = min(kScChunk, n - c0);
        for (int j = tid; j < m; j += kScThreads) stg[j] = decode_h(a, encode1(a, 0, T[c0 + j]));
        __syncthreads();
        if (tid == 0)
            for (int j = 0; j < m; j++) {
                const float d = __fsub_rn(stg[j], mt);
                acc = __fadd_rn(acc, __fmul_rn(d, d));
            }
        __syncthreads();
    }
    // pass 5: radial profiles (metrics.rs:45-61). Thread b owns radius bin b
    // and adds its cells in row-major order, the reference's order for that
    // bin, walking only the rows and columns of a widened annulus.
    float rm = fminf(fminf(fminf(cx, cy), __fsub_rn((float)a.nx, cx)), __fsub_rn((float)a.ny, cy));
    rm = fmaxf(floorf(rm), 1.0f);
    const int rmax = min((int)rm, a.cap - 1);
    double* pr = profs + (long long)k * 2 * a.cap;
    for (int b = tid; b <= rmax; b += kScThreads) {
        double sm = 0.0, st = 0.0;
        unsigned cnt = 0;
        const double ro = b + 1.5, ri = b - 1.5;
        const int y_lo = max(0, (int)ceil((double)cy - ro)), y_hi = min(a.ny - 1, (int)floor((double)cy + ro));
        for (int y = y_lo; y <= y_hi; y++) {
            const double dy = (double)y - (double)cy;
            const double o2 = ro * ro - dy * dy;
            if (o2 < 0.0) continue;
            const double xo = sqrt(o2);
            const double xi = (ri > 0.0 && ri * ri - dy * dy > 0.0) ? sqrt(ri * ri - dy * dy) : 0.0;
            int L0 = (int)ceil((double)cx - xo), L1 = (int)floor((double)cx - xi);
            int R0 = (int)ceil((double)cx + xi), R1 = (int)floor((double)cx + xo);
            L0 = max(L0, 0);
            R1 = min(R1, a.nx - 1);
            int segs[2][2];
            int ns = 0;
            if (xi <= 0.0 || L1 + 1 >= R0) {
                segs[0][0] = L0;
                segs[0][1] = R1;
                ns = 1;
            } else {
                segs[0][0] = L0;
                segs[0][1] = min(L1, a.nx - 1);
                segs[1][0] = max(R0, 0);
                segs[1][1] = R1;
                ns = 2;
            }
            for (int q = 0; q < ns; q++) {
                for (int x0 = segs[q][0]; x0 <= segs[q][1]; x0 += 8) {
                    float vm[8], vt[8];
                    bool in[8];
#pragma unroll
                    for (int j = 0; j < 8; j++) {
                        const int xx = x0 + j;
                        in[j] = xx <= segs[q][1] && radius_bin(xx, y, cx, cy) == b;
                        const long long o = (long long)y * a.nx + (in[j] ? xx : x0);
                        vm[j] = x[o];
                        vt[j] = T[o];
                    }
#pragma unroll
                    for (int j = 0; j < 8; j++)
                        if (in[j]) {
                            sm += (double)fabsf(decode_h(a, vm[j]));
                            st += (double)fabsf(decode_h(a, encode1(a, 0, vt[j])));
                            cnt++;
                        }
                }
            }
        }
        pr[b] = cnt == 0 ? 0.0 : sm / (double)cnt;
        pr[a.cap + b] = cnt == 0 ? 0.0 : st / (double)cnt;
    }
    if (tid == 0) {
        ScoreRec r;
        r.sab = s2[0];
        r.saa = s2[1];
        r.sbb = s2[2];
        r.sab_h = s2[3];
        r.saa_h = s2[4];
        r.sbb_h = s2[5];
        r.peak_m = pm;
        r.peak_t = pt;
        r.mean_m = means[0];
        r.mean_t = means[1];
        r.std_t = __fsqrt_rn(__fdiv_rn(acc, (float)n));
        r.len = rmax + 1;
        recs[k] = r;
    }
}

void score(const ScoreArgs& a, const float* const* xs, const float* truth, long long truth_stride,
           const float* centres, int count, ScoreRec* recs, double* profs, cudaStream_t s) {
    KScope k("eval_score", s);
    if (count <= 0) return;
    score_kernel<<<count, kScThreads, 0, s>>>(a, xs, truth, truth_stride, centres, recs, profs);
    cuda_check(cudaGetLastError(), "eval_score launch");
}

// metrics.rs:9-23 on host vectors (f32 values, f64 sums in order).
float correlation(const float* a, const float* b, int n) {
    double sa = 0.0, sb = 0.0;
    for (int i = 0; i < n; i++) sa += (double)a[i];
    for (int i = 0; i < n; i++) sb += (double)b[i];
    const double ma = sa / (double)n, mb = sb / (double)n;
    double sab = 0.0, saa = 0.0, sbb = 0.0;
    for (int i = 0; i < n; i++) {
        const double dx = (double)a[i] - ma, dy = (double)b[i] - mb;
        sab += dx * dy;
        saa += dx * dx;
        sbb += dy * dy;
    }
    if (saa <= 0.0 || sbb <= 0.0) return 0.0f;
    return (float)(sab / std::sqrt(saa * sbb));
}

// metrics.rs:63-77
float corr_at_lag(const double* model, const double* solver, int n, int lag) {
    std::vector<float> a, b;
    a.reserve(n);
    b.reserve(n);
    for (int i = 0; i < n; i++) {
        const int si = i - lag;
        if (si >= 0 && si < n) {
            a.push_back((float)model[i]);
            b.push_back((float)solver[si]);
        }
    }
    if (a.size() < 3) return -INFINITY;
    return correlation(a.data(), b.data(), (int)a.size());
}

// metrics.rs:81-101
float xcorr_lag(const double* model, const double* solver, int n, int max_lag) {
    int best_lag = 0;
    float best_c = -INFINITY;
    for (int lag = -max_lag; lag <= max_lag; lag++) {
        const float c = corr_at_lag(model, solver, n, lag);
        if (c > best_c) {
            best_c = c;
            best_lag = lag;
        }
    }
    if (best_lag > -max_lag && best_lag < max_lag) {
        const float l = corr_at_lag(model, solver, n, best_lag - 1), c = best_c,
                    r = corr_at_lag(model, solver, n, best_lag + 1);
        if (std::isfinite(l) && std::isfinite(r)) {
            const float den = l - 2.0f * c + r;
            if (den < 0.0f) return (float)best_lag + 0.5f * (l - r) / den;
        }
    }
    return (float)best_lag;
}

float corr_of(double sab, double saa, double sbb) {
    if (saa <= 0.0 || sbb <= 0.0) return 0.0f;
    return (float)(sab / std::sqrt(saa * sbb));
}

// eval.rs:165-171 from one record and its profiles.
jc_eval_row finish(const ScoreRec& r, const double* prof, int cap) {
    jc_eval_row row;
    row.corr = corr_of(r.sab, r.saa, r.sbb);
    row.corr_h = corr_of(r.sab_h, r.saa_h, r.sbb_h);
    row.amplitude_ratio = r.peak_m / r.peak_t;
    row.lag = xcorr_lag(prof, prof + cap, r.len, 8);
    row.bias = (r.mean_m - r.mean_t) / std::max(r.std_t, 1e-12f);
    return row;
}

// Normalizer::encode (norm.rs:27-34), host.
void encode(const jc_config& c, const float* h, const float* u, const float* v, long long n, float* out) {
    for (long long i = 0; i < n; i++) {
        out[i] = (h[i] - c.norm_depth - c.norm_mean[0]) / c.norm_std[0];
        out[n + i] = (u[i] - c.norm_mean[1]) / c.norm_std[1];
        out[2 * n + i] = (v[i] - c.norm_mean[2]) / c.norm_std[2];
    }
}

// Drop centres enter integer row and column bounds: keep them finite and
// within a million cells of the grid.
void check_centre(float cx, float cy) {
    if (!(std::fabs(cx) < 1e6f) || !(std::fabs(cy) < 1e6f))
        throw Error(JC_BAD_ARGUMENT, "drop centres must be finite and within 1e6 cells");
}

void initial_state(const jc_config& c, const jc_drop& d, float* phys, float* x) {
    check_centre(d.cx, d.cy);
    const long long cells = (long long)c.nx * c.ny;
    std::fill(phys, phys + cells, c.depth);
    std::fill(phys + cells, phys + 3 * cells, 0.0f);
    add_drop(c.nx, c.ny, phys, d.cx, d.cy, d.amp, d.sigma);
    encode(c, phys, phys + cells, phys + 2 * cells, cells, x);
}

// ---- the evaluator ------------------------------------------------------------

class Evaluator : public TickHook {
   public:
    Evaluator(jc_model* handle, int max_traj) : m_(handle->m), max_(max_traj) {
        if (max_traj < 1) throw Error(JC_BAD_ARGUMENT, "max_trajectories must be >= 1");
        const jc_config& c = m_->cfg;
        cells_ = (long long)c.nx * c.ny;
        len_ = 3 * cells_;
        cap_ = profile_cap(c.nx, c.ny);
        jc_model* list[1] = {handle};
        batch_.reset(new Batch(list, 1, max_traj, max_traj * cells_));
        cuda_check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
        for (int i = 0; i < 2; i++) truth_[i] = arena_.alloc_n<float>(max_ * len_);
        x0_ = arena_.alloc_n<float>(max_ * len_);
        final_ = arena_.alloc_n<float>(max_ * len_);
        meta_ = arena_.alloc_n<float>(64);
        centres_ = arena_.alloc_n<float>(2 * max_);
        xptr_ = arena_.alloc_n<const float*>(max_);
        std::vector<float> meta(64, 0.f);
        m_->meta_of(meta.data());
        cuda_check(cudaMemcpy(meta_, meta.data(), 64 * 4, cudaMemcpyHostToDevice), "meta upload", JC_MAP);
        cuda_check(cudaMallocHost(&h_states_, 2 * max_ * len_ * sizeof(float)), "cudaMallocHost", JC_OVER_BUDGET);
        jc_sw_params sp{c.nx, c.ny, c.dx, c.dt, c.g, c.depth, c.nu};
        sw_ = sw_dev(sp);
        sa_ = score_args(c, cap_);
    }
    ~Evaluator() override {
        if (h_states_) cudaFreeHost(h_states_);
        if (stream_) cudaStreamDestroy(stream_);
    }

    void run(const jc_drop* drops, int n, const int32_t* horizons, int nh, uint32_t flags, jc_eval_row* rows,
             double* max_violation) {
        if (n < 1 || n > max_) throw Error(JC_BAD_ARGUMENT, "trajectory count outside [1, max_trajectories]");
        if (!drops || !horizons || !rows || nh < 1) throw Error(JC_BAD_ARGUMENT, "null argument or no horizons");
        if (flags & ~3u) throw Error(JC_BAD_ARGUMENT, "unknown flag");
        for (int i = 0; i < nh; i++)
            if (horizons[i] < 1 || (i > 0 && horizons[i] <= horizons[i - 1]))
                throw Error(JC_BAD_ARGUMENT, "horizons must be >= 1 and strictly ascending");
        const jc_config& c = m_->cfg;
        n_ = n;
        horizons_.assign(horizons, horizons + nh);
        grow_records(nh);
        // initial solver states and their encodings (eval.rs:135-139)
        float* H = h_states_;
        float* X = h_states_ + max_ * len_;
        std::vector<float> cen(2 * n);
        for (int k = 0; k < n; k++) {
            initial_state(c, drops[k], H + k * len_, X + k * len_);
            cen[2 * k] = drops[k].cx;
            cen[2 * k + 1] = drops[k].cy;
        }
        cuda_check(cudaMemcpyAsync(truth_[0], H, n * len_ * sizeof(float), cudaMemcpyHostToDevice, stream_),
                   "H2D", JC_MAP);
        cuda_check(cudaMemcpyAsync(x0_, X, n * len_ * sizeof(float), cudaMemcpyHostToDevice, stream_), "H2D", JC_MAP);
        cuda_check(cudaMemcpyAsync(centres_, cen.data(), 2 * n * sizeof(float), cudaMemcpyHostToDevice, stream_),
                   "H2D", JC_MAP);
        std::vector<jc_instance> inst(n);
        std::vector<double> energy(2 * n, 0.0);
        for (int k = 0; k < n; k++) {
            jc_instance& I = inst[k];
            std::memset(&I, 0, sizeof(I));
            I.model = 0;
            I.ticks = horizons_.back();
            I.flags = flags;
            I.task = 0;
            I.x0 = x0_ + k * len_;
            I.meta = meta_;
            I.final_state = final_ + k * len_;
            I.energy = &energy[2 * k];
        }
        batch_->rollout(inst.data(), n, true, stream_, this);
        // records and profiles of every horizon
        std::vector<ScoreRec> rec((size_t)nh * max_);
        std::vector<double> prof((size_t)nh * max_ * 2 * cap_);
        cuda_check(cudaMemcpyAsync(rec.data(), recs_, rec.size() * sizeof(ScoreRec), cudaMemcpyDeviceToHost, stream_),
                   "D2H", JC_MAP);
        cuda_check(cudaMemcpyAsync(prof.data(), profs_, prof.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_),
                   "D2H", JC_MAP);
        cuda_check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize", JC_POLL);
        for (int i = 0; i < nh; i++)
            for (int k = 0; k < n; k++) {
                const size_t slot = (size_t)i * max_ + k;
                rows[(size_t)i * n + k] = finish(rec[slot], prof.data() + slot * 2 * cap_, cap_);
            }
        if (max_violation) {
            double w = 0.0;
            for (int k = 0; k < n; k++) w = std::max(w, energy[2 * k + 1]);
            *max_violation = w;
        }
    }

    void bind(const std::vector<float*>& states, cudaStream_t s) override {
        cuda_check(cudaMemcpyAsync(xptr_, states.data(), states.size() * sizeof(float*), cudaMemcpyHostToDevice, s),
                   "state pointers", JC_MAP);
        // the copy reads `states` after this call returns: keep it alive
        cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
    }

    void after_tick(int t, cudaStream_t s) const override {
        sw_step(sw_, truth_[(t - 1) & 1], truth_[t & 1], n_, s);
        for (size_t i = 0; i < horizons_.size(); i++)
            if (horizons_[i] == t)
                score(sa_, xptr_, truth_[t & 1], len_, centres_, n_, recs_ + i * max_,
                      profs_ + (long long)i * max_ * 2 * cap_, s);
    }

    long long key() const override {
        unsigned long long h = 1469598103934665603ull;
        auto mix = [&](unsigned long long v) { h = (h ^ v) * 1099511628211ull; };
        mix((unsigned long long)(uintptr_t)this);
        mix((unsigned long long)n_);
        mix((unsigned long long)(uintptr_t)recs_);
        mix((unsigned long long)(uintptr_t)profs_);
        for (int hz : horizons_) mix((unsigned long long)hz);
        return (long long)(h >> 1);
    }

   private:
    void grow_records(int nh) {
        if (nh <= rec_h_) return;
        if (recs_) arena_.release(recs_);
        if (profs_) arena_.release(profs_);
        recs_ = arena_.alloc_n<ScoreRec>((size_t)nh * max_);
        profs_ = arena_.alloc_n<double>((size_t)nh * max_ * 2 * cap_);
        cuda_check(cudaMemset(profs_, 0, (size_t)nh * max_ * 2 * cap_ * sizeof(double)), "cudaMemset");
        rec_h_ = nh;
    }

    Model* m_;
    int max_;
    long long cells_ = 0, len_ = 0;
    int cap_ = 0;
    std::unique_ptr<Batch> batch_;
    cudaStream_t stream_ = nullptr;
    DeviceArena arena_;
    float* truth_[2] = {nullptr, nullptr};
    float *x0_ = nullptr, *final_ = nullptr, *meta_ = nullptr, *centres_ = nullptr;
    const float** xptr_ = nullptr;
    ScoreRec* recs_ = nullptr;
    double* profs_ = nullptr;
    int rec_h_ = 0;
    float* h_states_ = nullptr;  // pinned: solver states | encoded states
    int n_ = 0;
    std::vector<int> horizons_;
    SwDev sw_{};
    ScoreArgs sa_{};
};

}  // namespace ev

// ---- entry points used by the C ABI -------------------------------------------

void sw_run_host(const jc_sw_params& p, float* states, int count, int steps) {
    ev::check_params(p);
    if (count < 0 || steps < 0) throw Error(JC_BAD_ARGUMENT, "count and steps must be >= 0");
    if (count == 0 || steps == 0) return;
    if (!states) throw Error(JC_BAD_ARGUMENT, "null states");
    const size_t bytes = 3 * (size_t)p.nx * p.ny * count * sizeof(float);
    cudaStream_t s;
    cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    DeviceArena a;
    try {
        float* d = static_cast<float*>(a.alloc(bytes));
        float* scratch = static_cast<float*>(a.alloc(bytes));
        cuda_check(cudaMemcpyAsync(d, states, bytes, cudaMemcpyHostToDevice, s), "H2D", JC_MAP);
        ev::sw_run(ev::sw_dev(p), d, scratch, count, steps, s);
        cuda_check(cudaMemcpyAsync(states, d, bytes, cudaMemcpyDeviceToHost, s), "D2H", JC_MAP);
        cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
    } catch (...) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
        throw;
    }
    cudaStreamDestroy(s);
}

void sw_run_device(const jc_sw_params& p, float* d_states, int count, int steps, cudaStream_t s) {
    ev::check_params(p);
    if (count < 0 || steps < 0) throw Error(JC_BAD_ARGUMENT, "count and steps must be >= 0");
    if (count == 0 || steps == 0) return;
    if (!d_states) throw Error(JC_BAD_ARGUMENT, "null states");
    const size_t bytes = 3 * (size_t)p.nx * p.ny * count * sizeof(float);
    void* scratch = nullptr;
    cuda_check(cudaMallocAsync(&scratch, bytes, s), "cudaMallocAsync", JC_OVER_BUDGET);
    try {
        ev::sw_run(ev::sw_dev(p), d_states, static_cast<float*>(scratch), count, steps, s);
    } catch (...) {
        cudaFreeAsync(scratch, s);
        throw;
    }
    cuda_check(cudaFreeAsync(scratch, s), "cudaFreeAsync");
}

namespace ev {
// h_k += field_f for the drops (k, f) landing at this tick; blockIdx.y = drop.
__global__ void __launch_bounds__(256) add_fields_kernel(float* states, long long state_stride, const int* traj,
                                                         const float* fields, long long n) {
    const int f = blockIdx.y;
    float* h = states + (long long)traj[f] * state_stride;
    const float* d = fields + (long long)f * n;
    for (long long i = (long long)blockIdx.x * 256 + threadIdx.x; i < n; i += (long long)gridDim.x * 256)
        h[i] = __fadd_rn(h[i], d[i]);
}

// Frame t of trajectory k (blockIdx.y): its state's three planes to
// frames_k + (c (T_k + 1) + t) n.
__global__ void __launch_bounds__(256) capture_kernel(const float* states, long long state_stride, float* const* frames,
                                                      const int* nframes, int t, long long n) {
    const int k = blockIdx.y;
    const float* s = states + (long long)k * state_stride;
    float* f = frames[k];
    const long long fc = (long long)nframes[k] * n;  // one channel's frames
    for (long long i = (long long)blockIdx.x * 256 + threadIdx.x; i < 3 * n; i += (long long)gridDim.x * 256) {
        const long long c = i / n, j = i - c * n;
        f[c * fc + (long long)t * n + j] = s[i];
    }
}
}  // namespace ev

void sw_trajectories_host(const jc_sw_params& p, const jc_sw_trajectory* tr, int n) {
    ev::check_params(p);
    if (n < 0 || (n > 0 && !tr)) throw Error(JC_BAD_ARGUMENT, "bad trajectory list");
    if (n == 0) return;
    if (n > 65535) throw Error(JC_LIMIT, "at most 65535 trajectories per call");
    const long long cells = (long long)p.nx * p.ny, len = 3 * cells;
    // longest first, so the trajectories still running at tick t are a prefix
    std::vector<int> order(n);
    for (int k = 0; k < n; k++) {
        const jc_sw_trajectory& t = tr[k];
        if (t.ticks < 0 || !t.x0 || !t.frames || t.n_drops < 0 || (t.n_drops > 0 && (!t.drop_ticks || !t.drop_fields)))
            throw Error(JC_BAD_ARGUMENT, "bad trajectory");
        for (int d = 0; d < t.n_drops; d++)
            if (t.drop_ticks[d] < 1 || t.drop_ticks[d] > t.ticks)
                throw Error(JC_BAD_ARGUMENT, "drop tick outside [1, ticks]");
        order[k] = k;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return tr[a].ticks > tr[b].ticks; });
    const int tmax = tr[order[0]].ticks;
    long long frame_floats = 0, n_fields = 0;
    for (int k = 0; k < n; k++) {
        frame_floats += (long long)(tr[k].ticks + 1) * len;
        n_fields += tr[k].n_drops;
    }
    cudaStream_t s;
    cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    DeviceArena a;
    try {
        float* st = a.alloc_n<float>(n * len);
        float* scratch = a.alloc_n<float>(n * len);
        float* frames = a.alloc_n<float>(frame_floats);
        float* fields = a.alloc_n<float>(std::max(1LL, n_fields) * cells);
        int* ftraj = a.alloc_n<int>(std::max(1LL, n_fields));
        float** fptr = a.alloc_n<float*>(n);
        int* nfr = a.alloc_n<int>(n);
        // packed in `order`: slot i holds trajectory order[i]
        std::vector<float*> hptr(n);
        std::vector<int> hnfr(n);
        std::vector<long long> foff(n);
        long long off = 0;
        for (int i = 0; i < n; i++) {
            const jc_sw_trajectory& t = tr[order[i]];
            cuda_check(cudaMemcpyAsync(st + i * len, t.x0, len * 4, cudaMemcpyHostToDevice, s), "H2D", JC_MAP);
            foff[i] = off;
            hptr[i] = frames + off;
            hnfr[i] = t.ticks + 1;
            off += (long long)(t.ticks + 1) * len;
        }
        cuda_check(cudaMemcpyAsync(fptr, hptr.data(), n * sizeof(float*), cudaMemcpyHostToDevice, s), "H2D", JC_MAP);
        cuda_check(cudaMemcpyAsync(nfr, hnfr.data(), n * sizeof(int), cudaMemcpyHostToDevice, s), "H2D", JC_MAP);
        // drop fields grouped into launches by landing tick; a trajectory's
        // drops of one tick go to successive launches, in their order (the
        // order apply_pending adds them in)
        struct Launch {
            int tick, first, count;
        };
        std::vector<std::vector<std::pair<int, const float*>>> at(tmax + 1);
        for (int i = 0; i < n; i++) {
            const jc_sw_trajectory& t = tr[order[i]];
            for (int d = 0; d < t.n_drops; d++) at[t.drop_ticks[d]].push_back({i, t.drop_fields + (size_t)d * cells});
        }
        std::vector<Launch> launches;
        std::vector<int> htraj;
        long long fi = 0;
        for (int t = 1; t <= tmax; t++) {
            std::vector<int> rank(n, 0);  // drops of each trajectory placed so far at this tick
            for (int rnk = 0;; rnk++) {
                const long long first = fi;
                std::fill(rank.begin(), rank.end(), 0);
                for (auto& pr : at[t]) {
                    if (rank[pr.first]++ != rnk) continue;
                    cuda_check(cudaMemcpyAsync(fields + fi * cells, pr.second, cells * 4, cudaMemcpyHostToDevice, s),
                               "H2D", JC_MAP);
                    htraj.push_back(pr.first);
                    fi++;
                }
                if (fi == first) break;
                if (fi - first > 65535) throw Error(JC_LIMIT, "too many drops at one tick");
                launches.push_back({t, (int)first, (int)(fi - first)});
            }
        }
        if (!htraj.empty())
            cuda_check(cudaMemcpyAsync(ftraj, htraj.data(), htraj.size() * sizeof(int), cudaMemcpyHostToDevice, s),
                       "H2D", JC_MAP);
        const ev::SwDev d = ev::sw_dev(p);
        const unsigned gx = (unsigned)std::min<long long>((3 * cells + 255) / 256, 1024);
        ev::capture_kernel<<<dim3(gx, n), 256, 0, s>>>(st, len, fptr, nfr, 0, cells);
        cuda_check(cudaGetLastError(), "capture launch");
        float* cur = st;
        float* nxt = scratch;
        int active = n;
        size_t li = 0;
        for (int t = 1; t <= tmax; t++) {
            while (active > 0 && tr[order[active - 1]].ticks < t) active--;
            ev::sw_step(d, cur, nxt, active, s);
            std::swap(cur, nxt);
            for (; li < launches.size() && launches[li].tick == t; li++) {
                const Launch& L = launches[li];
                const unsigned fx = (unsigned)std::min<long long>((cells + 255) / 256, 1024);
                ev::add_fields_kernel<<<dim3(fx, L.count), 256, 0, s>>>(cur, len, ftraj + L.first,
                                                                        fields + (long long)L.first * cells, cells);
                cuda_check(cudaGetLastError(), "drop launch");
            }
            ev::capture_kernel<<<dim3(gx, active), 256, 0, s>>>(cur, len, fptr, nfr, t, cells);
            cuda_check(cudaGetLastError(), "capture launch");
        }
        for (int i = 0; i < n; i++) {
            const jc_sw_trajectory& t = tr[order[i]];
            cuda_check(cudaMemcpyAsync(t.frames, frames + foff[i], (size_t)(t.ticks + 1) * len * 4,
                                       cudaMemcpyDeviceToHost, s),
                       "D2H", JC_MAP);
        }
        cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
    } catch (...) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
        throw;
    }
    cudaStreamDestroy(s);
}

void sw_add_drop_host(const jc_sw_params& p, float* h, float cx, float cy, float amp, float sigma) {
    ev::check_params(p);
    if (!h) throw Error(JC_BAD_ARGUMENT, "null h");
    ev::add_drop(p.nx, p.ny, h, cx, cy, amp, sigma);
}

void eval_score_host(const jc_config& c, const float* x, const float* truth, const float* centres, int count,
                     jc_eval_row* rows) {
    if (count < 0) throw Error(JC_BAD_ARGUMENT, "count must be >= 0");
    if (count == 0) return;
    if (!x || !truth || !centres || !rows) throw Error(JC_BAD_ARGUMENT, "null argument");
    if (c.nx < 1 || c.ny < 1) throw Error(JC_BAD_SHAPE, "grid must be at least 1 x 1");
    for (int k = 0; k < count; k++) ev::check_centre(centres[2 * k], centres[2 * k + 1]);
    if (!(c.norm_std[0] != 0.0f)) throw Error(JC_BAD_ARGUMENT, "normalizer std must be nonzero");
    const long long len = 3LL * c.nx * c.ny;
    const int cap = ev::profile_cap(c.nx, c.ny);
    cudaStream_t s;
    cuda_check(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "cudaStreamCreate");
    DeviceArena a;
    try {
        float* dx = a.alloc_n<float>(count * len);
        float* dt = a.alloc_n<float>(count * len);
        float* dc = a.alloc_n<float>(2 * count);
        const float** dp = a.alloc_n<const float*>(count);
        ev::ScoreRec* dr = a.alloc_n<ev::ScoreRec>(count);
        double* dprof = a.alloc_n<double>((size_t)count * 2 * cap);
        std::vector<const float*> ptrs(count);
        for (int k = 0; k < count; k++) ptrs[k] = dx + k * len;
        cuda_check(cudaMemcpyAsync(dx, x, count * len * 4, cudaMemcpyHostToDevice, s), "H2D", JC_MAP);
        cuda_check(cudaMemcpyAsync(dt, truth, count * len * 4, cudaMemcpyHostToDevice, s), "H2D", JC_MAP);
        cuda_check(cudaMemcpyAsync(dc, centres, 2 * count * 4, cudaMemcpyHostToDevice, s), "H2D", JC_MAP);
        cuda_check(cudaMemcpyAsync(dp, ptrs.data(), count * sizeof(float*), cudaMemcpyHostToDevice, s), "H2D", JC_MAP);
        ev::score(ev::score_args(c, cap), dp, dt, len, dc, count, dr, dprof, s);
        std::vector<ev::ScoreRec> rec(count);
        std::vector<double> prof((size_t)count * 2 * cap);
        cuda_check(cudaMemcpyAsync(rec.data(), dr, count * sizeof(ev::ScoreRec), cudaMemcpyDeviceToHost, s), "D2H",
                   JC_MAP);
        cuda_check(cudaMemcpyAsync(prof.data(), dprof, prof.size() * sizeof(double), cudaMemcpyDeviceToHost, s),
                   "D2H", JC_MAP);
        cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize", JC_POLL);
        for (int k = 0; k < count; k++) rows[k] = ev::finish(rec[k], prof.data() + (size_t)k * 2 * cap, cap);
    } catch (...) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
        throw;
    }
    cudaStreamDestroy(s);
}

}  // namespace jc

struct jc_eval {
    jc::ev::Evaluator* e;
};

namespace jc {
jc_eval* eval_create(jc_model* m, int max_traj) { return new jc_eval{new ev::Evaluator(m, max_traj)}; }
void eval_destroy(jc_eval* e) {
    delete e->e;
    delete e;
}
void eval_run(jc_eval* e, const jc_drop* drops, int n, const int32_t* horizons, int nh, uint32_t flags,
              jc_eval_row* rows, double* max_violation) {
    e->e->run(drops, n, horizons, nh, flags, rows, max_violation);
}
}  // namespace jc
