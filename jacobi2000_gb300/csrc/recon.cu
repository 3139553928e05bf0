// Reconstruct sweeps of the batch runner (the device side of its CUDA-graph
// while loop). Rule: X_t <- known_t ? value : mean of step_F(X_{t-1}) and
// step_R(X_{t+1}) where they exist, from X = 0 at unknown cells; an instance
// stops (freezes) when its largest change falls below its tolerance or it has
// run its sweep limit; the loop ends when every instance is frozen.
#include <stdexcept>
#include <string>

#include "engine.hpp"

namespace jc {

namespace {

void check(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// Layout of the volume kernels: one CTA per (block of 4 x blockDim.x cells,
// instance, time slice) - grid (x, y, z) - and one thread per 4 consecutive
// cells of one slice, all three channels; no loops and no index divisions,
// so every load of the slice is in flight at once. When the cell count is a
// multiple of 4 (grid sides are multiples of the patch) and the slice's
// planes start on 16-byte boundaries (and its mask on a 4-byte one), a
// thread moves its 4 cells as one 16-byte value per plane; otherwise it
// moves them one by one.
__device__ __forceinline__ bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }
__device__ __forceinline__ bool aligned4(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 3u) == 0; }

__global__ void recon_init_kernel(ReconDev* rd) {
    ReconDev& R = rd[blockIdx.y];
    const int t = (int)blockIdx.z;
    const long long cells = R.cells, per = 3 * cells;
    const long long c0 = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (blockIdx.x == 0 && t == 0 && threadIdx.x == 0) {
        R.sweeps = 0;
        R.frozen = 0;
        R.resid_bits = 0u;
        R.last_resid = 0.f;
    }
    if (t > R.H || c0 >= cells) return;
    float* __restrict__ vol = R.vol + (long long)t * per;
    const float* __restrict__ vals = R.vals + (long long)t * per;
    const uint8_t* __restrict__ known = R.known + (long long)t * cells;
    struct {
        float* vol;
        const float* vals;
        const uint8_t* known;
        long long cells;
        __device__ void one(long long c) {
            const bool k = known[c] != 0;
            for (int ch = 0; ch < 3; ch++) vol[ch * cells + c] = k ? vals[ch * cells + c] : 0.0f;
        }
        __device__ void vec(long long c) {
            const uchar4 k = *reinterpret_cast<const uchar4*>(known + c);
#pragma unroll
            for (int ch = 0; ch < 3; ch++) {
                const float4 v = *reinterpret_cast<const float4*>(vals + ch * cells + c);
                *reinterpret_cast<float4*>(vol + ch * cells + c) =
                    make_float4(k.x ? v.x : 0.f, k.y ? v.y : 0.f, k.z ? v.z : 0.f, k.w ? v.w : 0.f);
            }
        }
    } op{vol, vals, known, cells};
    if ((cells & 3) == 0 && aligned16(vol) && aligned16(vals) && aligned4(known)) {
        op.vec(c0);
    } else {
        for (long long c = c0; c < c0 + 4 && c < cells; c++) op.one(c);
    }
}

__global__ void recon_update_kernel(ReconDev* rd) {
    __shared__ float red[32];
    const ReconDev& R = rd[blockIdx.y];
    const int t = (int)blockIdx.z, H = R.H;
    if (R.frozen || t > H) return;  // uniform per block
    const long long cells = R.cells, per = 3 * cells;
    const long long c0 = 4 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    float local = 0.f;
    if (c0 < cells) {
        // v = F_t and / or R_t: slice t of the volume from the steps on either side
        float* __restrict__ vol = R.vol + (long long)t * per;
        const float* __restrict__ fs = t > 0 ? R.F + (long long)(t - 1) * per : nullptr;
        const float* __restrict__ rs = t < H ? R.R + (long long)t * per : nullptr;
        const uint8_t* __restrict__ known = R.known + (long long)t * cells;
        auto upd = [&](float v, float& cur) {
            local = fmaxf(local, fabsf(v - cur));
            cur = v;
        };
        auto val = [&](long long i) { return !fs ? rs[i] : !rs ? fs[i] : 0.5f * (fs[i] + rs[i]); };
        const bool vec = (cells & 3) == 0 && aligned16(vol) && aligned4(known) && (!fs || aligned16(fs)) &&
                         (!rs || aligned16(rs));
        if (vec) {
            const uchar4 k = *reinterpret_cast<const uchar4*>(known + c0);
#pragma unroll
            for (int ch = 0; ch < 3; ch++) {
                const long long i = ch * cells + c0;
                float4 cur = *reinterpret_cast<const float4*>(vol + i);
                float4 v;
                if (!fs) {
                    v = *reinterpret_cast<const float4*>(rs + i);
                } else if (!rs) {
                    v = *reinterpret_cast<const float4*>(fs + i);
                } else {
                    const float4 f = *reinterpret_cast<const float4*>(fs + i), r = *reinterpret_cast<const float4*>(rs + i);
                    v = make_float4(0.5f * (f.x + r.x), 0.5f * (f.y + r.y), 0.5f * (f.z + r.z), 0.5f * (f.w + r.w));
                }
                if (!k.x) upd(v.x, cur.x);
                if (!k.y) upd(v.y, cur.y);
                if (!k.z) upd(v.z, cur.z);
                if (!k.w) upd(v.w, cur.w);
                *reinterpret_cast<float4*>(vol + i) = cur;
            }
        } else {
            for (long long c = c0; c < c0 + 4 && c < cells; c++) {
                if (known[c]) continue;  // a known value stays
                for (int ch = 0; ch < 3; ch++) upd(val(ch * cells + c), vol[ch * cells + c]);
            }
        }
    }
    local = warp_max(local);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        v = warp_max(v);
        if (threadIdx.x == 0) atomicMax(const_cast<unsigned*>(&R.resid_bits), __float_as_uint(v));
    }
}

__global__ void recon_finalize_kernel(ReconDev* rd, int n, cudaGraphConditionalHandle h, int use_handle) {
    __shared__ int running;
    if (threadIdx.x == 0) running = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        ReconDev& R = rd[i];
        if (!R.frozen) {
            R.sweeps += 1;
            const float r = __uint_as_float(R.resid_bits);
            R.last_resid = r;
            R.resid_bits = 0u;
            if (r < R.tol || R.sweeps >= R.max_sweeps) R.frozen = 1;
        }
        if (!R.frozen) atomicOr(&running, 1);
    }
    __syncthreads();
    if (threadIdx.x == 0 && use_handle) cudaGraphSetConditional(h, running ? 1u : 0u);
}

}  // namespace

static dim3 recon_grid(int n, long long max_cells, int max_h) {
    return dim3((unsigned)((max_cells + 4 * 256 - 1) / (4 * 256)), (unsigned)n, (unsigned)(max_h + 1));
}

void recon_init(ReconDev* d, int n, long long max_cells, int max_h, cudaStream_t s) {
    if (n == 0) return;
    KScope k("recon_init", s);
    recon_init_kernel<<<recon_grid(n, max_cells, max_h), 256, 0, s>>>(d);
    check("recon_init");
}

void recon_update(ReconDev* d, int n, long long max_cells, int max_h, cudaStream_t s) {
    if (n == 0) return;
    KScope k("recon_update", s);
    recon_update_kernel<<<recon_grid(n, max_cells, max_h), 256, 0, s>>>(d);
    check("recon_update");
}

void recon_finalize(ReconDev* d, int n, unsigned long long handle, int use_handle, cudaStream_t s) {
    if (n == 0) return;
    KScope k("recon_finalize", s);
    recon_finalize_kernel<<<1, 256, 0, s>>>(d, n, (cudaGraphConditionalHandle)handle, use_handle);
    check("recon_finalize");
}

}  // namespace jc
