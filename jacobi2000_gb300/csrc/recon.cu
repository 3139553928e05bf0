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

__global__ void recon_init_kernel(ReconDev* rd) {
    ReconDev& R = rd[blockIdx.y];
    const long long per = 3 * R.cells, total = (long long)(R.H + 1) * per;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(i / per);
        const long long cell = (i - (long long)t * per) % R.cells;
        R.vol[i] = R.known[(long long)t * R.cells + cell] ? R.vals[i] : 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        R.sweeps = 0;
        R.frozen = 0;
        R.resid_bits = 0u;
        R.last_resid = 0.f;
    }
}

__global__ void recon_update_kernel(ReconDev* rd) {
    __shared__ float red[32];
    ReconDev& R = rd[blockIdx.y];
    if (R.frozen) return;  // uniform per block
    const long long per = 3 * R.cells, total = (long long)(R.H + 1) * per;
    const int H = R.H;
    float local = 0.f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int t = (int)(i / per);
        const long long rem = i - (long long)t * per, cell = rem % R.cells;
        if (R.known[(long long)t * R.cells + cell]) continue;  // stays the known value
        float v;
        if (t == 0) v = R.R[rem];
        else if (t == H) v = R.F[(long long)(H - 1) * per + rem];
        else v = 0.5f * (R.F[(long long)(t - 1) * per + rem] + R.R[(long long)t * per + rem]);
        local = fmaxf(local, fabsf(v - R.vol[i]));
        R.vol[i] = v;
    }
    local = warp_max(local);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x < 32) {
        float v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        v = warp_max(v);
        if (threadIdx.x == 0) atomicMax(&R.resid_bits, __float_as_uint(v));
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

void recon_init(ReconDev* d, int n, cudaStream_t s) {
    if (n == 0) return;
    KScope k("recon_init", s);
    recon_init_kernel<<<dim3(256, n), 256, 0, s>>>(d);
    check("recon_init");
}

void recon_update(ReconDev* d, int n, cudaStream_t s) {
    if (n == 0) return;
    KScope k("recon_update", s);
    recon_update_kernel<<<dim3(256, n), 256, 0, s>>>(d);
    check("recon_update");
}

void recon_finalize(ReconDev* d, int n, unsigned long long handle, int use_handle, cudaStream_t s) {
    if (n == 0) return;
    KScope k("recon_finalize", s);
    recon_finalize_kernel<<<1, 256, 0, s>>>(d, n, (cudaGraphConditionalHandle)handle, use_handle);
    check("recon_finalize");
}

}  // namespace jc
