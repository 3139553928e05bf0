// Shared device-side definitions for the jacobi2000 GB300 engine.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace jc {

// Per-instance projection scalars, f64 (one slot per instance).
struct ProjSlot {
    double mass0;       // target box mean of channel 0
    double energy;      // energy of the current (projected) state
    double max_viol;    // max relative energy violation so far
    double last_scale;  // last energy-projection scale
};

// One grid instance inside a packed launch. Token-level buffers of all
// instances are concatenated row-wise (instance i owns rows
// [row0, row0 + tx*ty)); cell-level channel-last buffers likewise own cells
// [cell0, cell0 + nx*ny). `state` is the instance's normalized
// [channels, ny, nx] f32 state.
// Instances of a launch are sorted by row0 and cell0 (both ascending), so a
// row or cell finds its instance by binary search.
struct InstDev {
    int row0;         // first token row
    int tx, ty;       // token grid
    int nx, ny;       // cell grid
    long long cell0;  // first cell in cell-level packed buffers
    float* state;     // [3][ny][nx], read by the forward, updated by the tick
    float* out;       // where the tick writes (next state or increment)
    const float* pos; // [tx*ty, dim]
    const float* meta;// [meta_dim]
    unsigned flags;   // projection flags: 1 mass, 2 energy, 4 no projection or energy record
    int tile0;        // first 16x16 cell tile of this instance in the launch
    int tt0;          // first 8x16 token tile (tensor-core token conv)
    int ct0;          // first 8x16 cell tile (tensor-core cell conv)
    ProjSlot* slot;   // this instance's projection scalars (device); null = the pack's slot array
};

constexpr int kCellTile = 16;  // side of the cell tiles of the cell-level kernels
constexpr int kConvTX = 8, kConvTY = 16;  // tensor-core conv tiles: 8 wide, 16 high (M = 128)

#ifdef __CUDACC__
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Index of the instance owning token row r: the last i with inst[i].row0 <= r.
__device__ __forceinline__ int inst_of_row(const InstDev* inst, int n, int r) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (inst[mid].row0 <= r) lo = mid; else hi = mid - 1;
    }
    return lo;
}
// The last i in [0, n) with key(i) <= v, for keys non-decreasing in i with
// key(0) <= v, found by a whole warp (every lane calls it with the same
// arguments and gets the answer): 32-way splits, one load per lane per
// round, so ceil(log32 n) dependent loads instead of ceil(log2 n).
template <class Key>
__device__ __forceinline__ int warp_find_last_le(int n, long long v, Key key) {
    const int lane = threadIdx.x & 31;
    int base = 0, span = n;
    while (span > 1) {
        const int step = (span + 31) >> 5;
        const bool le = lane * step < span && key(base + lane * step) <= v;
        const unsigned m = __ballot_sync(0xffffffffu, le);
        const int last = 31 - __clz(m);
        base += last * step;
        span = min(step, span - last * step);
    }
    return base;
}
__device__ __forceinline__ int inst_of_cell(const InstDev* inst, int n, long long c) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (inst[mid].cell0 <= c) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Exact-erf GELU, 0.5 x (1 + erf(x / sqrt 2)) (crates/engine/src/cpu.rs:67-74),
// with CUDA's erff.
__device__ __forceinline__ float gelu_erf(float x) {
    return 0.5f * x * (1.0f + erff(x * 0.70710678118654752440f));
}

// Asynchronous global -> shared copies (no register staging, many in flight
// per thread). `bytes` of the source are copied and the rest of the 4- or
// 16-byte destination is zero-filled, so bytes = 0 writes zeros (the source
// address must still be a valid one).
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(valid ? 4 : 0)
                 : "memory");
}
// Waits for every copy this thread issued (a __syncthreads() must follow
// before other threads read the data).
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// Closes this thread's group of copies issued since the last commit.
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// Waits until at most N of this thread's committed groups are in flight.
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Programmatic dependent launch. A kernel launched with programmatic stream
// serialization may start (be scheduled, set up shared memory, tensor memory
// and barriers) while the previous kernel in the stream is still running.
// JC_PDL_ENTRY lets the next kernel start early, then waits until the previous
// kernel has completed and its writes are visible; every kernel executes it
// before its first access to memory that other kernels write or read.
// Without the launch attribute both instructions are no-ops.
#define JC_PDL_ENTRY                                                      \
    do {                                                                  \
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");  \
        asm volatile("griddepcontrol.wait;" ::: "memory");               \
    } while (0)

// Neumaier compensated accumulator in f64.
struct Neu {
    double s, c;
    __device__ __forceinline__ void init() { s = 0.0; c = 0.0; }
    __device__ __forceinline__ void add(double v) {
        double t = s + v;
        if (fabs(s) >= fabs(v)) c += (s - t) + v; else c += (v - t) + s;
        s = t;
    }
    __device__ __forceinline__ double val() const { return s + c; }
};

#endif  // __CUDACC__

}  // namespace jc
