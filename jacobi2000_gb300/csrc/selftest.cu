// Self-test of the bounded device-side waits: the production mbarrier wait
// (tc::mbar_wait) with a caller-chosen limit, on a barrier that nothing
// arrives on (or, as the control case, one that its own thread completes).
// The kernel gives up, sets the error flag and returns; the host reads the
// flag with the check every batch call uses and reports JC_DEVICE_TIMEOUT.
// No kernel is left running and the context stays usable.
#include "runtime.hpp"
#include "tc.cuh"

namespace jc {

namespace {

__global__ void wait_selftest_kernel(int satisfy, unsigned long long limit_ns, int* err) {
    __shared__ uint64_t bar;
    __shared__ int cta_failed;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_barrier_init();
        cta_failed = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0 && satisfy) tc::mbar_arrive(&bar);
    // every thread of the CTA waits on phase 0; when the limit runs out the
    // first to notice sets the CTA flag and the others return at once
    tc::mbar_wait(&bar, 0, err, &cta_failed, limit_ns);
    __syncthreads();
}

}  // namespace

void selftest_device_wait(int satisfy, unsigned limit_us) {
    if (limit_us < 1 || limit_us > 2000000u) throw Error(JC_BAD_ARGUMENT, "limit_us must be in [1, 2000000]");
    int* flag = nullptr;
    cuda_check(cudaMalloc(&flag, sizeof(int)), "cudaMalloc", JC_OVER_BUDGET);
    struct Free {
        int* p;
        ~Free() { cudaFree(p); }
    } guard{flag};
    cuda_check(cudaMemset(flag, 0, sizeof(int)), "cudaMemset");
    wait_selftest_kernel<<<1, 64>>>(satisfy, (unsigned long long)limit_us * 1000ull, flag);
    cuda_check(cudaGetLastError(), "wait self-test launch");
    check_wait_flag(flag, nullptr);
}

}  // namespace jc
