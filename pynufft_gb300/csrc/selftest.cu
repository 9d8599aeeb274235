// Self-test of the bounded mbarrier wait used by the bulk-copy kernels: one
// block arms an mbarrier for 16 bytes of transactions that no copy will ever
// deliver, waits with a bounded number of polls and records whether the wait
// ran out.  Nothing faults or hangs: the wait always ends, no copy is in
// flight, and the context stays usable.  No counterpart in the reference.
#include "interp.cuh"

namespace nufft {

__global__ void bounded_wait_selftest_kernel(int polls, int* __restrict__ result) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_arrive_expect_tx(&bar, 16u);   // bytes that never arrive
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0, polls);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) *result = 1;
}

}  // namespace nufft

extern "C" int nufft_selftest_bounded_wait(int polls, int* timed_out) {
    using namespace nufft;
    if (polls < 1 || polls > (1 << 22) || !timed_out) {
        set_error("nufft_selftest_bounded_wait: polls must be in [1, 2^22] and timed_out non-NULL");
        return NUFFT_EINVAL;
    }
    int* d = nullptr;
    NUFFT_CUDA_TRY(cudaMalloc(&d, sizeof(int)));
    cudaError_t e = cudaMemset(d, 0, sizeof(int));
    if (e == cudaSuccess) {
        bounded_wait_selftest_kernel<<<1, 64>>>(polls, d);
        e = cudaGetLastError();
    }
    int h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) {
        set_error(std::string("nufft_selftest_bounded_wait: ") + cudaGetErrorString(e));
        return NUFFT_ECUDA;
    }
    *timed_out = h;
    return NUFFT_OK;
}
