// selftest.cu -- failure-detection self-tests: a bounded wait that runs out,
// and injected device-allocation failures.
//
// The kernels never trap: every wait on a bulk-copy mbarrier has an
// iteration limit, after which the waiting thread sets kErrWaitTimeout in the
// device error word and the kernel finishes (the host turns the bit into
// NBGB_ERR_DEVICE_TIMEOUT).  This entry point exercises exactly that path on
// demand: one thread waits, through the production mbar_wait(), on an
// mbarrier nothing ever arrives at, with a caller-chosen iteration limit.
#include "bh.cuh"
#include "common.cuh"
#include "runtime.cuh"

namespace nbgb {

__global__ void wait_timeout_kernel(uint32_t* err, uint32_t max_iters) {
  __shared__ alignas(8) uint64_t bar;
  if (threadIdx.x == 0) mbar_init(&bar, 1);  // expects one arrival that never comes
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait(&bar, 0, err, max_iters);
  __syncthreads();
}

}  // namespace nbgb

using namespace nbgb;

extern "C" nbgb_status nbgb_selftest_wait_timeout(uint32_t max_iters, uint32_t* error_bits) {
  uint32_t* d = nullptr;
  uint32_t h = 0;
  try {
    if (max_iters == 0 || max_iters > (1u << 20))
      fail(NBGB_ERR_INVALID_ARG, "Validation Error: iteration limit must be in [1, 2^20]");
    NBGB_CUDA(cudaMalloc(&d, sizeof(uint32_t)));
    NBGB_CUDA(cudaMemset(d, 0, sizeof(uint32_t)));
    wait_timeout_kernel<<<1, 32>>>(d, max_iters);
    NBGB_LAUNCH_CHECK();
    NBGB_CUDA(cudaDeviceSynchronize());
    NBGB_CUDA(cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost));
    cudaFree(d);
  } catch (const Error& e) {
    if (d) cudaFree(d);
    return set_error(e.status, e.what());
  }
  if (error_bits) *error_bits = h;
  if (h & kErrWaitTimeout)
    return set_error(NBGB_ERR_DEVICE_TIMEOUT, "device wait ran out of iterations (self-test)");
  return NBGB_OK;
}

namespace nbgb {
std::atomic<int64_t> g_alloc_fault_countdown{0};
}

extern "C" nbgb_status nbgb_selftest_fail_allocation(int32_t nth) {
  if (nth < 0)
    return set_error(NBGB_ERR_INVALID_ARG, "Validation Error: allocation index must be >= 0");
  g_alloc_fault_countdown.store(nth);
  return set_error(NBGB_OK, std::string());
}

extern "C" nbgb_status nbgb_selftest_group_walk_stack(int32_t entries) {
  if (entries < 64 || entries > 512)
    return set_error(NBGB_ERR_INVALID_ARG, "Validation Error: stack entries must be in [64, 512]");
  bh_set_group_stack_limit(entries);
  return NBGB_OK;
}
