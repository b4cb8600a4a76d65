// Diagnostic: the bounded-wait path of the kernels, exercised on purpose.
//
// Every mbarrier wait of the tcgen05 kernels gives up after a time limit,
// raises CORR_ERR_DEVICE_TIMEOUT in the call's status word and lets the CTA
// wind down, so a lost arrival never hangs the GPU.  This entry point runs
// that path: one CTA waits, with the same primitive, on an mbarrier phase that
// nothing completes, for a caller-chosen limit.  No fault, trap or unbounded
// loop is involved; the context stays usable afterwards.
#include "abi_internal.h"
#include "common.cuh"

namespace corr {
namespace {

__global__ void wait_selftest_kernel(unsigned long long limit_ns, int* status) {
  __shared__ uint64_t bar;
  __shared__ int abort_flag;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);  // one arrival expected; none is ever made
    abort_flag = 0;
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_wait_for(&bar, 0, &abort_flag, status, limit_ns);
}

}  // namespace
}  // namespace corr

using namespace corr;

extern "C" {

int corr_selftest_wait_timeout(corr_context* c, int limit_ms) {
  CORR_CHECK_ARG(c != nullptr, "null context");
  CORR_CHECK_ARG(limit_ms >= 1 && limit_ms <= 2000,
                 "corr_selftest_wait_timeout: limit_ms must be in [1, 2000]");
  CORR_CUDA(cudaSetDevice(c->device));
  CORR_CUDA(cudaMemsetAsync(c->dres, 0, sizeof(ResultBlock), c->stream));
  wait_selftest_kernel<<<1, 32, 0, c->stream>>>((unsigned long long)limit_ms * 1000000ull,
                                                &c->dres->status);
  CORR_CUDA(cudaGetLastError());
  c->launches += 1;
  return finish_results(c, 0);
}

}  // extern "C"
