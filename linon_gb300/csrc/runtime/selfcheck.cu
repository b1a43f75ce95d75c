// selfcheck.cu — exercises the failure path of the bounded device waits.
//
// The march kernels stage small scenes into shared memory with one bulk copy
// and wait for it on an mbarrier with a bounded number of polls
// (march.cuh mbar_wait_bounded); when the budget runs out the kernel sets
// error bit 1 in the context's error word, and linon_synchronize reports
// LINON_ETIMEOUT.  This kernel runs that wait on an mbarrier that no copy and
// no thread ever completes, so the wait always runs out: it tests the path
// without a fault, a hang or anything left in flight (no copy is issued).
#include "../device/march.cuh"
#include "kernels.hpp"

namespace linon {
namespace {

__global__ void __launch_bounds__(32) bounded_wait_check_kernel(int* err, int polls) {
  __shared__ unsigned long long bar;
  const unsigned b = smem_addr(&bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(b), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // phase 0 expects one arrival that never comes
  const bool done = mbar_wait_bounded(b, 0, polls);
  if (threadIdx.x == 0 && !done) atomicOr(err, 1);
}

}  // namespace

cudaError_t launch_bounded_wait_check(int* err, int polls, cudaStream_t stream) {
  bounded_wait_check_kernel<<<1, 32, 0, stream>>>(err, polls);
  return cudaGetLastError();
}

}  // namespace linon
