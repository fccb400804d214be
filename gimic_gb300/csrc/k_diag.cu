// Self-test of the bounded device waits (no reference counterpart).
//
// Every pipeline wait of the library gives up after a time limit, records a
// code in the context's device error word and lets its kernel return, so
// that a stalled pipeline becomes GG_ETIMEDOUT on the host instead of a hung
// GPU.  wait_timeout_kernel exercises exactly that path: one thread waits on
// an mbarrier that nothing will ever arrive at, with a short limit, through
// the same mbar_wait_for that the pipeline kernels use.
#include "gg_kernels.h"

namespace gg {

__global__ void wait_timeout_kernel(int* err, uint64_t limit_ns, int code, unsigned long long* waited_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);  // one arrival expected; none comes
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint64_t t0 = global_ns();
    mbar_wait_for(&bar, 0, err, code, limit_ns);
    if (waited_ns) *waited_ns = global_ns() - t0;
  }
}

cudaError_t launch_wait_timeout(int* err, uint64_t limit_ns, int code, unsigned long long* waited_ns,
                                cudaStream_t st) {
  wait_timeout_kernel<<<1, 32, 0, st>>>(err, limit_ns, code, waited_ns);
  return cudaGetLastError();
}

// One global-timer stamp (ns) on the stream, e.g. the start of a launch
// whose kernels stamp their own completion.
__global__ void stamp_kernel(unsigned long long* p) { *p = global_ns(); }

cudaError_t launch_stamp(unsigned long long* p, cudaStream_t st) {
  stamp_kernel<<<1, 1, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace gg
