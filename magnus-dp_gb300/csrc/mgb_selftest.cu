// Self-test of the bounded device-side wait and its error path.
//
// Every mbarrier wait in the tensor-core and bulk-copy kernels gives up after
// a time limit, raises the device flag g_device_timeout and lets the kernel
// return, so that a lost arrival ends as MGB_ERR_DEVICE_TIMEOUT on the host
// instead of a hung GPU.  This kernel exercises that path on purpose and
// safely: one CTA initialises an mbarrier that nothing will ever arrive at
// (no copy or MMA is issued, nothing is in flight), waits on it with a short
// limit, raises the flag when the wait gives up and returns.
#include <cstdint>

#include "mgb_tc.cuh"
#include "mgb_tuned.h"

namespace mgb {
namespace {

__global__ void k_wait_selftest(uint64_t limit_ns, int* __restrict__ tflag) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar);
        tc::mbar_init_fence();
    }
    __syncthreads();
    const bool ok = tc::mbar_wait_ns(tc::su32(&bar), 0, limit_ns);
    if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(tflag, 1);
}

}  // namespace

cudaError_t launch_wait_selftest(uint64_t limit_ns, cudaStream_t st) {
    int* flag = device_timeout_ptr();
    if (!flag) return cudaErrorInvalidValue;
    k_wait_selftest<<<1, 32, 0, st>>>(limit_ns, flag);
    return cudaGetLastError();
}

}  // namespace mgb
