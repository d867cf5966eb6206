// Failure-reporting probe: one CTA waits on an mbarrier phase that nothing
// completes (it expects 16 bytes of transaction that no copy delivers), with
// the wait bounded at a caller-given number of SM clocks.  When the bound
// runs out the kernel records the timeout in the device status word exactly
// as the sweep kernels' bounded waits do (flag, then block / plane / slot /
// phase) and returns normally: nothing faults, no copy is in flight, and the
// host reads the status through the same path as after a sweep.
#include <cuda_runtime.h>

#include <cstdint>

#include "uhs_kernels.h"

namespace uhs {
namespace {

__global__ void k_wait_probe(unsigned *err, long long cycles) {
    __shared__ __align__(8) uint64_t bar;
    const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(&bar));
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(a) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        // arrive with 16 bytes of expected transaction that never arrive
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], 16;\n" ::"r"(a) : "memory");
    }
    __syncthreads();
    const long long t0 = clock64();
    bool done = false;
    while (!done) {
        unsigned r;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(r)
            : "r"(a)
            : "memory");
        done = r != 0;
        if (!done && clock64() - t0 > cycles) break;
    }
    if (__syncthreads_or(!done) && threadIdx.x == 0) {
        atomicOr(err, kDevErrTimeout);
        if (atomicCAS(err + 2, 0u, 1u) == 0u) {
            err[3] = blockIdx.x;
            err[4] = blockIdx.z;
            err[5] = 0;
            err[6] = 0;
            err[7] = 0;
        }
    }
}

}  // namespace

cudaError_t launch_wait_probe(unsigned *err, long long cycles, cudaStream_t st) {
    k_wait_probe<<<1, 32, 0, st>>>(err, cycles);
    count_launch();
    return cudaGetLastError();
}

}  // namespace uhs
