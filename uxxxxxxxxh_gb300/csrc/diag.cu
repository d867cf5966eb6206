// Failure-reporting probe: one CTA waits on an mbarrier phase that nothing
// completes (it expects 16 bytes of transaction that no copy delivers), with
// the wait bounded at a caller-given number of SM clocks.  When the bound
// runs out the kernel records the timeout in the device status word exactly
// as the sweep kernels' bounded waits do (flag, then block / plane / slot /
// phase) and returns normally: nothing faults, no copy is in flight, and the
// host reads the status through the same path as after a sweep.
//
// FP64 pipe probe: every SM runs independent chains of DFMA for a fixed
// count, timed with CUDA events; the rate is the ceiling of any sweep in
// native FP64 arithmetic (one DFMA per term and point).
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

// Consumes the chains' sums so the compiler keeps them; written only when a
// sum equals a value it never takes.
__device__ double g_dfma_sink;

constexpr int kDfmaChains = 8;

__global__ void __launch_bounds__(256) k_dfma_rate(int iters, double a, double b) {
    double x[kDfmaChains];
#pragma unroll
    for (int i = 0; i < kDfmaChains; ++i) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kDfmaChains; ++i) x[i] = fma(x[i], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < kDfmaChains; ++i) s += x[i];
    if (s == -1.0e300) g_dfma_sink = s;
}

}  // namespace

cudaError_t probe_dfma_rate(double *per_second, cudaStream_t st) {
    const int sms = device_sm_count(), iters = 4096;
    const dim3 grid(static_cast<unsigned>(sms) * 8u), block(256);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) {
        k_dfma_rate<<<grid, block, 0, st>>>(64, 0.999999, 1e-6);  // warm-up
        e = cudaEventRecord(e0, st);
    }
    if (e == cudaSuccess) {
        k_dfma_rate<<<grid, block, 0, st>>>(iters, 0.999999, 1e-6);
        count_launch(2);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e == cudaSuccess)
        *per_second = static_cast<double>(grid.x) * block.x * iters * kDfmaChains / (static_cast<double>(ms) * 1e-3);
    return e;
}

cudaError_t launch_wait_probe(unsigned *err, long long cycles, cudaStream_t st) {
    k_wait_probe<<<1, 32, 0, st>>>(err, cycles);
    count_launch();
    return cudaGetLastError();
}

}  // namespace uhs
