// Exponent range of an FP64 grid, for choosing the arithmetic of an FP64
// program: float pairs (df32) hold a value to 2^-48 of itself only between
// 2^-74 and 2^128, so the planner runs df32 only when the largest magnitude,
// grown by (sum |c|)^T, stays well below 2^128 and the smallest nonzero
// magnitude well above 2^-74.  Reads the grid's whole span (padding
// included) once as 64-bit words and folds the biased exponent fields with
// integer max and min; one atomicMax and one atomicMin per warp.
#include "uhs_kernels.h"

namespace uhs {
namespace {

__global__ void __launch_bounds__(256) k_exponent_range(const unsigned long long *w, int64_t n, unsigned *max_out,
                                                        unsigned *min_out) {
    unsigned hi = 0u, lo = 0x7ffu;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const unsigned long long v = w[i];
        const unsigned e = static_cast<unsigned>(v >> 52) & 0x7ffu;
        hi = max(hi, e);
        if (v << 1) lo = min(lo, e);  // nonzero magnitude (the sign bit shifted out)
    }
    for (int o = 16; o > 0; o >>= 1) {
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(max_out, hi);
        atomicMin(min_out, lo);
    }
}

}  // namespace

cudaError_t launch_exponent_range(const void *data, int64_t n_words, unsigned *max_out, unsigned *min_out, int sms,
                                  cudaStream_t st) {
    if (n_words <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((n_words + 255) / 256, static_cast<int64_t>(sms) * 8);
    k_exponent_range<<<static_cast<unsigned>(blocks), 256, 0, st>>>(static_cast<const unsigned long long *>(data),
                                                                     n_words, max_out, min_out);
    count_launch();
    return cudaGetLastError();
}

}  // namespace uhs
