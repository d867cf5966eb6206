// Largest binary exponent in an FP64 grid, for choosing the arithmetic of an
// FP64 program: float pairs (df32) cover magnitudes below 2^128, so the
// planner runs df32 only when max|x| * (sum |c|)^T stays well inside that.
// Reads the grid's whole span (padding included) once as 64-bit words and
// folds the biased exponent fields with integer max; one atomicMax per warp.
#include "uhs_kernels.h"

namespace uhs {
namespace {

__global__ void __launch_bounds__(256) k_max_exponent(const unsigned long long *w, int64_t n, unsigned *out) {
    unsigned m = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        m = max(m, static_cast<unsigned>(w[i] >> 52) & 0x7ffu);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

}  // namespace

cudaError_t launch_max_exponent(const void *data, int64_t n_words, unsigned *out, int sms, cudaStream_t st) {
    if (n_words <= 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((n_words + 255) / 256, static_cast<int64_t>(sms) * 8);
    k_max_exponent<<<static_cast<unsigned>(blocks), 256, 0, st>>>(static_cast<const unsigned long long *>(data),
                                                                   n_words, out);
    count_launch();
    return cudaGetLastError();
}

}  // namespace uhs
