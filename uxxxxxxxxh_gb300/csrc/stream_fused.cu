// Temporal fusion (the kernel: stream_fused.cuh): rank-3 shapes, the launch
// entry for both ranks, and the device check that both grids hold the same
// halo.
#include "stream_fused.cuh"

namespace uhs {
namespace {

// Number of cells outside the domain whose bytes differ between the grids.
__global__ void k_halo_diff(const unsigned char *pa, const unsigned char *pb, int eb, int64_t s0a, int64_t s1a,
                            int64_t s0b, int64_t s1b, int64_t n0, int64_t n1, int64_t n2, int64_t lb0, int64_t lb1,
                            int64_t lb2, int64_t ub0, int64_t ub1, int64_t ub2, unsigned *count) {
    unsigned bad = 0;
    const int64_t total = n0 * n1;
    for (int64_t row = blockIdx.x * static_cast<int64_t>(blockDim.y) + threadIdx.y; row < total;
         row += static_cast<int64_t>(gridDim.x) * blockDim.y) {
        const int64_t z = row / n1, y = row % n1;
        const bool row_in = z >= lb0 && z < ub0 && y >= lb1 && y < ub1;
        for (int64_t x = threadIdx.x; x < n2; x += blockDim.x) {
            if (row_in && x >= lb2 && x < ub2) continue;
            const unsigned char *ca = pa + ((z * s0a + y * s1a) + x) * eb;
            const unsigned char *cb = pb + ((z * s0b + y * s1b) + x) * eb;
            for (int k = 0; k < eb; ++k)
                if (ca[k] != cb[k]) {
                    ++bad;
                    break;
                }
        }
    }
    if (bad) atomicAdd(count, bad);
}

}  // namespace

cudaError_t launch_fused(const StreamCall &c, int K) {
    if (c.shape == kStar2 || c.shape == kBox2) return launch_fused_2d(c, K);
    return fused::launch_fused_rank<kStar3, kBox3>(c, K);
}

cudaError_t launch_halo_diff(const GridView &a, const GridView &b, int eb, const int64_t lb[3], const int64_t ub[3],
                             unsigned *count, int sms, cudaStream_t st) {
    const int64_t rows = a.n[0] * a.n[1];
    const unsigned blocks = static_cast<unsigned>(std::max<int64_t>(1, std::min<int64_t>((rows + 7) / 8, int64_t(sms) * 16)));
    k_halo_diff<<<blocks, dim3(32, 8), 0, st>>>(static_cast<const unsigned char *>(a.data),
                                                static_cast<const unsigned char *>(b.data), eb, a.s[0], a.s[1], b.s[0],
                                                b.s[1], a.n[0], a.n[1], a.n[2], lb[0], lb[1], lb[2], ub[0], ub[1], ub[2],
                                                count);
    count_launch();
    return cudaGetLastError();
}

}  // namespace uhs
