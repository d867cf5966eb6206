// FP64 grid <-> float-pair grid conversion for pair-resident runs.
// The pairs may hold the values scaled by a power of two (df32.cuh): the
// split applies the run's scale and the join removes it.
//
// A program of T >= 8 float-pair sweeps on FP64 grids (pair_eligible in
// uhs_runtime.cpp) runs on float-pair
// copies of its grids: each FP64 value is split once
// (split_f64) into a {hi, lo} float pair, the T sweeps read and write pairs
// (no split on every load, no join on every store: the sweep kernel's
// float-pair variant), and the domain of each grid a sweep wrote is joined
// back into the FP64 grid at the end.  Cells outside the domain (the halo)
// are read from the FP64 grids' own values and never written back, so they
// stay bit-exact.
#include "df32.cuh"
#include "uhs_kernels.h"

namespace uhs {
namespace {

constexpr int kConvThreads = 256;

struct PairConv {
    const void *src;
    void *dst;
    int64_t s0s, s1s, s0d, s1d;  // row strides (elements) of source and destination
    int64_t n0, n1, n2;          // grid sizes
    int64_t lb0, lb1, lb2, ub0, ub1, ub2;
    int halo_only;  // to pairs: convert only cells outside [lb, ub)
    int bias;       // exponent rebias of the pairs: they hold x * 2^shift (pair_bias, df32.cuh)
    unsigned *err;
};

// FP64 -> pairs over the whole grid, or its halo only: one warp per row at a
// time (rows of the grid, slowest axes flattened), lanes striding along x.
__global__ void __launch_bounds__(kConvThreads) k_to_pairs(const PairConv a) {
    const int64_t rows = a.n0 * a.n1;
    const int wpb = kConvThreads / 32, lane = threadIdx.x & 31;
    unsigned rerr = 0;
    for (int64_t row = static_cast<int64_t>(blockIdx.x) * wpb + (threadIdx.x >> 5); row < rows;
         row += static_cast<int64_t>(gridDim.x) * wpb) {
        const int64_t z = row / a.n1, y = row % a.n1;
        const double *s = static_cast<const double *>(a.src) + z * a.s0s + y * a.s1s;
        float2 *d = static_cast<float2 *>(a.dst) + z * a.s0d + y * a.s1d;
        const bool inner_row = z >= a.lb0 && z < a.ub0 && y >= a.lb1 && y < a.ub1;
        if (a.halo_only && inner_row) {
            // the row's x halo only: [0, lb2) and [ub2, n2)
            const int64_t left = a.lb2, right = a.n2 - a.ub2;
            for (int64_t i = lane; i < left + right; i += 32) {
                const int64_t x = i < left ? i : a.ub2 + (i - left);
                d[x] = split_f64(s[x], rerr, a.bias);
            }
        } else {
#pragma unroll 4
            for (int64_t x = lane; x < a.n2; x += 32) d[x] = split_f64(s[x], rerr, a.bias);
        }
    }
    if (rerr) atomicOr(a.err, kDevErrRange);
}

// pairs -> FP64 over the domain [lb, ub): each value the double nearest
// hi + lo.  One warp per row at a time.  A pair whose hi is Inf or NaN grew
// out of the float range during the sweeps: the range flag is set, as a
// split of an out-of-range value does.
__global__ void __launch_bounds__(kConvThreads) k_from_pairs(const PairConv a) {
    const int64_t ny = a.ub1 - a.lb1, rows = (a.ub0 - a.lb0) * ny;
    const int wpb = kConvThreads / 32, lane = threadIdx.x & 31;
    unsigned rerr = 0;
    for (int64_t row = static_cast<int64_t>(blockIdx.x) * wpb + (threadIdx.x >> 5); row < rows;
         row += static_cast<int64_t>(gridDim.x) * wpb) {
        const int64_t z = a.lb0 + row / ny, y = a.lb1 + row % ny;
        const float2 *s = static_cast<const float2 *>(a.src) + z * a.s0s + y * a.s1s;
        double *d = static_cast<double *>(a.dst) + z * a.s0d + y * a.s1d;
#pragma unroll 4
        for (int64_t x = a.lb2 + lane; x < a.ub2; x += 32) {
            const float2 v = s[x];
            rerr |= (__float_as_uint(v.x) & 0x7f800000u) == 0x7f800000u;
            d[x] = join_f64(v.x, v.y, a.bias);
        }
    }
    if (rerr) atomicOr(a.err, kDevErrRange);
}

// CTAs of 8 warps, one row per warp at a time: at most 8 resident CTAs on
// each SM.
unsigned conv_blocks(int64_t rows) {
    const int64_t need = (rows + kConvThreads / 32 - 1) / (kConvThreads / 32),
                  cap = static_cast<int64_t>(device_sm_count()) * 8;
    return static_cast<unsigned>(need < 1 ? 1 : need < cap ? need : cap);
}

}  // namespace

cudaError_t launch_to_pairs(const GridView &src, const GridView &dst, const int64_t lb[3], const int64_t ub[3],
                            bool halo_only, int shift, unsigned *err, cudaStream_t st) {
    PairConv a{src.data, dst.data, src.s[0], src.s[1], dst.s[0], dst.s[1], src.n[0], src.n[1], src.n[2],
               lb[0], lb[1], lb[2], ub[0], ub[1], ub[2], halo_only ? 1 : 0, pair_bias(shift), err};
    if (src.n[0] * src.n[1] <= 0 || src.n[2] <= 0) return cudaSuccess;
    k_to_pairs<<<conv_blocks(src.n[0] * src.n[1]), kConvThreads, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_from_pairs(const GridView &src, const GridView &dst, const int64_t lb[3], const int64_t ub[3],
                              int shift, unsigned *err, cudaStream_t st) {
    PairConv a{src.data, dst.data, src.s[0], src.s[1], dst.s[0], dst.s[1], src.n[0], src.n[1], src.n[2],
               lb[0], lb[1], lb[2], ub[0], ub[1], ub[2], 0, pair_bias(shift), err};
    const int64_t rows = (ub[0] - lb[0]) * (ub[1] - lb[1]);
    if (rows <= 0 || ub[2] <= lb[2]) return cudaSuccess;
    k_from_pairs<<<conv_blocks(rows), kConvThreads, 0, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace uhs
