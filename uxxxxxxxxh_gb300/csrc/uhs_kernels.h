// Internal interface between the host runtime (uhs_runtime.cpp) and the sweep
// kernels (*.cu).  Not part of the C ABI.
#pragma once
#include <algorithm>
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/uhs.h"

namespace uhs {

// One grid as the kernels see it: element pointer of (0,0,0), element strides.
struct GridView {
    void *data;
    int64_t n[3];   // sizes, slowest first
    int64_t s[3];   // strides in elements (s[2] == 1)
};

// A stencil program reduced to what a sweep needs.
struct SweepSpec {
    int rank;
    int dtype;
    int64_t lb[3], ub[3];
    int nterms;
    int32_t dz[UHS_MAX_TERMS], dy[UHS_MAX_TERMS], dx[UHS_MAX_TERMS];
    double coef[UHS_MAX_TERMS];
    int rz, ry, rx;        // max |offset| per axis
    int shape;             // kShapeGeneric / kShapeStar / kShapeBox
    int radius;            // for star/box
};

enum { kShapeGeneric = 0, kShapeStar = 1, kShapeBox = 2 };

struct LaunchCfg {
    int kernel;      // UHS_KERNEL_*
    int arith;       // UHS_ARITH_*
    int tile_x, tile_y, tile_z;
    int k_temporal;
    int use_tma;
};

// Device-side error word written by kernels that detect a problem (range
// overflow in float-pair arithmetic, a bounded wait that ran out).
enum : unsigned { kDevErrRange = 1u, kDevErrTimeout = 2u };
// A status word is kStatusWords unsigned words in device memory:
//   0 kernel status flags; 1 range-scan largest exponent / halo-check count;
//   2-7 where the first bounded wait gave up (set, block x, block z, plane,
//   ring slot, phase); 8 range-scan smallest exponent of a nonzero value.
constexpr int kStatusWords = 16;
unsigned *stream_error_word(int device, cudaStream_t stream);

// Generic smem plane-ring sweep: any term list, expression order.
cudaError_t launch_generic(const SweepSpec &sp, const LaunchCfg &cfg, const GridView &in,
                           const GridView &out, cudaStream_t st);

// FP64 error reduction (error_norms.cu).  The domain is cut into work units
// of kErrRowsPerUnit rows (and, when that gives too few units to balance the
// GPU -- few long rows, as in 2D grids -- into x-chunks of at least 256
// elements); at most kErrBlocks CTAs take the units round-robin, each writing
// 4 doubles of partials into scratch; the result (4 doubles) follows the
// partials.  Scratch holds 4 * (nblocks + 1) doubles.  The split depends only
// on the domain's shape, never on the device, so the FP64 sums are added in
// the same order and the results are the same on every GPU: kErrBlocks is a
// fixed count (608, four resident 256-thread CTAs on each of a GB300's 152
// SMs), not the queried SM count.
constexpr int kErrRowsPerUnit = 16;
constexpr int64_t kErrBlocks = 608;
inline void err_split(int64_t rows, int64_t width, int64_t *units, int *xchunks, int *nblocks) {
    const int64_t ru = (rows + kErrRowsPerUnit - 1) / kErrRowsPerUnit, want = 8 * kErrBlocks;
    int64_t xc = 1;
    if (ru > 0 && ru < want) {
        const int64_t a = (want + ru - 1) / ru, b = (width + 255) / 256;
        xc = a < b ? a : b;
        if (xc < 1) xc = 1;
    }
    *units = ru * xc;
    *xchunks = static_cast<int>(xc);
    *nblocks = static_cast<int>(*units < kErrBlocks ? *units : kErrBlocks);
}
struct ErrNormsCall {
    int dtype;   // element type of x
    GridView x;  // grid under test
    GridView r;  // FP64 reference grid
    int64_t lb[3], ub[3];
    int nblocks;    // CTAs = partial slots (err_split)
    int xchunks;    // x-chunks per row unit
    int64_t units;  // row units x xchunks
    double *scratch;
    cudaStream_t stream;
};
cudaError_t launch_error_norms(const ErrNormsCall &c);

// Pair-resident runs (pairs.cu): an FP64 grid's values split into a
// contiguous float-pair grid (the whole grid, or only the cells outside the
// domain [lb, ub)), and the domain of a float-pair grid joined back.
// The pairs hold the values times 2^shift (the run's scale, df32.cuh).
cudaError_t launch_to_pairs(const GridView &src, const GridView &dst, const int64_t lb[3], const int64_t ub[3],
                            bool halo_only, int shift, unsigned *err, cudaStream_t st);
// The join sets kDevErrRange in *err when a pair holds Inf or NaN (a value
// that outgrew the float range during the sweeps).
cudaError_t launch_from_pairs(const GridView &src, const GridView &dst, const int64_t lb[3], const int64_t ub[3],
                              int shift, unsigned *err, cudaStream_t st);

// Exponent range of n_words doubles: the largest biased exponent field into
// *max_out (atomicMax; must start at 0) and the smallest biased exponent field
// of a nonzero value (zeros of either sign are skipped; a subnormal counts as
// exponent 0) into *min_out (atomicMin; must start at 0xffffffff).
cudaError_t launch_exponent_range(const void *data, int64_t n_words, unsigned *max_out, unsigned *min_out, int sms,
                                  cudaStream_t st);

// FP32 3D box stencils of radius 2 and 3 on the tensor cores (box_mma.cu).
// Coefficients in box slot order ((dz+R)*D + (dy+R))*D + (dx+R), D = 2R+1.
// xtile: 16 or 32 output columns per CTA tile (32 for R = 2 only).
struct MmaCall {
    GridView in, out;
    int64_t lb[3], ub[3];
    int R;
    int xtile;
    int a_tmem;  // 1: A operand staged in tensor memory (16-column tiles only)
    const double *coef;
    unsigned *err;
    cudaStream_t stream;
    int *occ_out;  // when set: report CTAs per SM and launch nothing
};
cudaError_t launch_box_mma(const MmaCall &c);

// Failure-reporting probe (diag.cu): a bounded wait that cannot complete.
cudaError_t launch_wait_probe(unsigned *err, long long cycles, cudaStream_t st);
// FP64 pipe rate (diag.cu): DFMA per second over all SMs, timed on st.
cudaError_t probe_dfma_rate(double *per_second, cudaStream_t st);

// Library-owned device allocations go through dev_alloc, which honours the
// diagnostic cap set by uhs_set_alloc_cap (a request above the cap fails as
// an out-of-memory would).
cudaError_t dev_alloc(void **p, size_t bytes);

// Launch counter shared by every launcher.
void count_launch(int n = 1);

// Streaming multiprocessors of the current device (queried once per device;
// 1 if the query fails, which only shrinks the grids the launchers size).
int device_sm_count();

}  // namespace uhs
