// Host-visible description of a streaming-kernel launch (stream_kernel.cuh
// holds the kernels, stream_launch.cuh the argument packing).  Shared by the
// runtime, which plans launches, and the per-storage translation units.
#pragma once
#include <cuda.h>

#include "uhs_kernels.h"

namespace uhs {

enum { kStar3 = 0, kBox3 = 1, kStar2 = 2, kBox2 = 3, kSep3 = 4, kSep2 = 5 };
// kSep3 / kSep2: box stencils whose coefficients factor as a (x) b (x) c
// (rank 1), applied as three (two) 1D passes; coefficients [a | b | c].
// Rank-2 shapes (streamed along y in the kernel frame):
constexpr bool is_rank2_shape(int shape) { return shape == kStar2 || shape == kBox2 || shape == kSep2; }
enum { kStF64 = 0, kStF32 = 1, kStF32x2 = 2 };
enum { kArNative = 0, kArDf32 = 1 };
enum { kLdCpAsync = 0, kLdTma = 1 };
// Term capacity of a batched grid's arguments (the 7x7x7 box).
constexpr int kBatchNT = 343;

constexpr int ct_round_up(int v, int m) { return (v + m - 1) / m * m; }

template <int NT>
struct StreamArgs {
    CUtensorMap tmap;  // TMA loader only
    const void *in;
    void *out;
    int64_t in_s0, in_s1, out_s0, out_s1;
    int64_t n0, n1, n2;
    int64_t lb0, lb1, lb2, ub0, ub1, ub2;
    int zchunk;
    int shift;       // TMA box starts this many elements left of x0 - R (16-byte granule)
    int pair_loads;  // cp.async of 4-byte elements in 8-byte pairs (origin and pitches even)
    int pair_shift;  // FP64 grids in float pairs: the pairs hold x * 2^pair_shift (df32.cuh)
    // two points per thread along x: the tiles start xoff (0 or 1) columns
    // left of lb2, so each thread's pair of output cells starts on an even
    // element of the output row (vector stores); cells left of lb2 are not
    // written
    int xoff;
    unsigned *err;
    double cd[NT];
    float2 chl[NT];  // float rounding of each coefficient and its rounding error (hi, lo)
    // Float grids: sum of the coefficients' float rounding errors (c - ch),
    // per pass (sep: z, y, x; otherwise [0]); applied once per point to the
    // centre value so the sweep keeps the FP64 coefficients' sum.
    float cl_sum[3];
    // |ch| of each coefficient: the float-pair bounded sums' bound (df32.cuh
    // bound_add) reads it as an operand instead of holding |ch| in registers
    float cab[NT];
};

// Coefficients in the three forms the kernels use, plus the per-pass sums of
// the float rounding errors (separable shapes: passes z | y | x, D each).
inline void fill_coefs(double *cd, float2 *chl, float *cl_sum, const double *coef, int nt, int shape, int R) {
    const int D = 2 * R + 1;
    double sums[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < nt; ++k) {
        const double v = coef[k];
        const float h = static_cast<float>(v);
        cd[k] = v;
        chl[k] = make_float2(h, static_cast<float>(v - static_cast<double>(h)));
        const int pass = (shape == kSep3 || shape == kSep2) ? k / D : 0;
        sums[pass < 3 ? pass : 2] += v - static_cast<double>(h);
    }
    for (int i = 0; i < 3; ++i) cl_sum[i] = static_cast<float>(sums[i]);
}
inline void fill_coef_abs(float *cab, const float2 *chl, int nt) {
    for (int k = 0; k < nt; ++k) cab[k] = chl[k].x < 0.0f ? -chl[k].x : chl[k].x;
}

// Everything one streaming launch needs (filled by the runtime).
struct StreamCall {
    int shape, R, st, ar, ld, tile, zchunk;
    const double *coef;  // NT coefficients in coef_slot order
    GridView in, out;    // views in the kernel's (z, y, x) frame
    int64_t lb[3], ub[3];
    const CUtensorMap *tmap;
    int shift;
    int pair_loads;
    int pair_shift;  // FP64 grids in float pairs: power-of-two scale of the pairs (0: none)
    int xshuffle;    // rank-2 stars: x-neighbours by warp shuffles (UHS_FLAG_XSHUFFLE)
    int xoff;        // two points per thread along x: tile origin lb[2] - xoff (StreamArgs::xoff)
    unsigned *err;
    cudaStream_t stream;
    int *occ_out;  // when set: report CTAs per SM of the variant instead of launching
};

// Tile variants: rank-3 (BX, TYT, VY) and rank-2 (BX).
//   rank 3: 0 = 32 x 32 (VY 4), 1 = 32 x 16 (VY 4), 2 = 64 x 8 (VY 2), 3 = 32 x 16 (VY 2)
//           (box stencils of radius 2 and 3 always use 32 x 16, VY 2)
//   rank 2: 0 = 128, 1 = 64, 2 = 256 (cp.async only: a TMA box is <= 256 wide);
//           stars also 3 = 64 x 2 points along x, 4 = 128 x 2 (cp.async only)
struct TileShape {
    int bx, tyt, vy, vx;
};
inline TileShape tile_shape(bool is2d, int tile) {
    if (is2d) {
        switch (tile) {
            case 1: return TileShape{64, 1, 1, 1};
            case 2: return TileShape{256, 1, 1, 1};
            case 3: return TileShape{64, 1, 1, 2};
            case 4: return TileShape{128, 1, 1, 2};
            default: return TileShape{128, 1, 1, 1};
        }
    }
    switch (tile) {
        case 4: return TileShape{32, 4, 8, 1};
        case 1: return TileShape{32, 4, 4, 1};
        case 2: return TileShape{64, 4, 2, 1};
        case 3: return TileShape{32, 8, 2, 1};
        default: return TileShape{32, 8, 4, 1};
    }
}

// Per translation unit entry points (stream_<storage>_<rank>.cu).
cudaError_t launch_stream_f64n_3d(const StreamCall &c);
cudaError_t launch_stream_f64df_3d(const StreamCall &c);
cudaError_t launch_stream_f32_3d(const StreamCall &c);
cudaError_t launch_stream_f32x2_3d(const StreamCall &c);
cudaError_t launch_stream_f64n_2d(const StreamCall &c);
cudaError_t launch_stream_f64df_2d(const StreamCall &c);
cudaError_t launch_stream_f32_2d(const StreamCall &c);
cudaError_t launch_stream_f32x2_2d(const StreamCall &c);

// Geometry of a variant as the kernel template computes it (host mirror).
inline void stream_box(const StreamCall &c, int eb, int *W, int *H) {
    const bool is2d = is_rank2_shape(c.shape);
    const TileShape t = tile_shape(is2d, c.tile);
    const int q = 16 / eb;
    const bool big_box = (c.shape == kBox3 && c.R >= 2);
    const int bx = big_box ? 32 : t.bx * t.vx, by = big_box ? 16 : t.tyt * t.vy;
    *W = ct_round_up(bx + 2 * c.R + (c.ld == kLdTma ? q - 1 : 0), q);
    *H = by + (is2d ? 0 : 2 * c.R);
}
inline void stream_tile_xy(const StreamCall &c, int *bx, int *by) {
    const bool is2d = is_rank2_shape(c.shape);
    const TileShape t = tile_shape(is2d, c.tile);
    const bool big_box = (c.shape == kBox3 && c.R >= 2);
    *bx = big_box ? 32 : t.bx * t.vx;
    *by = big_box ? 16 : t.tyt * t.vy;
}

}  // namespace uhs

namespace uhs {

// ---- batched persistent launches (stream_batch.cu) ----------------------
// Every grid of a batch carries its arguments at the largest term count
// (343, the 7x7x7 box), once per ping-pong direction, and the index of its
// variant inside the persistent kernel's variant pack.
// A distinct type (not an alias of StreamArgs<343>): the kernels read a
// BatchArgs from shared memory, a StreamArgs from the parameter bank, and
// choose their coefficient loads by this type.
struct BatchArgs : StreamArgs<kBatchNT> {};
struct alignas(64) BatchGrid {
    BatchArgs dir[2];  // [0]: a -> b, [1]: b -> a
    int kind;
};
// Packs: 0 = float-pair FP64 and native FP32 variants of all 12 shapes (one
// launch per step covers a mixed FP32/FP64 batch); 1 = native FP64.
enum { kPackMain = 0, kPackF64Native = 1, kNumPacks = 2 };
struct BatchPackInfo {
    int smem, threads, occ;
};
// Variant index of (shape, R, storage, arithmetic) in a pack, or -1.
int batch_kind(int pack, int shape, int R, int st, int ar);
// Tile and z-chunk every batch item of that variant uses.
void batch_tile(int shape, int R, int st, int *bx, int *by, int *zchunk);
cudaError_t batch_prepare(int pack, BatchPackInfo *info);
// CTAs take items in list order through *counter (zero before the launch):
// a list ordered by decreasing cost then ends with the cheapest items.
cudaError_t batch_launch(int pack, const BatchGrid *grids, const int4 *items, int n_items, int dir, int ctas,
                         int *counter, cudaStream_t st);
// Temporal fusion (stream_fused.cu): K in {2, 4} steps of the 3D 7-point
// star per pass; and the halo comparison that gates it.
cudaError_t launch_fused(const StreamCall &c, int K);
cudaError_t launch_fused_2d(const StreamCall &c, int K);  // stream_fused_2d.cu
cudaError_t launch_halo_diff(const GridView &a, const GridView &b, int eb, const int64_t lb[3], const int64_t ub[3],
                             unsigned *count, int sms, cudaStream_t st);

// Host-side packing of one direction's arguments (coefficients in slot order).
void batch_fill_args(BatchArgs *a, const StreamCall &c, int nt);

}  // namespace uhs
