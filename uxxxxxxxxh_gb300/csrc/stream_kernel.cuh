// 2.5D streaming sweep kernels for star and box stencils of radius 1..3.
//
// One CTA owns a BX x BY tile of the (y, x) plane and walks a chunk of planes
// along the slowest axis z (for a rank-2 grid the rows play the part of the
// planes and the tile is one row segment).  Each input plane of the tile,
// halo included, is fetched from HBM once per CTA into a ring of shared-
// memory slots, either by one TMA tensor copy per plane (completion on an
// mbarrier) or by cp.async from every thread; loads run PD planes ahead of
// the plane being computed.  For star stencils the z-neighbours of each
// thread's points live in a register queue (the 2.5D register-streaming
// scheme: a plane's own column is read from shared memory once and then
// shifts through registers), so shared memory holds only the planes whose
// in-plane neighbours are still needed; box stencils keep the 2R+1 planes a
// point touches.  Each thread computes VY points stacked along y and reuses
// the column it reads from shared memory across them.
//
// Arithmetic policies:
//   native  double grids in DFMA, float grids in FFMA;
//   df32    double grids split once per element into float pairs (integer
//           bit operations, no FP64 instruction), swept with error-free
//           float-pair products and sums, joined back to double on store;
//           float-pair grids (UHS_F32X2, interleaved {hi, lo}) use the same
//           arithmetic without the split and join.
// The reference emits one generic NVVM kernel per stencil for this step
// (examples/2d5pt_star/2d5pt_gpu.mlir:10-102): scalar loads into a shared
// input tile, a barrier, per-thread sums into a shared output tile, a second
// barrier and a write-back.
#pragma once
#include <cuda.h>

#include <type_traits>

#include "df32.cuh"
#include "stream_call.h"

namespace uhs {


template <int SHAPE, int R>
struct ShapeInfo {
    static constexpr bool is2d = is_rank2_shape(SHAPE);
    static constexpr bool star = (SHAPE == kStar3 || SHAPE == kStar2);
    static constexpr bool sep = (SHAPE == kSep3 || SHAPE == kSep2);
    static constexpr int RY = is2d ? 0 : R;
    static constexpr int D = 2 * R + 1;
    static constexpr int NT = sep ? (is2d ? 2 * D : 3 * D)
                                  : star ? (is2d ? 4 * R + 1 : 6 * R + 1) : (is2d ? D * D : D * D * D);
};

// Coefficient slot of each offset (the host writes the descriptor's
// coefficients in this order).
//   star3: z(-1,+1,-2,+2..), y(..), x(..), centre      star2: z(..), x(..), centre
//   box3 : ((dz+R)*D + dy+R)*D + dx+R                  box2 : (dz+R)*D + dx+R
template <int SHAPE, int R>
__host__ __device__ constexpr int coef_slot(int dz, int dy, int dx) {
    constexpr int D = 2 * R + 1;
    if (SHAPE == kBox3) return ((dz + R) * D + (dy + R)) * D + (dx + R);
    if (SHAPE == kBox2) return (dz + R) * D + (dx + R);
    const int axes = SHAPE == kStar3 ? 3 : 2;
    if (dz == 0 && dy == 0 && dx == 0) return axes * 2 * R;
    int axis, d;
    if (dz != 0) {
        axis = 0;
        d = dz;
    } else if (dy != 0) {
        axis = 1;
        d = dy;
    } else {
        axis = SHAPE == kStar3 ? 2 : 1;
        d = dx;
    }
    const int ad = d < 0 ? -d : d;
    return axis * 2 * R + (ad - 1) * 2 + (d > 0 ? 1 : 0);
}

// XS: rank-2 stars take their x-neighbours by warp shuffles (UHS_FLAG_XSHUFFLE).
// VX: points per thread along x (rank-2 stars: 1 or 2); a CTA tile is
// CX = BX * VX columns wide.
template <int SHAPE_, int R_, int ST_, int AR_, int LD_, int BX_, int TYT_, int VY_, int PD_, int XS_ = 0,
          int VX_ = 1>
struct StreamCfg {
    static constexpr int SHAPE = SHAPE_, R = R_, ST = ST_, AR = AR_, LD = LD_, BX = BX_, TYT = TYT_, VY = VY_,
                         PD = PD_, XS = XS_, VX = VX_;
    static constexpr int CX = BX * VX;
    using SI = ShapeInfo<SHAPE, R>;
    using TS = std::conditional_t<ST == kStF64, double, std::conditional_t<ST == kStF32, float, float2>>;
    static constexpr bool CONVERT = (ST == kStF64 && AR == kArDf32);
    using TC = std::conditional_t<CONVERT, float2, TS>;
    static constexpr int EB = sizeof(TS);
    static constexpr int Q = 16 / EB;  // TMA x-coordinate granule, elements
    static constexpr int RY = SI::RY;
    static constexpr int BY = TYT * VY;
    static constexpr int W = ct_round_up(CX + 2 * R + (LD == kLdTma ? Q - 1 : 0), Q);
    static constexpr int H = BY + 2 * RY;
    static constexpr int NCMP = SI::sep ? 1 : SI::star ? R + 1 : 2 * R + 1;
    static constexpr int NSTG = CONVERT ? PD + 1 : NCMP + PD;
    static constexpr int STG_SLOT = ct_round_up(W * H * EB, 128);
    static constexpr int CMP_SLOT = ct_round_up(W * H * (int)sizeof(TC), 128);
    static constexpr int SMEM = NSTG * STG_SLOT + (CONVERT ? NCMP * CMP_SLOT : 0) + NSTG * 8;
    static constexpr int THREADS = BX * TYT;
    static constexpr int NT = SI::NT;
    // Float-pair sweeps sum a thread's points two at a time in packed FP32
    // instructions in standalone launches: rows 2p, 2p+1 in 3D, the two
    // columns of a rank-2 thread with VX = 2 (dfs2_*_s for stars and
    // separable passes, df2_*_s for term-by-term boxes, df32.cuh).  GB300 at
    // 512^3 (256^3 for radius 2-3 boxes), GStencil/s per sweep, scalar ->
    // packed (with TwoSum sums; bounded sums came after): stars on float-pair grids r1/r2/r3 330/184/129
    // -> 341/186/134 (best tiles), on FP64 grids 169/114/86 -> 191/130/97;
    // separable boxes FP64 141/92/63 -> 163/102/68; radius-3 boxes 5.5/6.0 ->
    // 7.5/7.2.  Term-by-term boxes of radius 1 on float-pair grids (100 ->
    // 96) and of radius 2 (21.2 -> 20.4, FP64 19.3 -> 19.0) keep the scalar
    // sums.
    static constexpr bool PACKED = AR == kArDf32 && (SI::is2d ? VX == 2 : VY % 2 == 0) &&
                                   !(SHAPE == kBox3 && (R == 2 || (R == 1 && ST == kStF32x2)));
    static_assert(LD != kLdTma || W <= 256, "TMA boxes are at most 256 elements wide");
    static_assert(!SI::is2d || (TYT == 1 && VY == 1), "rank-2 tiles are one row");
    static_assert(!XS || (SI::is2d && SI::star), "lane shuffles: rank-2 stars");
    static_assert(VX == 1 || (VX == 2 && SI::is2d && SI::star && !XS), "two points along x: rank-2 stars");
    // points per thread, and their spacing in shared memory: rows along y
    // (rank 3), or adjacent columns (rank 2 with VX = 2)
    static constexpr int NPT = VX == 2 ? 2 : VY;
};


// ---- asynchronous copy primitives --------------------------------------
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem, bool valid) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    const int n = valid ? BYTES : 0;
    if constexpr (BYTES == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(bar));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(a), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(bar));
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(a), "r"(bytes) : "memory");
}
// Bounded wait for phase `parity` of an mbarrier: false when about one second
// of SM clock (2^31 cycles) passed without the phase completing.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    const unsigned a = static_cast<unsigned>(__cvta_generic_to_shared(bar));
    const long long t0 = clock64();
    for (;;) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > (1ll << 31)) return false;
    }
}
__device__ __forceinline__ void tma_load_3d(void *smem, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    const unsigned b = static_cast<unsigned>(__cvta_generic_to_shared(bar));
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];\n" ::"r"(s),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(b)
        : "memory");
}

// Lane shuffles of a value of the compute type (float, double or a float pair).
template <class T>
__device__ __forceinline__ T shfl_up_tc(T v, int d) {
    if constexpr (std::is_same_v<T, float2>)
        return make_float2(__shfl_up_sync(0xffffffffu, v.x, d), __shfl_up_sync(0xffffffffu, v.y, d));
    else
        return __shfl_up_sync(0xffffffffu, v, d);
}
template <class T>
__device__ __forceinline__ T shfl_down_tc(T v, int d) {
    if constexpr (std::is_same_v<T, float2>)
        return make_float2(__shfl_down_sync(0xffffffffu, v.x, d), __shfl_down_sync(0xffffffffu, v.y, d));
    else
        return __shfl_down_sync(0xffffffffu, v, d);
}

// ---- arithmetic policies -----------------------------------------------
// Coefficient reads.  Kernel parameters (StreamArgs) sit in the constant
// bank and feed the FMA directly.  The batched kernel keeps each item's
// arguments in shared memory (BatchArgs) and reads every coefficient where
// it is used, through a volatile load the compiler cannot hoist out of the
// plane loop: hoisted, even a 13-term star's float pairs push the batched
// kernel's item functions (80 registers at 3 CTAs of 256 threads) into
// spilling, and 343 of them would exhaust the register file.
template <class C, class Args>
__device__ __forceinline__ double coef_d(const Args &a, int k) {
    if constexpr (std::is_same_v<Args, BatchArgs>) {
        double v;
        asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"((unsigned)__cvta_generic_to_shared(&a.cd[k])));
        return v;
    } else {
        return a.cd[k];
    }
}
template <class C, class Args>
__device__ __forceinline__ float coef_f(const Args &a, const float *p) {
    if constexpr (std::is_same_v<Args, BatchArgs>) {
        float v;
        asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"((unsigned)__cvta_generic_to_shared(p)));
        return v;
    } else {
        return *p;
    }
}

// The (hi, lo) float pair of coefficient k in one 8-byte read.
template <class C, class Args>
__device__ __forceinline__ float2 coef_f2(const Args &a, int k) {
    if constexpr (std::is_same_v<Args, BatchArgs>) {
        float2 v;
        asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];"
                     : "=f"(v.x), "=f"(v.y)
                     : "r"((unsigned)__cvta_generic_to_shared(&a.chl[k])));
        return v;
    } else {
        return a.chl[k];
    }
}

// |ch| of coefficient k (the bounded sums' bound)
template <class C, class Args>
__device__ __forceinline__ float coef_abs(const Args &a, int k) {
    if constexpr (std::is_same_v<Args, BatchArgs>) {
        float v;
        asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"((unsigned)__cvta_generic_to_shared(&a.cab[k])));
        return v;
    } else {
        return a.cab[k];
    }
}

template <class C, int AR = C::AR>
struct Arith;

// Native arithmetic: one DFMA / FFMA per term.  Float grids use the float
// rounding ch of each coefficient; the rounding errors cl = c - ch would sum,
// for a normalised stencil, to a delta that scales the field by (1 + delta)
// every step -- an error growing linearly with T.  centre() adds
// (sum of cl) * centre value once per point, which restores the FP64
// coefficients' sum exactly (and their action exactly on locally constant
// fields) for one FFMA.
template <class C>
struct Arith<C, kArNative> {
    using TS = typename C::TS;
    static constexpr bool F32 = std::is_same_v<TS, float>;
    using Acc = TS;
    template <class Args>
    __device__ static __forceinline__ TS coef(const Args &a, int k) {
        if constexpr (!F32) return coef_d<C>(a, k);
        else return coef_f<C>(a, &a.chl[k].x);
    }
    template <class Args>
    __device__ static __forceinline__ void first(Acc &acc, const Args &a, int k, TS v) {
        acc = coef(a, k) * v;
    }
    template <class Args>
    __device__ static __forceinline__ void add(Acc &acc, const Args &a, int k, TS v) {
        acc = fma(coef(a, k), v, acc);
    }
    template <class Args>
    __device__ static __forceinline__ void centre(Acc &acc, const Args &a, int pass, TS v) {
        if constexpr (F32) acc = fmaf(a.cl_sum[pass], v, acc);
    }
    __device__ static __forceinline__ void store(TS *p, const Acc &acc, unsigned &, int) { *p = acc; }
    // bounded sums (float pairs only): the plain sum here
    static constexpr bool kBounded = false;
    template <class Args>
    __device__ static __forceinline__ void bfirst(Acc &acc, float, const Args &a, int k, TS v) {
        first(acc, a, k, v);
    }
    template <class Args>
    __device__ static __forceinline__ void badd(Acc &acc, float, const Args &a, int k, TS v) {
        add(acc, a, k, v);
    }
    // two adjacent points, p aligned to 2 * sizeof(TS)
    static constexpr bool kVecStore = true;
    __device__ static __forceinline__ void store2(TS *p, const Acc &a0, const Acc &a1, unsigned &, int) {
        if constexpr (F32) *reinterpret_cast<float2 *>(p) = make_float2(a0, a1);
        else *reinterpret_cast<double2 *>(p) = make_double2(a0, a1);
    }
    __device__ static __forceinline__ TS level(const Acc &acc) { return acc; }
};

template <class C>
struct Arith<C, kArDf32> {
    using Acc = df;
    template <class Args>
    __device__ static __forceinline__ void first(Acc &acc, const Args &a, int k, float2 v) {
        const float2 c = coef_f2<C>(a, k);
        df_mul(acc, c.x, c.y, v);
    }
    template <class Args>
    __device__ static __forceinline__ void add(Acc &acc, const Args &a, int k, float2 v) {
        const float2 c = coef_f2<C>(a, k);
        df_fma(acc, c.x, c.y, v);
    }
    // Star and separable sums: bounded sums (dfs_mul / dfs_fma in df32.cuh),
    // sg = the point's sigma_of.  Term-by-term boxes keep first / add.
    static constexpr bool kBounded = true;
    template <class Args>
    __device__ static __forceinline__ void bfirst(Acc &acc, float sg, const Args &a, int k, float2 v) {
        const float2 c = coef_f2<C>(a, k);
        dfs_mul(acc, sg, c.x, c.y, v);
    }
    template <class Args>
    __device__ static __forceinline__ void badd(Acc &acc, float sg, const Args &a, int k, float2 v) {
        const float2 c = coef_f2<C>(a, k);
        dfs_fma(acc, sg, c.x, c.y, v);
    }
    // FP64 grids: joined back with the run's exponent bias (the pairs hold
    // x * 2^pair_shift).  A sum that outgrew the float range (hi Inf or NaN)
    // would join to a finite double; it sets the range flag instead of
    // passing unnoticed.
    __device__ static __forceinline__ void store(typename C::TS *p, const Acc &acc, unsigned &range_err, int bias) {
        if constexpr (C::ST == kStF64) {
            range_err |= (__float_as_uint(acc.h) & 0x7f800000u) == 0x7f800000u;
            *p = join_f64(acc.h, acc.l, bias);
        } else {
            *p = renorm(acc);
        }
    }
    static constexpr bool kVecStore = true;
    __device__ static __forceinline__ void store2(typename C::TS *p, const Acc &a0, const Acc &a1, unsigned &range_err,
                                                  int bias) {
        if constexpr (C::ST == kStF64) {
            range_err |= (__float_as_uint(a0.h) & 0x7f800000u) == 0x7f800000u;
            range_err |= (__float_as_uint(a1.h) & 0x7f800000u) == 0x7f800000u;
            *reinterpret_cast<double2 *>(p) = make_double2(join_f64(a0.h, a0.l, bias), join_f64(a1.h, a1.l, bias));
        } else {
            const float2 r0 = renorm(a0), r1 = renorm(a1);
            *reinterpret_cast<float4 *>(p) = make_float4(r0.x, r0.y, r1.x, r1.y);
        }
    }
    __device__ static __forceinline__ float2 level(const Acc &acc) { return renorm(acc); }
    template <class Args>
    __device__ static __forceinline__ void centre(Acc &, const Args &, int, float2) {}
};

// Bound B of a star point's bounded sum (df32.cuh): sum |ch_k| |xh_k| over
// its inputs in the sum's order -- centre, +-d along z, y (rank 3), x.
// zq: the point's z-queue (centre at [R]); cell: the point's own cell in
// the staged centre plane (y-neighbours W apart, x-neighbours adjacent).
// The sums that follow read the same cells; the code generator keeps the
// loaded values in registers between the two (a warp barrier between them
// forces reloads and cuts the 3D 13-point float-pair sweep from 118 to 72
// registers per thread, but measured 4 % slower: 208 against 217 GStencil/s
// per sweep at 512^3).
template <class C, class Args, class TC>
__device__ __forceinline__ float star_bound(const Args &a, const TC *zq, const TC *cell) {
    constexpr int R = C::R, W = C::W;
    float b = bound_add(0.0f, coef_abs<C>(a, coef_slot<C::SHAPE, R>(0, 0, 0)), zq[R]);
#pragma unroll
    for (int d = 1; d <= R; ++d) {
        b = bound_add(b, coef_abs<C>(a, coef_slot<C::SHAPE, R>(-d, 0, 0)), zq[R - d]);
        b = bound_add(b, coef_abs<C>(a, coef_slot<C::SHAPE, R>(d, 0, 0)), zq[R + d]);
    }
    if constexpr (!C::SI::is2d) {
#pragma unroll
        for (int d = 1; d <= R; ++d) {
            b = bound_add(b, coef_abs<C>(a, coef_slot<C::SHAPE, R>(0, -d, 0)), cell[-d * W]);
            b = bound_add(b, coef_abs<C>(a, coef_slot<C::SHAPE, R>(0, d, 0)), cell[d * W]);
        }
    }
#pragma unroll
    for (int d = 1; d <= R; ++d) {
        b = bound_add(b, coef_abs<C>(a, coef_slot<C::SHAPE, R>(0, 0, -d)), cell[-d]);
        b = bound_add(b, coef_abs<C>(a, coef_slot<C::SHAPE, R>(0, 0, d)), cell[d]);
    }
    return b;
}

// ---- the kernel ---------------------------------------------------------
// One work item: the (bx, by) tile of the (y, x) plane over z-chunk bz.
// Returns false when a bounded wait ran out (the status word is set).
// Leaves no copy in flight and ends with a barrier, so a persistent caller can
// start its next item on the same shared memory right away.
template <class C, class Args>
__device__ __forceinline__ bool stream_item(const Args &a, int bxi, int byi, int bzi, unsigned char *smem) {
    using TS = typename C::TS;
    using TC = typename C::TC;
    using A = Arith<C>;
    using Acc = typename A::Acc;
    constexpr int R = C::R, RY = C::RY, BX = C::BX, TYT = C::TYT, VY = C::VY, W = C::W, H = C::H;
    constexpr int NSTG = C::NSTG, NCMP = C::NCMP, PD = C::PD;
    constexpr int STG_ELEMS = C::STG_SLOT / C::EB, CMP_ELEMS = C::CMP_SLOT / (int)sizeof(TC);
    constexpr bool STAR = C::SI::star, IS2D = C::SI::is2d;
    constexpr int NLOAD_ROWS = (H + TYT - 1) / TYT;  // cp.async: rows per thread

    // Thread coordinates from the linear index, so a caller launched with
    // another 256-thread block shape (the batched kernel) maps the same way.
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int tx = tid % BX, ty = tid / BX;
    constexpr int VX = C::VX, CX = C::CX, NPT = C::NPT;
    const int64_t x0 = a.lb2 - (VX == 2 ? a.xoff : 0) + static_cast<int64_t>(bxi) * CX;
    const int64_t y0 = a.lb1 + static_cast<int64_t>(byi) * C::BY;
    const int64_t zs = a.lb0 + static_cast<int64_t>(bzi) * a.zchunk;
    const int64_t ze = min(zs + static_cast<int64_t>(a.zchunk), a.ub0);
    const int64_t gx0 = x0 - R - a.shift, gy0 = y0 - RY;
    const int64_t qbeg = zs - R;
    const int nq = static_cast<int>(ze + R - qbeg);
    TS *const stg_base = reinterpret_cast<TS *>(smem);
    TC *const cmp_base = C::CONVERT ? reinterpret_cast<TC *>(smem + NSTG * C::STG_SLOT) : reinterpret_cast<TC *>(smem);
    uint64_t *const mbar = reinterpret_cast<uint64_t *>(smem + NSTG * C::STG_SLOT + (C::CONVERT ? NCMP * C::CMP_SLOT : 0));
    constexpr int CMP_STRIDE = C::CONVERT ? CMP_ELEMS : STG_ELEMS;
    constexpr int NRING = C::CONVERT ? NCMP : NSTG;  // ring the compute reads

    // cp.async: per-thread row offsets inside a plane (32-bit: a plane holds
    // fewer than 2^31 elements, which the host checks) and validity.
    // 8-byte elements recompute each copy's source per plane (fewest live
    // registers: these variants run at the compiler's register choice).
    // 4-byte elements (FP32, held to 64 or 128 registers) hoist it: each
    // copy's in-plane offset (0 when zero-filled) and a validity bit are
    // computed once per z-chunk and only the plane pointer moves -- 2-4 %
    // faster on GB300.
    constexpr bool HOIST = C::EB == 4;
    int row_off[NLOAD_ROWS];  // 8-byte elements
    bool row_ok[NLOAD_ROWS];
    int off_a[NLOAD_ROWS], off_b[NLOAD_ROWS];  // 4-byte elements
    unsigned ok_a = 0u, ok_b = 0u;
    const bool pairs = C::EB == 4 && a.pair_loads;  // 8-byte granules, columns 2tx, 2tx+1
    constexpr int NPAIR = (CX + 2 * R + 1) / 2;
    // columns a thread copies: tx, tx + BX and, two points along x, tx + 2BX
    // (the last one only for the 2R halo columns beyond the tile)
    const int gxa = static_cast<int>(gx0) + tx, gxb = gxa + BX, gxc = gxb + BX;
    const bool col_a = gxa >= 0 && gxa < a.n2;
    const bool col_b = (VX == 2 || tx < 2 * R) && gxb < a.n2;
    const bool col_c = VX == 2 && tx < 2 * R && gxc < a.n2;
    int off_c[NLOAD_ROWS];
    unsigned ok_c = 0u;
    // pairs mode with two points along x: pair tx and pair tx + BX
    const bool pair_b = VX == 2 && tx + BX < NPAIR;
    if constexpr (HOIST) {
        const int gx1 = pairs ? static_cast<int>(gx0) + 2 * tx : gxa;
        const bool c1 = pairs ? (tx < NPAIR && gx1 + 1 < a.n2) : col_a;
        // second copy: pair tx + BX (pairs mode, two points along x) or column tx + BX
        const int gx2 = pairs ? gx1 + 2 * BX : gxb;
        const bool c2 = pairs ? (pair_b && gx2 + 1 < a.n2) : col_b;
        const bool c3 = !pairs && col_c;
#pragma unroll
        for (int i = 0; i < NLOAD_ROWS; ++i) {
            const int r = ty + i * TYT;
            const int64_t gy = gy0 + r;
            const bool row = r < H && gy >= 0 && gy < a.n1;
            const int ro = row ? static_cast<int>(gy * a.in_s1) : 0;
            off_a[i] = row && c1 ? ro + gx1 : 0;
            off_b[i] = row && c2 ? ro + gx2 : 0;
            off_c[i] = row && c3 ? ro + gxc : 0;
            ok_a |= static_cast<unsigned>(row && c1) << i;
            ok_b |= static_cast<unsigned>(row && c2) << i;
            ok_c |= static_cast<unsigned>(row && c3) << i;
        }
    } else {
#pragma unroll
        for (int i = 0; i < NLOAD_ROWS; ++i) {
            const int r = ty + i * TYT;
            const int64_t gy = gy0 + r;
            row_ok[i] = r < H && gy >= 0 && gy < a.n1;
            row_off[i] = row_ok[i] ? static_cast<int>(gy * a.in_s1) : 0;
        }
    }
    const TS *plane_src = static_cast<const TS *>(a.in) + qbeg * a.in_s0;  // plane of the next issue

    auto issue = [&](int j, int slot) {
        const int64_t p = qbeg + j;
        if constexpr (C::LD == kLdCpAsync && HOIST) {
            const TS *plane = plane_src;  // planes are issued in order, one each
            plane_src += a.in_s0;
            TS *dst = stg_base + slot * STG_ELEMS;
            if (pairs) {
#pragma unroll
                for (int i = 0; i < NLOAD_ROWS; ++i) {
                    const int r = ty + i * TYT;
                    if (r < H && tx < NPAIR) cp_async<8>(dst + r * W + 2 * tx, plane + off_a[i], (ok_a >> i) & 1u);
                    if (VX == 2 && r < H && pair_b)
                        cp_async<8>(dst + r * W + 2 * (tx + BX), plane + off_b[i], (ok_b >> i) & 1u);
                }
            } else {
#pragma unroll
                for (int i = 0; i < NLOAD_ROWS; ++i) {
                    const int r = ty + i * TYT;
                    if (r < H) {
                        cp_async<C::EB>(dst + r * W + tx, plane + off_a[i], (ok_a >> i) & 1u);
                        if (VX == 2 || tx < 2 * R)
                            cp_async<C::EB>(dst + r * W + tx + BX, plane + off_b[i], (ok_b >> i) & 1u);
                        if (VX == 2 && tx < 2 * R)
                            cp_async<C::EB>(dst + r * W + tx + 2 * BX, plane + off_c[i], (ok_c >> i) & 1u);
                    }
                }
            }
        } else if constexpr (C::LD == kLdCpAsync) {
            const TS *plane = static_cast<const TS *>(a.in) + p * a.in_s0;
            TS *dst = stg_base + slot * STG_ELEMS;
#pragma unroll
            for (int i = 0; i < NLOAD_ROWS; ++i) {
                const int r = ty + i * TYT;
                if (r < H) {
                    const TS *src = plane + row_off[i];
                    cp_async<C::EB>(dst + r * W + tx, row_ok[i] && col_a ? src + gxa : plane, row_ok[i] && col_a);
                    if (VX == 2 || tx < 2 * R)
                        cp_async<C::EB>(dst + r * W + tx + BX, row_ok[i] && col_b ? src + gxb : plane,
                                        row_ok[i] && col_b);
                    if (VX == 2 && tx < 2 * R)
                        cp_async<C::EB>(dst + r * W + tx + 2 * BX, row_ok[i] && col_c ? src + gxc : plane,
                                        row_ok[i] && col_c);
                }
            }
        } else {
            if (tid == 0) {
                asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
                mbar_expect_tx(mbar + slot, static_cast<unsigned>(W * H * C::EB));
                tma_load_3d(stg_base + slot * STG_ELEMS, &a.tmap, static_cast<int>(gx0), static_cast<int>(gy0),
                            static_cast<int>(p), mbar + slot);
            }
        }
    };

#pragma unroll 1
    for (int j = 0; j < PD; ++j) {
        if (j < nq) issue(j, j % NSTG);
        if constexpr (C::LD == kLdCpAsync) cp_commit();
    }

    const int cx = VX * tx + R + a.shift;  // smem column of this thread's (first) x
    const int own = (ty * VY + RY) * W + cx;
    // spacing of a thread's points in shared memory and in the output grid
    constexpr int PSTEP = VX == 2 ? 1 : W;
    const int64_t ostep = VX == 2 ? 1 : a.out_s1;
    constexpr bool SEP = C::SI::sep;
    TC q[NPT][(STAR || SEP) ? 2 * R + 1 : 1];  // z-queue, q[v][R + dz]: star: raw values; sep: xy-filtered
    // Float-pair sweeps (standalone launches): a thread's points are
    // summed two at a time (rows 2p, 2p+1, or a rank-2 thread's two columns)
    // into packed accumulators, acc[p] of df2 (dfs2_fma_s / df2_fma_s in
    // df32.cuh).
    constexpr bool PACK = C::PACKED && !std::is_same_v<Args, BatchArgs>;
    constexpr int NPR = PACK ? NPT / 2 : 1;
    unsigned range_err = 0;
    const bool x_ok = x0 + VX * tx < a.ub2;
    // output pointer of (zs, y0 + ty*VY, x0 + VX*tx); points vmin..vmax-1
    // are written: rows beyond ub1 are masked, and with two points along x
    // columns beyond ub2 and the column left of lb2 (xoff)
    TS *optr = static_cast<TS *>(a.out) + zs * a.out_s0 + (y0 + ty * VY) * a.out_s1 + x0 + VX * tx;
    int vmax = VX == 2 ? static_cast<int>(min(static_cast<int64_t>(2), a.ub2 - (x0 + 2 * tx)))
                       : static_cast<int>(min(static_cast<int64_t>(VY), a.ub1 - (y0 + ty * VY)));
    if (!x_ok) vmax = 0;
    const int vmin = VX == 2 && x0 + 2 * tx < a.lb2 ? 1 : 0;

    int s_stg = 0;       // staging slot of plane j
    unsigned phase = 0;  // mbarrier phase of plane j's slot
    int s_iss = PD % NSTG;
    int s_cmp = 0;  // compute-ring slot of plane j
    // 2R+1 copies of the plane step, the length of the z-queue, so its shifts
    // become register renaming: 2D stars and separable boxes, and 3D radius-1
    // stars.  GB300, GStencil/s: 3d7pt float pairs 175.4 -> 179.8, 2d5pt
    // 176.4 -> 182.3 (FP32 490 -> 511); at 8192^2 2d9pt 145.6 -> 153.8 (FP32
    // 544 -> 587), 2d13pt 110.3 -> 124.5 (FP32 479 -> 521), separable 2D
    // boxes r1/r2/r3 +4/+14/+8 %.  3D stars of radius 2-3, whose loop bodies
    // are several times larger, lose (3d13pt 118.5 -> 94.4), and so does the
    // separable 3D r1 box (148.0 -> 145.6).
    constexpr int UNROLL_Q = ((STAR && R == 1) || ((STAR || SEP) && IS2D)) ? 2 * R + 1 : 1;
#pragma unroll UNROLL_Q
    for (int j = 0; j < nq; ++j) {
        bool ok = true;
        if constexpr (C::LD == kLdCpAsync) {
            cp_wait<PD - 1>();
            __syncthreads();
        } else {
            ok = mbar_wait(mbar + s_stg, phase);
            if (__syncthreads_or(!ok)) {
                if (tid == 0) {
                    atomicOr(a.err, kDevErrTimeout);
                    // first timeout records where it happened: block, plane, slot, phase
                    if (atomicCAS(a.err + 2, 0u, 1u) == 0u) {
                        a.err[3] = blockIdx.x;
                        a.err[4] = blockIdx.z;
                        a.err[5] = static_cast<unsigned>(j);
                        a.err[6] = static_cast<unsigned>(s_stg);
                        a.err[7] = phase;
                    }
                    for (int k = j; k < min(j + PD, nq); ++k)
                        (void)mbar_wait(mbar + (k % NSTG), static_cast<unsigned>((k / NSTG) & 1));
                }
                return false;
            }
        }
        if (j + PD < nq) issue(j + PD, s_iss);
        if constexpr (C::LD == kLdCpAsync) cp_commit();

        if constexpr (C::CONVERT) {
            // Columns the loader wrote: the whole TMA box, or CX + 2R for cp.async.
            constexpr int WL = C::LD == kLdTma ? W : CX + 2 * R;
            const double *sp = reinterpret_cast<const double *>(stg_base + s_stg * STG_ELEMS);
            float2 *dp = cmp_base + s_cmp * CMP_ELEMS;
#pragma unroll
            for (int i = 0; i < NLOAD_ROWS; ++i) {
                const int r = ty + i * TYT;
                if (r < H) {
#pragma unroll
                    for (int c0 = 0; c0 < WL; c0 += BX)
                        if (c0 + tx < WL)
                            dp[r * W + c0 + tx] = split_f64(sp[r * W + c0 + tx], range_err, pair_bias(a.pair_shift));
                }
            }
            __syncthreads();
        }
        const int slot_j = C::CONVERT ? s_cmp : s_stg;
        const TC *cur = cmp_base + slot_j * CMP_STRIDE;
        if constexpr (SEP && PACK) {
            // as below, rows and points in pairs
            constexpr int D = 2 * R + 1;
            constexpr int CX0 = 2 * D;
            constexpr int NROW = VY + 2 * R;
            TC xr[NROW];
#pragma unroll
            for (int i = 0; i < NROW; i += 2) {
                const TC *r0 = cur + own + (i - R) * W, *r1 = r0 + W;
                float b0 = 0.0f, b1 = 0.0f;
#pragma unroll
                for (int dx = -R; dx <= R; ++dx) {
                    const float ch = coef_abs<C>(a, CX0 + dx + R);
                    b0 = bound_add(b0, ch, r0[dx]);
                    b1 = bound_add(b1, ch, r1[dx]);
                }
                const u64 sg = pk2(sigma_of(b0), sigma_of(b1));
                df2 t;
                float2 c = coef_f2<C>(a, CX0);
                dfs2_mul_s(t, sg, c.x, c.y, r0[-R], r1[-R]);
#pragma unroll
                for (int dx = -R + 1; dx <= R; ++dx) {
                    c = coef_f2<C>(a, CX0 + dx + R);
                    dfs2_fma_s(t, sg, c.x, c.y, r0[dx], r1[dx]);
                }
                u64 hh, ll;
                renorm2(t, hh, ll);
                upk2(hh, xr[i].x, xr[i + 1].x);
                upk2(ll, xr[i].y, xr[i + 1].y);
            }
#pragma unroll
            for (int v = 0; v < VY; v += 2) {
#pragma unroll
                for (int k = 0; k < 2 * R; ++k) {
                    q[v][k] = q[v][k + 1];
                    q[v + 1][k] = q[v + 1][k + 1];
                }
                float b0 = 0.0f, b1 = 0.0f;
#pragma unroll
                for (int dy = -R; dy <= R; ++dy) {
                    const float ch = coef_abs<C>(a, D + dy + R);
                    b0 = bound_add(b0, ch, xr[v + R + dy]);
                    b1 = bound_add(b1, ch, xr[v + 1 + R + dy]);
                }
                const u64 sg = pk2(sigma_of(b0), sigma_of(b1));
                df2 t;
                float2 c = coef_f2<C>(a, D);
                dfs2_mul_s(t, sg, c.x, c.y, xr[v], xr[v + 1]);
#pragma unroll
                for (int dy = -R + 1; dy <= R; ++dy) {
                    c = coef_f2<C>(a, D + dy + R);
                    dfs2_fma_s(t, sg, c.x, c.y, xr[v + R + dy], xr[v + 1 + R + dy]);
                }
                u64 hh, ll;
                renorm2(t, hh, ll);
                upk2(hh, q[v][2 * R].x, q[v + 1][2 * R].x);
                upk2(ll, q[v][2 * R].y, q[v + 1][2 * R].y);
            }
        } else if constexpr (SEP) {
            // xy-filter the arriving plane for this thread's points and push
            // the results into the z-queue: x pass per row (rows of the point
            // column plus the y halo), then y pass (rank 3 only).
            constexpr int D = 2 * R + 1;
            constexpr int CX0 = IS2D ? D : 2 * D;  // slot of c (x coefficients)
            constexpr int NROW = IS2D ? 1 : VY + 2 * R;
            TC xr[NROW];
#pragma unroll
            for (int i = 0; i < NROW; ++i) {
                const TC *row = cur + own + (IS2D ? 0 : (i - R) * W);
                float sg = 0.0f;
                if constexpr (A::kBounded) {
                    float b = 0.0f;
#pragma unroll
                    for (int dx = -R; dx <= R; ++dx) b = bound_add(b, coef_abs<C>(a, CX0 + dx + R), row[dx]);
                    sg = sigma_of(b);
                }
                Acc t;
                A::bfirst(t, sg, a, CX0, row[-R]);
#pragma unroll
                for (int dx = -R + 1; dx <= R; ++dx) A::badd(t, sg, a, CX0 + dx + R, row[dx]);
                A::centre(t, a, IS2D ? 1 : 2, row[0]);
                xr[i] = A::level(t);
            }
#pragma unroll
            for (int v = 0; v < VY; ++v) {
#pragma unroll
                for (int k = 0; k < 2 * R; ++k) q[v][k] = q[v][k + 1];
                if constexpr (IS2D) {
                    q[v][2 * R] = xr[0];
                } else {
                    float sg = 0.0f;
                    if constexpr (A::kBounded) {
                        float b = 0.0f;
#pragma unroll
                        for (int dy = -R; dy <= R; ++dy) b = bound_add(b, coef_abs<C>(a, D + dy + R), xr[v + R + dy]);
                        sg = sigma_of(b);
                    }
                    Acc t;
                    A::bfirst(t, sg, a, D, xr[v]);
#pragma unroll
                    for (int dy = -R + 1; dy <= R; ++dy) A::badd(t, sg, a, D + dy + R, xr[v + R + dy]);
                    A::centre(t, a, 1, xr[v + R]);
                    q[v][2 * R] = A::level(t);
                }
            }
        }
        if constexpr (STAR) {
#pragma unroll
            for (int v = 0; v < NPT; ++v) {
#pragma unroll
                for (int k = 0; k < 2 * R; ++k) q[v][k] = q[v][k + 1];
                q[v][2 * R] = cur[own + v * PSTEP];
            }
        }
        if constexpr (PACK) {
            if (j >= 2 * R) {
                // The scalar sweep below with the sums of rows 2p and 2p+1
                // packed: per point the same terms in the same order and the
                // same roundings.
                df2 acc[NPR];
                if constexpr (SEP) {
#pragma unroll
                    for (int p = 0; p < NPR; ++p) {
                        float b0 = 0.0f, b1 = 0.0f;
#pragma unroll
                        for (int dz = 0; dz < 2 * R + 1; ++dz) {
                            const float ch = coef_abs<C>(a, dz);
                            b0 = bound_add(b0, ch, q[2 * p][dz]);
                            b1 = bound_add(b1, ch, q[2 * p + 1][dz]);
                        }
                        const u64 sg = pk2(sigma_of(b0), sigma_of(b1));
                        float2 c = coef_f2<C>(a, 0);
                        dfs2_mul_s(acc[p], sg, c.x, c.y, q[2 * p][0], q[2 * p + 1][0]);
#pragma unroll
                        for (int dz = 1; dz < 2 * R + 1; ++dz) {
                            c = coef_f2<C>(a, dz);
                            dfs2_fma_s(acc[p], sg, c.x, c.y, q[2 * p][dz], q[2 * p + 1][dz]);
                        }
                    }
                } else if constexpr (STAR) {
                    const int sl = slot_j >= R ? slot_j - R : slot_j - R + NRING;
                    const TC *pl = cmp_base + sl * CMP_STRIDE;
                    // each point's sigma from all its inputs
                    u64 sg[NPR];
#pragma unroll
                    for (int p = 0; p < NPR; ++p) {
                        float b[2];
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const int v = 2 * p + h;
                            b[h] = star_bound<C>(a, q[v], pl + own + v * PSTEP);
                        }
                        sg[p] = pk2(sigma_of(b[0]), sigma_of(b[1]));
                    }
#pragma unroll
                    for (int p = 0; p < NPR; ++p) {
                        const float2 c = coef_f2<C>(a, coef_slot<C::SHAPE, R>(0, 0, 0));
                        dfs2_mul_s(acc[p], sg[p], c.x, c.y, q[2 * p][R], q[2 * p + 1][R]);
                    }
#pragma unroll
                    for (int d = 1; d <= R; ++d)
#pragma unroll
                        for (int p = 0; p < NPR; ++p) {
                            const float2 cm = coef_f2<C>(a, coef_slot<C::SHAPE, R>(-d, 0, 0));
                            const float2 cp = coef_f2<C>(a, coef_slot<C::SHAPE, R>(d, 0, 0));
                            dfs2_fma_s(acc[p], sg[p], cm.x, cm.y, q[2 * p][R - d], q[2 * p + 1][R - d]);
                            dfs2_fma_s(acc[p], sg[p], cp.x, cp.y, q[2 * p][R + d], q[2 * p + 1][R + d]);
                        }
                    if constexpr (!IS2D) {
                        TC col[VY + 2 * R];
#pragma unroll
                        for (int i = 0; i < VY + 2 * R; ++i) col[i] = pl[own + (i - R) * W];
#pragma unroll
                        for (int d = 1; d <= R; ++d)
#pragma unroll
                            for (int p = 0; p < NPR; ++p) {
                                const float2 cm = coef_f2<C>(a, coef_slot<C::SHAPE, R>(0, -d, 0));
                                const float2 cp = coef_f2<C>(a, coef_slot<C::SHAPE, R>(0, d, 0));
                                dfs2_fma_s(acc[p], sg[p], cm.x, cm.y, col[2 * p + R - d], col[2 * p + 1 + R - d]);
                                dfs2_fma_s(acc[p], sg[p], cp.x, cp.y, col[2 * p + R + d], col[2 * p + 1 + R + d]);
                            }
                    }
#pragma unroll
                    for (int d = 1; d <= R; ++d)
#pragma unroll
                        for (int p = 0; p < NPR; ++p) {
                            const TC *r0 = pl + own + 2 * p * PSTEP, *r1 = r0 + PSTEP;
                            const float2 cm = coef_f2<C>(a, coef_slot<C::SHAPE, R>(0, 0, -d));
                            const float2 cp = coef_f2<C>(a, coef_slot<C::SHAPE, R>(0, 0, d));
                            dfs2_fma_s(acc[p], sg[p], cm.x, cm.y, r0[-d], r1[-d]);
                            dfs2_fma_s(acc[p], sg[p], cp.x, cp.y, r0[d], r1[d]);
                        }
                } else {
#pragma unroll
                    for (int dz = -R; dz <= R; ++dz) {
                        const int back = R - dz;
                        const int sl = slot_j >= back ? slot_j - back : slot_j - back + NRING;
                        const TC *pl = cmp_base + sl * CMP_STRIDE;
#pragma unroll
                        for (int dx = -R; dx <= R; ++dx) {
                            TC col[VY + 2 * R];
#pragma unroll
                            for (int i = 0; i < VY + 2 * R; ++i) col[i] = pl[own + (i - R) * W + dx];
#pragma unroll
                            for (int dy = -R; dy <= R; ++dy)
#pragma unroll
                                for (int p = 0; p < NPR; ++p) {
                                    const float2 c = coef_f2<C>(a, coef_slot<C::SHAPE, R>(dz, dy, dx));
                                    if (dz == -R && dx == -R && dy == -R)
                                        df2_mul_s(acc[p], c.x, c.y, col[2 * p + R + dy], col[2 * p + 1 + R + dy]);
                                    else
                                        df2_fma_s(acc[p], c.x, c.y, col[2 * p + R + dy], col[2 * p + 1 + R + dy]);
                                }
                        }
                    }
                }
#pragma unroll
                for (int p = 0; p < NPR; ++p) {
                    float h0, h1, l0, l1;
                    if constexpr (C::ST == kStF32x2) {
                        u64 hh, ll;
                        renorm2(acc[p], hh, ll);
                        upk2(hh, h0, h1);
                        upk2(ll, l0, l1);
                        if (VX == 2 && vmin == 0 && vmax == 2 && (reinterpret_cast<uintptr_t>(optr) & 15u) == 0) {
                            *reinterpret_cast<float4 *>(optr) = make_float4(h0, l0, h1, l1);
                        } else {
                            if (2 * p >= vmin && 2 * p < vmax) optr[2 * p * ostep] = make_float2(h0, l0);
                            if (2 * p + 1 < vmax) optr[(2 * p + 1) * ostep] = make_float2(h1, l1);
                        }
                    } else {
                        upk2(acc[p].h, h0, h1);
                        upk2(acc[p].l, l0, l1);
                        if (VX == 2 && vmin == 0 && vmax == 2 && (reinterpret_cast<uintptr_t>(optr) & 15u) == 0) {
                            A::store2(optr, df{h0, l0}, df{h1, l1}, range_err, pair_bias(a.pair_shift));
                        } else {
                            if (2 * p >= vmin && 2 * p < vmax)
                                A::store(optr + 2 * p * ostep, df{h0, l0}, range_err, pair_bias(a.pair_shift));
                            if (2 * p + 1 < vmax)
                                A::store(optr + (2 * p + 1) * ostep, df{h1, l1}, range_err, pair_bias(a.pair_shift));
                        }
                    }
                }
                optr += a.out_s0;
            }
        } else if (j >= 2 * R) {
            Acc acc[NPT];
            if constexpr (SEP) {
#pragma unroll
                for (int v = 0; v < VY; ++v) {
                    float sg = 0.0f;
                    if constexpr (A::kBounded) {
                        float b = 0.0f;
#pragma unroll
                        for (int dz = 0; dz < 2 * R + 1; ++dz) b = bound_add(b, coef_abs<C>(a, dz), q[v][dz]);
                        sg = sigma_of(b);
                    }
                    A::bfirst(acc[v], sg, a, 0, q[v][0]);
#pragma unroll
                    for (int dz = 1; dz < 2 * R + 1; ++dz) A::badd(acc[v], sg, a, dz, q[v][dz]);
                    A::centre(acc[v], a, 0, q[v][R]);
                }
            } else if constexpr (STAR) {
                const int sl = slot_j >= R ? slot_j - R : slot_j - R + NRING;
                const TC *pl = cmp_base + sl * CMP_STRIDE;
                // each point's sigma from all its inputs (float pairs)
                float sg[NPT];
#pragma unroll
                for (int v = 0; v < NPT; ++v) {
                    sg[v] = 0.0f;
                    if constexpr (A::kBounded) sg[v] = sigma_of(star_bound<C>(a, q[v], pl + own + v * PSTEP));
                }
#pragma unroll
                for (int v = 0; v < NPT; ++v) {
                    A::bfirst(acc[v], sg[v], a, coef_slot<C::SHAPE, R>(0, 0, 0), q[v][R]);
                    A::centre(acc[v], a, 0, q[v][R]);
                }
#pragma unroll
                for (int d = 1; d <= R; ++d)
#pragma unroll
                    for (int v = 0; v < NPT; ++v) {
                        A::badd(acc[v], sg[v], a, coef_slot<C::SHAPE, R>(-d, 0, 0), q[v][R - d]);
                        A::badd(acc[v], sg[v], a, coef_slot<C::SHAPE, R>(d, 0, 0), q[v][R + d]);
                    }
                if constexpr (!IS2D) {
                    TC col[VY + 2 * R];
#pragma unroll
                    for (int i = 0; i < VY + 2 * R; ++i) col[i] = pl[own + (i - R) * W];
#pragma unroll
                    for (int d = 1; d <= R; ++d)
#pragma unroll
                        for (int v = 0; v < VY; ++v) {
                            A::badd(acc[v], sg[v], a, coef_slot<C::SHAPE, R>(0, -d, 0), col[v + R - d]);
                            A::badd(acc[v], sg[v], a, coef_slot<C::SHAPE, R>(0, d, 0), col[v + R + d]);
                        }
                }
                if constexpr (IS2D && C::XS) {
                    // x-neighbours from the lanes d columns away (the warp's
                    // lanes hold consecutive columns; their centre values are
                    // in the z-queue), the warp's edge lanes from shared memory
                    const int lane = tid & 31;
                    const TC cen = q[0][R];
                    const TC *row = pl + own;
#pragma unroll
                    for (int d = 1; d <= R; ++d) {
                        TC lft = shfl_up_tc(cen, d), rgt = shfl_down_tc(cen, d);
                        if (lane < d) lft = row[-d];
                        if (lane >= 32 - d) rgt = row[d];
                        A::badd(acc[0], sg[0], a, coef_slot<C::SHAPE, R>(0, 0, -d), lft);
                        A::badd(acc[0], sg[0], a, coef_slot<C::SHAPE, R>(0, 0, d), rgt);
                    }
                } else {
#pragma unroll
                    for (int d = 1; d <= R; ++d)
#pragma unroll
                        for (int v = 0; v < NPT; ++v) {
                            const TC *row = pl + own + v * PSTEP;
                            A::badd(acc[v], sg[v], a, coef_slot<C::SHAPE, R>(0, 0, -d), row[-d]);
                            A::badd(acc[v], sg[v], a, coef_slot<C::SHAPE, R>(0, 0, d), row[d]);
                        }
                }
            } else {
#pragma unroll
                for (int dz = -R; dz <= R; ++dz) {
                    const int back = R - dz;  // plane j - R + dz is `back` planes behind j
                    const int sl = slot_j >= back ? slot_j - back : slot_j - back + NRING;
                    const TC *pl = cmp_base + sl * CMP_STRIDE;
                    if constexpr (IS2D) {
#pragma unroll
                        for (int dx = -R; dx <= R; ++dx) {
                            const TC v0 = pl[own + dx];
                            if (dz == -R && dx == -R) A::first(acc[0], a, coef_slot<C::SHAPE, R>(dz, 0, dx), v0);
                            else A::add(acc[0], a, coef_slot<C::SHAPE, R>(dz, 0, dx), v0);
                            if (dz == 0 && dx == 0) A::centre(acc[0], a, 0, v0);
                        }
                    } else {
#pragma unroll
                        for (int dx = -R; dx <= R; ++dx) {
                            TC col[VY + 2 * R];
#pragma unroll
                            for (int i = 0; i < VY + 2 * R; ++i) col[i] = pl[own + (i - R) * W + dx];
#pragma unroll
                            for (int dy = -R; dy <= R; ++dy)
#pragma unroll
                                for (int v = 0; v < VY; ++v) {
                                    if (dz == -R && dx == -R && dy == -R)
                                        A::first(acc[v], a, coef_slot<C::SHAPE, R>(dz, dy, dx), col[v + R + dy]);
                                    else
                                        A::add(acc[v], a, coef_slot<C::SHAPE, R>(dz, dy, dx), col[v + R + dy]);
                                    if (dz == 0 && dx == 0 && dy == 0) A::centre(acc[v], a, 0, col[v + R]);
                                }
                        }
                    }
                }
            }
            if constexpr (VX == 2 && A::kVecStore) {
                // two adjacent columns in one vector store when aligned
                if (vmin == 0 && vmax == 2 && (reinterpret_cast<uintptr_t>(optr) & (2 * sizeof(TS) - 1)) == 0)
                    A::store2(optr, acc[0], acc[1], range_err, pair_bias(a.pair_shift));
                else
#pragma unroll
                    for (int v = 0; v < NPT; ++v)
                        if (v >= vmin && v < vmax) A::store(optr + v * ostep, acc[v], range_err, pair_bias(a.pair_shift));
            } else {
#pragma unroll
                for (int v = 0; v < NPT; ++v)
                    if (v >= vmin && v < vmax) A::store(optr + v * ostep, acc[v], range_err, pair_bias(a.pair_shift));
            }
            optr += a.out_s0;
        }
        // advance the rings
        s_stg = s_stg + 1 == NSTG ? 0 : s_stg + 1;
        if (s_stg == 0) phase ^= 1u;
        s_iss = s_iss + 1 == NSTG ? 0 : s_iss + 1;
        if constexpr (C::CONVERT) s_cmp = s_cmp + 1 == NCMP ? 0 : s_cmp + 1;
    }
    if constexpr (C::CONVERT) {
        if (range_err) atomicOr(a.err, kDevErrRange);
    }
    __syncthreads();
    return true;
}

// One CTA's work: mbarrier set-up for the TMA loader, then the item.
template <class C>
__device__ __forceinline__ void stream_cta(const StreamArgs<C::NT> &a) {
    extern __shared__ __align__(128) unsigned char smem[];
    if constexpr (C::LD == kLdTma) {
        uint64_t *const mbar = reinterpret_cast<uint64_t *>(smem + C::NSTG * C::STG_SLOT +
                                                            (C::CONVERT ? C::NCMP * C::CMP_SLOT : 0));
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            for (int s = 0; s < C::NSTG; ++s) mbar_init(mbar + s, 1);
            asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        }
        __syncthreads();
    }
    (void)stream_item<C>(a, blockIdx.x, blockIdx.y, blockIdx.z, smem);
}

template <class C>
__global__ void __launch_bounds__(C::THREADS) k_stream(const __grid_constant__ StreamArgs<C::NT> a) {
    stream_cta<C>(a);
}

// FP32 variants run as k_stream_occ4, held to 4 CTAs per SM: the 256-thread
// tiles to 64 registers (half the warp slots instead of 3/8 at the 72 they
// would take; no spills, 2-3 % faster on GB300, cfg2 FP32 584 vs 573
// GStencil/s) and the 128-thread VY 8 tiles to 128 (3d3r FP32 star 421 vs 305
// GStencil/s at the 185 registers and 2 CTAs they would take).  The other
// variants keep ptxas's own register choice: the float-pair 3d7pt kernel
// takes 32 registers there and 47 under an explicit minimum of one CTA,
// which costs it 10 %.
template <class C>
constexpr bool stream_occ4() {
    return C::ST == kStF32 && (C::THREADS == 256 || C::VY == 8);
}
template <class C>
__global__ void __launch_bounds__(C::THREADS, 4) k_stream_occ4(const __grid_constant__ StreamArgs<C::NT> a) {
    stream_cta<C>(a);
}

}  // namespace uhs
