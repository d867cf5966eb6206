// Temporal fusion: K timesteps of a star or box stencil (radius R, rank 2 or
// 3) per pass over HBM.
//
// A CTA owns an output tile -- 32 x 16 cells of a plane in 3D (32 x 8 for
// radius 2-3), a strip of 256 - 2KR columns of a row in 2D -- and streams its
// chunk of planes (rows in 2D).  It loads the input tile enlarged by KR
// cells on every side (cp.async, two planes ahead) and, for every plane that
// arrives, computes level 1 on the tile shrunk by R cells, level 2 on the
// tile shrunk by 2R, ..., level K on the output tile, each level from the
// previous level's ring of 2R + 1 planes in shared memory (level j trails
// the input plane by jR planes).  Only level 0 is read from HBM and only
// level K is written.
//
// Cells outside the domain keep the previous level's value: the sweep never
// writes them, so at every level they hold the grid's halo.  That equals the
// reference's two-buffer semantics when both grids hold the same halo values
// (the reference's serial drivers initialise both grids identically,
// UH-SW/3d1r_star/stencil_3d7pt_driver.serial.c:96-105); the runtime checks
// this on the device before fusing (k_halo_diff).
//
// Arithmetic: native FP32/FP64, or float pairs for FP64 grids (levels are
// stored renormalised; the join to double happens once, at level K).
// Terms are summed in the streaming kernel's order: centre, then +-d along
// z, y, x (stars); z-major over the box (boxes).
#pragma once
#include "stream_launch.cuh"

namespace uhs {
namespace fused {

template <int SHAPE_, int R_, int ST_, int AR_, int K_>
struct FusedCfg {
    static constexpr int SHAPE = SHAPE_, R = R_, ST = ST_, AR = AR_, K = K_;
    static constexpr bool IS2D = (SHAPE == kStar2 || SHAPE == kBox2);
    static constexpr bool STAR = (SHAPE == kStar2 || SHAPE == kStar3);
    static constexpr int THREADS = 256, PD = 2;
    static constexpr int D = 2 * R + 1;
    static constexpr int HALO = K * R;
    // output tile: a 256-cell row less the halo (2D); 32 x 16, or 32 x 8 for radius 2-3 (3D)
    static constexpr int BX = IS2D ? THREADS - 2 * HALO : 32;
    static constexpr int BY = IS2D ? 1 : (R >= 2 ? 8 : 16);
    static constexpr int W0 = BX + 2 * HALO, H0 = IS2D ? 1 : BY + 2 * HALO;
    static constexpr int PLANE = W0 * H0;
    using TS = std::conditional_t<ST == kStF64, double, float>;
    static constexpr bool CONVERT = (AR == kArDf32);
    using TC = std::conditional_t<CONVERT, float2, TS>;
    static constexpr int EB = sizeof(TS);
    // level-0 staging: raw planes until converted (float pairs), else the
    // D planes a level-1 plane reads plus the PD in flight
    static constexpr int NSTG = CONVERT ? PD + 1 : D + PD;
    static constexpr int SMEM = NSTG * PLANE * EB + (CONVERT ? D * PLANE * (int)sizeof(TC) : 0) +
                                (K - 1) * D * PLANE * (int)sizeof(TC);
    static constexpr int NT = STAR ? (IS2D ? 4 * R + 1 : 6 * R + 1) : (IS2D ? D * D : D * D * D);
    static_assert(BX > 0 && SMEM <= 227 * 1024, "fused tile does not fit shared memory");
};

template <int NT>
struct FusedArgs {
    const void *in;
    void *out;
    int64_t in_s0, in_s1, out_s0, out_s1;
    int64_t n0, n1, n2;
    int64_t lb0, lb1, lb2, ub0, ub1, ub2;
    int zchunk;
    int pair_shift;  // FP64 grids in float pairs: the pairs hold x * 2^pair_shift (df32.cuh)
    unsigned *err;
    double cd[NT];
    float2 chl[NT];
    float cl_sum;
};

template <class C, int AR = C::AR>
struct FArith;
template <class C>
struct FArith<C, kArNative> {  // float grids: centre correction as in Arith (stream_kernel.cuh)
    using T = typename C::TS;
    using Args = FusedArgs<C::NT>;
    static constexpr bool F32 = std::is_same_v<T, float>;
    using Acc = T;
    __device__ static T c(const Args &a, int k) {
        if constexpr (F32) return a.chl[k].x;
        else return a.cd[k];
    }
    __device__ static void first(Acc &s, const Args &a, int k, T v) { s = c(a, k) * v; }
    __device__ static void add(Acc &s, const Args &a, int k, T v) { s = fma(c(a, k), v, s); }
    __device__ static void centre(Acc &s, const Args &a, T v) {
        if constexpr (F32) s = fmaf(a.cl_sum, v, s);
    }
    __device__ static T level(const Acc &s) { return s; }
    __device__ static void store(T *p, const Acc &s, unsigned &, int) { *p = s; }
};
template <class C>
struct FArith<C, kArDf32> {
    using Args = FusedArgs<C::NT>;
    using Acc = df;
    __device__ static void first(Acc &s, const Args &a, int k, float2 v) { df_mul(s, a.chl[k].x, a.chl[k].y, v); }
    __device__ static void add(Acc &s, const Args &a, int k, float2 v) { df_fma(s, a.chl[k].x, a.chl[k].y, v); }
    __device__ static void centre(Acc &, const Args &, float2) {}
    __device__ static float2 level(const Acc &s) { return renorm(s); }
    // joined with the run's exponent bias; a sum that outgrew the float range
    // sets the range flag (as in Arith)
    __device__ static void store(double *p, const Acc &s, unsigned &range_err, int bias) {
        range_err |= (__float_as_uint(s.h) & 0x7f800000u) == 0x7f800000u;
        *p = join_f64(s.h, s.l, bias);
    }
};

template <class C>
__global__ void __launch_bounds__(256) k_fused(const __grid_constant__ FusedArgs<C::NT> a) {
    using TS = typename C::TS;
    using TC = typename C::TC;
    using A = FArith<C>;
    constexpr int K = C::K, R = C::R, D = C::D, HALO = C::HALO, W0 = C::W0, H0 = C::H0, PLANE = C::PLANE;
    constexpr int NSTG = C::NSTG, PD = C::PD, SH = C::SHAPE;
    extern __shared__ __align__(128) unsigned char smem[];
    TS *const stg = reinterpret_cast<TS *>(smem);
    TC *const lvl0 = C::CONVERT ? reinterpret_cast<TC *>(smem + NSTG * PLANE * C::EB) : nullptr;
    TC *const rings = reinterpret_cast<TC *>(smem + NSTG * PLANE * C::EB + (C::CONVERT ? D * PLANE * sizeof(TC) : 0));

    const int tid = threadIdx.x;
    const int64_t x0 = a.lb2 + static_cast<int64_t>(blockIdx.x) * C::BX;
    const int64_t y0 = a.lb1 + static_cast<int64_t>(blockIdx.y) * C::BY;
    const int64_t zs = a.lb0 + static_cast<int64_t>(blockIdx.z) * a.zchunk;
    const int64_t ze = min(zs + static_cast<int64_t>(a.zchunk), a.ub0);
    const int64_t gx0 = x0 - HALO, gy0 = C::IS2D ? y0 : y0 - HALO, qbeg = zs - HALO;
    const int nq = static_cast<int>(ze - zs) + 2 * HALO;
    unsigned range_err = 0;

    auto issue = [&](int i) {
        const int64_t p = qbeg + i;
        const bool pin = p >= 0 && p < a.n0;
        TS *dst = stg + (i % NSTG) * PLANE;
        const TS *src = static_cast<const TS *>(a.in);
        for (int e = tid; e < PLANE; e += C::THREADS) {
            const int r = e / W0, c = e % W0;
            const int64_t gy = gy0 + r, gx = gx0 + c;
            const bool ok = pin && gy >= 0 && gy < a.n1 && gx >= 0 && gx < a.n2;
            cp_async<C::EB>(dst + e, ok ? src + p * a.in_s0 + gy * a.in_s1 + gx : src, ok);
        }
    };
    // value of level j (0..K-1) of plane sp (relative to qbeg) at cell e
    auto lv = [&](int j, int sp, int e) -> TC {
        if (j == 0) {
            if constexpr (C::CONVERT) return lvl0[(sp % D) * PLANE + e];
            else return stg[(sp % NSTG) * PLANE + e];
        }
        return rings[((j - 1) * D + sp % D) * PLANE + e];
    };

    for (int i = 0; i < PD; ++i) {
        if (i < nq) issue(i);
        cp_commit();
    }
#pragma unroll 1
    for (int i = 0; i < nq; ++i) {
        cp_wait<PD - 1>();
        __syncthreads();
        if (i + PD < nq) issue(i + PD);
        cp_commit();
        if constexpr (C::CONVERT) {
            const double *sp = reinterpret_cast<const double *>(stg + (i % NSTG) * PLANE);
            float2 *dp = lvl0 + (i % D) * PLANE;
            for (int e = tid; e < PLANE; e += C::THREADS) dp[e] = split_f64(sp[e], range_err, pair_bias(a.pair_shift));
            __syncthreads();
        }
#pragma unroll
        for (int j = 1; j <= K; ++j) {
            if (i < 2 * j * R) break;        // level j's first plane needs iteration 2jR
            const int sp_ = i - j * R;       // plane of level j computed now, relative to qbeg (>= jR)
            const int64_t p = qbeg + sp_;
            const bool zin = p >= a.lb0 && p < a.ub0;
            const int m = j * R;             // level j covers the tile shrunk by jR
            const int Wj = W0 - 2 * m, Hj = C::IS2D ? 1 : H0 - 2 * m;
            for (int e2 = tid; e2 < Wj * Hj; e2 += C::THREADS) {
                const int r = C::IS2D ? 0 : m + e2 / Wj, c = m + e2 % Wj;
                const int e = r * W0 + c;
                const int64_t gy = gy0 + r, gx = gx0 + c;
                const bool in_dom = zin && gy >= a.lb1 && gy < a.ub1 && gx >= a.lb2 && gx < a.ub2;
                typename A::Acc acc;
                if (in_dom) {
                    if constexpr (C::STAR) {
                        const TC cen = lv(j - 1, sp_, e);
                        A::first(acc, a, coef_slot<SH, R>(0, 0, 0), cen);
                        A::centre(acc, a, cen);
#pragma unroll
                        for (int d = 1; d <= R; ++d) {
                            A::add(acc, a, coef_slot<SH, R>(-d, 0, 0), lv(j - 1, sp_ - d, e));
                            A::add(acc, a, coef_slot<SH, R>(d, 0, 0), lv(j - 1, sp_ + d, e));
                        }
                        if constexpr (!C::IS2D) {
#pragma unroll
                            for (int d = 1; d <= R; ++d) {
                                A::add(acc, a, coef_slot<SH, R>(0, -d, 0), lv(j - 1, sp_, e - d * W0));
                                A::add(acc, a, coef_slot<SH, R>(0, d, 0), lv(j - 1, sp_, e + d * W0));
                            }
                        }
#pragma unroll
                        for (int d = 1; d <= R; ++d) {
                            A::add(acc, a, coef_slot<SH, R>(0, 0, -d), lv(j - 1, sp_, e - d));
                            A::add(acc, a, coef_slot<SH, R>(0, 0, d), lv(j - 1, sp_, e + d));
                        }
                    } else {
                        constexpr int RY = C::IS2D ? 0 : R;
                        bool first = true;
#pragma unroll 1
                        for (int dz = -R; dz <= R; ++dz)
#pragma unroll
                            for (int dy = -RY; dy <= RY; ++dy)
#pragma unroll
                                for (int dx = -R; dx <= R; ++dx) {
                                    const TC v = lv(j - 1, sp_ + dz, e + dy * W0 + dx);
                                    const int k = coef_slot<SH, R>(dz, dy, dx);
                                    if (first) A::first(acc, a, k, v);
                                    else A::add(acc, a, k, v);
                                    first = false;
                                    if (dz == 0 && dy == 0 && dx == 0) A::centre(acc, a, v);
                                }
                    }
                }
                if (j < K) {
                    TC v;
                    if (in_dom) v = A::level(acc);
                    else v = lv(j - 1, sp_, e);
                    rings[((j - 1) * D + sp_ % D) * PLANE + e] = v;
                } else if (in_dom) {
                    A::store(static_cast<TS *>(a.out) + p * a.out_s0 + gy * a.out_s1 + gx, acc, range_err,
                             pair_bias(a.pair_shift));
                }
            }
            __syncthreads();
        }
    }
    if constexpr (C::CONVERT) {
        if (range_err) atomicOr(a.err, kDevErrRange);
    }
}

template <class C>
cudaError_t launch_fused_t(const StreamCall &c) {
    FusedArgs<C::NT> a{};
    a.in = c.in.data;
    a.out = c.out.data;
    a.in_s0 = c.in.s[0];
    a.in_s1 = c.in.s[1];
    a.out_s0 = c.out.s[0];
    a.out_s1 = c.out.s[1];
    a.n0 = c.in.n[0];
    a.n1 = c.in.n[1];
    a.n2 = c.in.n[2];
    a.lb0 = c.lb[0];
    a.lb1 = c.lb[1];
    a.lb2 = c.lb[2];
    a.ub0 = c.ub[0];
    a.ub1 = c.ub[1];
    a.ub2 = c.ub[2];
    a.zchunk = c.zchunk;
    a.pair_shift = c.pair_shift;
    a.err = c.err;
    float sums[3];
    fill_coefs(a.cd, a.chl, sums, c.coef, C::NT, c.shape, c.R);
    a.cl_sum = sums[0];
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(k_fused<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (c.occ_out) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(c.occ_out, k_fused<C>, C::THREADS, C::SMEM);
    const int64_t nz = c.ub[0] - c.lb[0], ny = c.ub[1] - c.lb[1], nx = c.ub[2] - c.lb[2];
    if (nz <= 0 || ny <= 0 || nx <= 0) return cudaSuccess;
    dim3 grid(static_cast<unsigned>((nx + C::BX - 1) / C::BX), static_cast<unsigned>((ny + C::BY - 1) / C::BY),
              static_cast<unsigned>((nz + c.zchunk - 1) / c.zchunk));
    k_fused<C><<<grid, C::THREADS, C::SMEM, c.stream>>>(a);
    count_launch();
    return cudaGetLastError();
}

// Depths per radius: 2 and 4 in 2D; in 3D 2 and, for radius 1, 4 (deeper
// 3D tiles of radius 2-3 do not fit shared memory).
template <int SHAPE, int ST, int AR>
cudaError_t launch_fused_shape(const StreamCall &c, int K) {
    constexpr bool is2d = (SHAPE == kStar2 || SHAPE == kBox2);
    switch (c.R * 10 + K) {
        case 12: return launch_fused_t<FusedCfg<SHAPE, 1, ST, AR, 2>>(c);
        case 14: return launch_fused_t<FusedCfg<SHAPE, 1, ST, AR, 4>>(c);
        case 22: return launch_fused_t<FusedCfg<SHAPE, 2, ST, AR, 2>>(c);
        case 32: return launch_fused_t<FusedCfg<SHAPE, 3, ST, AR, 2>>(c);
        case 24:
            if constexpr (is2d) return launch_fused_t<FusedCfg<SHAPE, 2, ST, AR, 4>>(c);
            else return cudaErrorInvalidValue;
        case 34:
            if constexpr (is2d) return launch_fused_t<FusedCfg<SHAPE, 3, ST, AR, 4>>(c);
            else return cudaErrorInvalidValue;
        default: return cudaErrorInvalidValue;
    }
}

template <int STAR, int BOX>
cudaError_t launch_fused_rank(const StreamCall &c, int K) {
    const int sh = c.shape == STAR ? STAR : c.shape == BOX ? BOX : -1;
    if (sh < 0) return cudaErrorInvalidValue;
    if (c.st == kStF64 && c.ar == kArDf32)
        return sh == STAR ? launch_fused_shape<STAR, kStF64, kArDf32>(c, K) : launch_fused_shape<BOX, kStF64, kArDf32>(c, K);
    if (c.st == kStF64 && c.ar == kArNative)
        return sh == STAR ? launch_fused_shape<STAR, kStF64, kArNative>(c, K)
                          : launch_fused_shape<BOX, kStF64, kArNative>(c, K);
    if (c.st == kStF32 && c.ar == kArNative)
        return sh == STAR ? launch_fused_shape<STAR, kStF32, kArNative>(c, K)
                          : launch_fused_shape<BOX, kStF32, kArNative>(c, K);
    return cudaErrorInvalidValue;
}

}  // namespace fused
}  // namespace uhs
