// Temporal fusion: K timesteps of a 3D 7-point star per pass over HBM.
//
// A CTA owns a 32 x 16 output tile and streams its z-chunk.  It loads the
// input tile enlarged by K cells on every side (cp.async, two planes ahead)
// and, for every plane that arrives, computes level 1 on the tile shrunk by
// one cell, level 2 on the tile shrunk by two, ..., level K on the output
// tile, each level from the previous level's three-plane ring in shared
// memory (the wavefront of levels trails the input plane by one plane per
// level).  Only level 0 is read from HBM and only level K is written.
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
#include "stream_launch.cuh"

namespace uhs {
namespace {

template <int ST_, int AR_, int K_>
struct FusedCfg {
    static constexpr int ST = ST_, AR = AR_, K = K_, R = 1;
    static constexpr int BX = 32, BY = 16, THREADS = 256, PD = 2;
    using TS = std::conditional_t<ST == kStF64, double, float>;
    static constexpr bool CONVERT = (AR == kArDf32);
    using TC = std::conditional_t<CONVERT, float2, TS>;
    static constexpr int EB = sizeof(TS);
    static constexpr int W0 = BX + 2 * K, H0 = BY + 2 * K;
    static constexpr int PLANE = W0 * H0;
    static constexpr int NSTG = CONVERT ? PD + 1 : 3 + PD;  // level-0 staging ring
    static constexpr int SMEM = NSTG * PLANE * EB + (CONVERT ? 3 * PLANE * (int)sizeof(TC) : 0) +
                                (K - 1) * 3 * PLANE * (int)sizeof(TC);
    static constexpr int NT = 7;
};

struct FusedArgs {
    const void *in;
    void *out;
    int64_t in_s0, in_s1, out_s0, out_s1;
    int64_t n0, n1, n2;
    int64_t lb0, lb1, lb2, ub0, ub1, ub2;
    int zchunk;
    int pair_shift;  // FP64 grids in float pairs: the pairs hold x * 2^pair_shift (df32.cuh)
    unsigned *err;
    double cd[7];
    float2 chl[7];
    float cl_sum;
};

template <class C, int AR = C::AR>
struct FArith;
template <class C>
struct FArith<C, kArNative> {  // float grids: centre correction as in Arith (stream_kernel.cuh)
    using T = typename C::TS;
    static constexpr bool F32 = std::is_same_v<T, float>;
    using Acc = T;
    __device__ static T c(const FusedArgs &a, int k) {
        if constexpr (F32) return a.chl[k].x;
        else return a.cd[k];
    }
    __device__ static void first(Acc &s, const FusedArgs &a, int k, T v) { s = c(a, k) * v; }
    __device__ static void add(Acc &s, const FusedArgs &a, int k, T v) { s = fma(c(a, k), v, s); }
    __device__ static void centre(Acc &s, const FusedArgs &a, T v) {
        if constexpr (F32) s = fmaf(a.cl_sum, v, s);
    }
    __device__ static T level(const Acc &s) { return s; }
    __device__ static void store(T *p, const Acc &s, unsigned &, int) { *p = s; }
};
template <class C>
struct FArith<C, kArDf32> {
    using Acc = df;
    __device__ static void first(Acc &s, const FusedArgs &a, int k, float2 v) {
        df_mul(s, a.chl[k].x, a.chl[k].y, v);
    }
    __device__ static void add(Acc &s, const FusedArgs &a, int k, float2 v) { df_fma(s, a.chl[k].x, a.chl[k].y, v); }
    __device__ static void centre(Acc &, const FusedArgs &, float2) {}
    __device__ static float2 level(const Acc &s) { return renorm(s); }
    // joined with the run's exponent bias; a sum that outgrew the float range
    // sets the range flag (as in Arith)
    __device__ static void store(double *p, const Acc &s, unsigned &range_err, int bias) {
        range_err |= (__float_as_uint(s.h) & 0x7f800000u) == 0x7f800000u;
        *p = join_f64(s.h, s.l, bias);
    }
};

template <class C>
__global__ void __launch_bounds__(256) k_fused(const __grid_constant__ FusedArgs a) {
    using TS = typename C::TS;
    using TC = typename C::TC;
    using A = FArith<C>;
    constexpr int K = C::K, W0 = C::W0, H0 = C::H0, PLANE = C::PLANE, NSTG = C::NSTG, PD = C::PD;
    extern __shared__ __align__(128) unsigned char smem[];
    TS *const stg = reinterpret_cast<TS *>(smem);
    TC *const lvl0 = C::CONVERT ? reinterpret_cast<TC *>(smem + NSTG * PLANE * C::EB) : nullptr;
    TC *const rings = reinterpret_cast<TC *>(smem + NSTG * PLANE * C::EB + (C::CONVERT ? 3 * PLANE * sizeof(TC) : 0));

    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    const int64_t x0 = a.lb2 + static_cast<int64_t>(blockIdx.x) * C::BX;
    const int64_t y0 = a.lb1 + static_cast<int64_t>(blockIdx.y) * C::BY;
    const int64_t zs = a.lb0 + static_cast<int64_t>(blockIdx.z) * a.zchunk;
    const int64_t ze = min(zs + static_cast<int64_t>(a.zchunk), a.ub0);
    const int64_t gx0 = x0 - K, gy0 = y0 - K, qbeg = zs - K;
    const int nq = static_cast<int>(ze - zs) + 2 * K;
    unsigned range_err = 0;

    auto issue = [&](int i) {
        const int64_t p = qbeg + i;
        const bool pin = p >= 0 && p < a.n0;
        TS *dst = stg + (i % NSTG) * PLANE;
        const TS *src = static_cast<const TS *>(a.in);
        for (int e = tid; e < PLANE; e += 256) {
            const int r = e / W0, c = e % W0;
            const int64_t gy = gy0 + r, gx = gx0 + c;
            const bool ok = pin && gy >= 0 && gy < a.n1 && gx >= 0 && gx < a.n2;
            cp_async<C::EB>(dst + e, ok ? src + p * a.in_s0 + gy * a.in_s1 + gx : src, ok);
        }
    };
    // value of level j (0..K-1) in plane slot s at cell e
    auto lv = [&](int j, int slot_plane, int e) -> TC {
        if (j == 0) {
            if constexpr (C::CONVERT) return lvl0[(slot_plane % 3) * PLANE + e];
            else return stg[(slot_plane % NSTG) * PLANE + e];
        }
        return rings[((j - 1) * 3 + slot_plane % 3) * PLANE + e];
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
            float2 *dp = lvl0 + (i % 3) * PLANE;
            for (int e = tid; e < PLANE; e += 256) dp[e] = split_f64(sp[e], range_err, pair_bias(a.pair_shift));
            __syncthreads();
        }
#pragma unroll
        for (int j = 1; j <= K; ++j) {
            if (i < 2 * j) break;  // level j's first plane needs iteration 2j
            const int64_t p = qbeg + i - j;  // plane of level j computed now
            const int sp_ = i - j;           // its index relative to qbeg (>= j)
            const bool zin = p >= a.lb0 && p < a.ub0;
            const int Wj = W0 - 2 * j, Hj = H0 - 2 * j;
            for (int e2 = tid; e2 < Wj * Hj; e2 += 256) {
                const int r = j + e2 / Wj, c = j + e2 % Wj;
                const int e = r * W0 + c;
                const int64_t gy = gy0 + r, gx = gx0 + c;
                const bool in_dom = zin && gy >= a.lb1 && gy < a.ub1 && gx >= a.lb2 && gx < a.ub2;
                typename A::Acc acc;
                if (in_dom) {
                    A::first(acc, a, coef_slot<kStar3, 1>(0, 0, 0), lv(j - 1, sp_, e));
                    A::add(acc, a, coef_slot<kStar3, 1>(-1, 0, 0), lv(j - 1, sp_ - 1, e));
                    A::add(acc, a, coef_slot<kStar3, 1>(1, 0, 0), lv(j - 1, sp_ + 1, e));
                    A::add(acc, a, coef_slot<kStar3, 1>(0, -1, 0), lv(j - 1, sp_, e - W0));
                    A::add(acc, a, coef_slot<kStar3, 1>(0, 1, 0), lv(j - 1, sp_, e + W0));
                    A::add(acc, a, coef_slot<kStar3, 1>(0, 0, -1), lv(j - 1, sp_, e - 1));
                    A::add(acc, a, coef_slot<kStar3, 1>(0, 0, 1), lv(j - 1, sp_, e + 1));
                    A::centre(acc, a, lv(j - 1, sp_, e));
                }
                if (j < K) {
                    TC v;
                    if (in_dom) v = A::level(acc);
                    else v = lv(j - 1, sp_, e);
                    rings[((j - 1) * 3 + sp_ % 3) * PLANE + e] = v;
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

template <class C>
cudaError_t launch_fused_t(const StreamCall &c) {
    FusedArgs a{};
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
    fill_coefs(a.cd, a.chl, sums, c.coef, 7, c.shape, c.R);
    a.cl_sum = sums[0];
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(k_fused<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (c.occ_out) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(c.occ_out, k_fused<C>, 256, C::SMEM);
    const int64_t nz = c.ub[0] - c.lb[0], ny = c.ub[1] - c.lb[1], nx = c.ub[2] - c.lb[2];
    if (nz <= 0 || ny <= 0 || nx <= 0) return cudaSuccess;
    dim3 grid(static_cast<unsigned>((nx + C::BX - 1) / C::BX), static_cast<unsigned>((ny + C::BY - 1) / C::BY),
              static_cast<unsigned>((nz + c.zchunk - 1) / c.zchunk));
    k_fused<C><<<grid, dim3(32, 8), C::SMEM, c.stream>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_fused(const StreamCall &c, int K) {
    if (c.shape != kStar3 || c.R != 1) return cudaErrorInvalidValue;
    if (c.st == kStF64 && c.ar == kArDf32) {
        if (K == 2) return launch_fused_t<FusedCfg<kStF64, kArDf32, 2>>(c);
        if (K == 4) return launch_fused_t<FusedCfg<kStF64, kArDf32, 4>>(c);
    } else if (c.st == kStF64) {
        if (K == 2) return launch_fused_t<FusedCfg<kStF64, kArNative, 2>>(c);
        if (K == 4) return launch_fused_t<FusedCfg<kStF64, kArNative, 4>>(c);
    } else if (c.st == kStF32) {
        if (K == 2) return launch_fused_t<FusedCfg<kStF32, kArNative, 2>>(c);
        if (K == 4) return launch_fused_t<FusedCfg<kStF32, kArNative, 4>>(c);
    }
    return cudaErrorInvalidValue;
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
