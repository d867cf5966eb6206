// FP32 3D box stencils of radius 2 and 3 on the fifth-generation tensor cores
// (tcgen05, kind::tf32, accumulators in tensor memory).
//
// The box update out[z][y][x] = sum_{dz,dy,dx} c[dz][dy][dx] in[z+dz][y+dy][x+dx]
// is, for one input plane z+dz and one row shift dy, a product of the plane's
// rows with a banded Toeplitz matrix along x:
//
//   D[m][n] += sum_k A[m][k] * B[k][n],   A[m][k] = in[z+dz][y0+m+dy][x0-4+k],
//                                         B[k][n] = c[dz][dy][k-4-n]  (0 outside |dx| <= R)
//
// with M = 128 output rows (y), N = 16 output columns (x) and K = 24 window
// columns (16 + 4 + R <= 24).  The A operand is the staged input plane itself:
// shared memory holds it in the canonical no-swizzle K-major layout with every
// row 16 bytes from the next (core-matrix groups 128 bytes apart, K chunks of 4
// floats LBO bytes apart), so the row shift dy is a 16*dy byte offset of the
// matrix descriptor and no data moves per (dz, dy).  B is one of D*D small
// Toeplitz images built once per CTA.
//
// Accuracy: tf32 keeps 11 significant bits, so operands are split into
// round-to-nearest tf32 hi + lo parts and each product is formed as
// hi*hi + lo*hi + hi*lo (three MMAs; the dropped lo*lo term is below 2^-22
// relative with random sign).  Accumulation is FP32 in tensor memory.
//
// Streaming: a CTA walks z.  Input plane zi contributes to the 2R+1 output
// planes zi-R..zi+R, each an accumulator in tensor memory; 2R+2 accumulators
// rotate, so the one completed by the previous plane is drained (tcgen05.ld ->
// global) while the current plane's MMAs run.  Two input stages alternate;
// the next plane's global loads are in flight in registers meanwhile.  The
// kernel is persistent: each CTA takes a contiguous range of (tile, z) plane
// tiles, so the SMs get equal shares whatever the grid's shape.
//
// Variant (UHS_FLAG_MMA_TMEM_A): the A operand staged in tensor memory, D
// row-shifted hi/lo copies per input plane made by tcgen05.cp, so the MMAs
// read only the small B from shared memory.  Tensor memory holds one set of
// copies beside the accumulators (464 of 512 columns for R = 3), so a plane's
// copies wait for the previous plane's MMAs.  Measured on GB300 it is slower
// (15 vs 20 GStencil/s, 343-point box): the MMA instructions themselves, at
// N = 16, not the operand reads, set the pace.
//
// Every wait is bounded: a wait that runs out sets the device error word,
// waits (bounded) for its own MMAs, frees its tensor memory and returns.
#include <cuda_runtime.h>

#include <cstdint>

#include "stream_kernel.cuh"
#include "uhs_kernels.h"

namespace uhs {
namespace {

constexpr int kMmaThreads = 128;  // 4 warps: one per 32-lane quarter of tensor memory
constexpr int kMmaM = 128;        // output rows per tile (MMA M)

struct MmaArgs {
    const float *in;
    float *out;
    int64_t si0, so0;  // plane strides (elements)
    int si1, so1;      // row strides (elements)
    int lb0, lb1, lb2, ub0, ub1, ub2;
    int tiles_x;
    int nz;
    long long work;  // tiles * nz plane tiles
    unsigned *err;
    double cd[343];
};

template <int R, int NS, bool ATMEM>
struct MmaCfg {
    static constexpr int D = 2 * R + 1;
    static constexpr int YR = kMmaM + 2 * R;  // staged rows
    static constexpr int XT = 16 * NS;        // output columns per tile
    static constexpr int XW = XT + 8;         // staged columns, from x0 - 4
    static constexpr int NCH = XW / 4;        // 16-byte K chunks per row
    static constexpr uint32_t LBO_A = YR * 16;
    static constexpr uint32_t HALF = NCH * LBO_A;  // one of hi / lo
    static constexpr uint32_t STG = 2 * HALF;
    static constexpr uint32_t BMAT = 6 * 256;  // K = 24 (6 chunks) x N = 16
    static constexpr uint32_t BPAIR = 2 * BMAT;
    static constexpr uint32_t B_OFF = 2 * STG;
    static constexpr uint32_t BAR_OFF = B_OFF + D * D * BPAIR;
    static constexpr uint32_t SMEM = BAR_OFF + 32;
    static constexpr int NSLOT = 2 * R + 2;
    // A in tensor memory: D row-shifted copies of the staged plane, each
    // 24 hi + 24 lo columns, after the accumulators.
    static constexpr int ACOL0 = NSLOT * XT;
    static constexpr int COLS = ATMEM ? ACOL0 + D * 48 : NSLOT * XT;
    static constexpr uint32_t NCOLS = COLS <= 32 ? 32 : COLS <= 64 ? 64 : COLS <= 128 ? 128 : COLS <= 256 ? 256 : 512;
    static constexpr int NE = YR * XW;
    static constexpr int NQ = (NE + kMmaThreads - 1) / kMmaThreads;
    // instruction descriptor: D f32, A/B tf32, both K-major, N = 16, M = 128
    static constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
    static_assert(COLS <= 512, "tensor memory holds 512 columns");
    static_assert(!ATMEM || NS == 1, "A in tensor memory: one 16-column tile");
    static_assert(SMEM <= 232448, "shared memory per CTA");
    static_assert(D * D * D * 8 <= STG, "coefficient table fits in stage 0");
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ float tf32_rna(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;\n" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// Shared-memory matrix descriptor, no swizzle (layout 0), version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return static_cast<uint64_t>((addr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>(lbo >> 4) << 16) |
           (static_cast<uint64_t>(sbo >> 4) << 32) | (static_cast<uint64_t>(1) << 46);
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
// A from tensor memory (lanes = rows, columns = K), B from shared memory.
__device__ __forceinline__ void mma_tf32_ta(uint32_t d, uint32_t a_tmem, uint64_t b, uint32_t idesc,
                                            uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n}\n" ::"r"(d),
        "r"(a_tmem), "l"(b), "r"(idesc), "r"(acc));
}
// Shared memory (128 rows x 32 bytes, canonical layout) -> tensor memory
// lanes 0-127, 8 columns.
__device__ __forceinline__ void tmem_cp_128x256b(uint32_t taddr, uint64_t src) {
    asm volatile("tcgen05.cp.cta_group::1.128x256b [%0], %1;\n" ::"r"(taddr), "l"(src) : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// 16 consecutive accumulator columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

template <class C, int R>
__device__ __forceinline__ void load_plane(float (&v)[C::NQ], const MmaArgs &a, int z, int x0, int y0) {
    const float *pl = a.in + static_cast<int64_t>(z) * a.si0;
#pragma unroll
    for (int q = 0; q < C::NQ; ++q) {
        const int e = threadIdx.x + q * kMmaThreads;
        const int r = e / C::XW, j = e - r * C::XW;
        const int y = y0 - R + r, x = x0 - 4 + j;
        // cells outside [lb - R, ub + R) never enter the sum: stage zeros there
        const bool ok = e < C::NE && y >= a.lb1 - R && y < a.ub1 + R && x >= a.lb2 - R && x < a.ub2 + R;
        v[q] = ok ? __ldg(pl + y * a.si1 + x) : 0.0f;
    }
}

template <class C>
__device__ __forceinline__ void store_plane(const float (&v)[C::NQ], unsigned char *stage) {
#pragma unroll
    for (int q = 0; q < C::NQ; ++q) {
        const int e = threadIdx.x + q * kMmaThreads;
        if (e < C::NE) {
            const int r = e / C::XW, j = e - r * C::XW;
            const float h = tf32_rna(v[q]);
            const float l = tf32_rna(v[q] - h);
            const uint32_t off = static_cast<uint32_t>(j >> 2) * C::LBO_A + static_cast<uint32_t>(r) * 16u +
                                 static_cast<uint32_t>(j & 3) * 4u;
            *reinterpret_cast<float *>(stage + off) = h;
            *reinterpret_cast<float *>(stage + C::HALF + off) = l;
        }
    }
}

// All MMAs of input plane zi (one thread).  With A in tensor memory the
// plane's D row-shifted hi/lo copies are made first (tcgen05.cp, executed
// before the MMAs issued after them by the same thread).
template <class C, int R, int NS, bool ATMEM>
__device__ __forceinline__ void issue_plane(uint32_t st_addr, uint32_t b_addr, uint32_t tbase, int zi, int zs,
                                            int ze) {
    if constexpr (ATMEM) {
#pragma unroll 1
        for (int dyi = 0; dyi < C::D; ++dyi)
#pragma unroll
            for (int half = 0; half < 2; ++half)
#pragma unroll
                for (int c3 = 0; c3 < 3; ++c3)
                    tmem_cp_128x256b(tbase + C::ACOL0 + (dyi * 2 + half) * 24 + 8 * c3,
                                     sdesc(st_addr + half * C::HALF + (2u * c3) * C::LBO_A + dyi * 16u, C::LBO_A,
                                           128));
#pragma unroll 1
        for (int dzi = 0; dzi < C::D; ++dzi) {
            const int zo = zi + R - dzi;
            if (zo < zs || zo >= ze) continue;
            const uint32_t dcol = tbase + static_cast<uint32_t>((zo - zs) % C::NSLOT) * C::XT;
#pragma unroll 1
            for (int dyi = 0; dyi < C::D; ++dyi) {
                const uint64_t bh = sdesc(b_addr + static_cast<uint32_t>(dzi * C::D + dyi) * C::BPAIR, 256, 128);
                const uint64_t bl = bh + (C::BMAT >> 4);
                const uint32_t ah = tbase + C::ACOL0 + dyi * 48, al = ah + 24;
#pragma unroll
                for (int ks = 0; ks < 3; ++ks) {
                    const uint64_t kb = (2u * ks * 256u) >> 4;
                    const uint32_t acc = (dzi == 0 && dyi == 0 && ks == 0) ? 0u : 1u;
                    mma_tf32_ta(dcol, ah + 8 * ks, bh + kb, C::IDESC, acc);
                    mma_tf32_ta(dcol, al + 8 * ks, bh + kb, C::IDESC, 1u);
                    mma_tf32_ta(dcol, ah + 8 * ks, bl + kb, C::IDESC, 1u);
                }
            }
        }
        return;
    }
#pragma unroll 1
    for (int dzi = 0; dzi < C::D; ++dzi) {
        const int zo = zi + R - dzi;  // dz = dzi - R, zo = zi - dz
        if (zo < zs || zo >= ze) continue;
        const uint32_t dcol = tbase + static_cast<uint32_t>((zo - zs) % C::NSLOT) * C::XT;
#pragma unroll 1
        for (int dyi = 0; dyi < C::D; ++dyi) {
            const uint64_t bh = sdesc(b_addr + static_cast<uint32_t>(dzi * C::D + dyi) * C::BPAIR, 256, 128);
            const uint64_t bl = bh + (C::BMAT >> 4);
#pragma unroll
            for (int t = 0; t < NS; ++t) {
                const uint64_t ah = sdesc(st_addr + static_cast<uint32_t>(4 * t) * C::LBO_A + dyi * 16u, C::LBO_A, 128);
                const uint64_t al = ah + (C::HALF >> 4);
#pragma unroll
                for (int ks = 0; ks < 3; ++ks) {
                    const uint64_t ka = (2u * ks * C::LBO_A) >> 4, kb = (2u * ks * 256u) >> 4;
                    // dzi == 0 is the first input plane of output zo
                    const uint32_t acc = (dzi == 0 && dyi == 0 && ks == 0) ? 0u : 1u;
                    mma_tf32(dcol + 16 * t, ah + ka, bh + kb, C::IDESC, acc);
                    mma_tf32(dcol + 16 * t, al + ka, bh + kb, C::IDESC, 1u);
                    mma_tf32(dcol + 16 * t, ah + ka, bl + kb, C::IDESC, 1u);
                }
            }
        }
    }
}

template <class C, int NS>
__device__ __forceinline__ void drain(const MmaArgs &a, uint32_t tbase, int zo, int zs, int x0, int y0) {
    const int warp = threadIdx.x >> 5;
    const int y = y0 + static_cast<int>(threadIdx.x);  // lane of tensor memory = output row
    const uint32_t col = tbase + (static_cast<uint32_t>(warp * 32) << 16) +
                         static_cast<uint32_t>((zo - zs) % C::NSLOT) * C::XT;
#pragma unroll
    for (int t = 0; t < NS; ++t) {
        float v[16];
        tmem_ld16(col + 16 * t, v);
        if (y < a.ub1) {
            float *row = a.out + static_cast<int64_t>(zo) * a.so0 + static_cast<int64_t>(y) * a.so1;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int x = x0 + 16 * t + j;
                if (x < a.ub2) row[x] = v[j];
            }
        }
    }
}

// First timeout records where it happened: block, input plane, stage, phase.
__device__ void record_timeout(const MmaArgs &a, int zi, int stage, unsigned phase) {
    atomicOr(a.err, kDevErrTimeout);
    if (atomicCAS(a.err + 2, 0u, 1u) != 0u) return;
    a.err[3] = blockIdx.x;
    a.err[4] = 0;
    a.err[5] = static_cast<unsigned>(zi);
    a.err[6] = static_cast<unsigned>(stage);
    a.err[7] = phase;
}

template <int R, int NS, bool ATMEM>
__global__ void __launch_bounds__(kMmaThreads, 1) k_box_mma(const __grid_constant__ MmaArgs a) {
    using C = MmaCfg<R, NS, ATMEM>;
    extern __shared__ __align__(1024) unsigned char smem[];
    const int tid = threadIdx.x, warp = tid >> 5;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + C::BAR_OFF);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(smem + C::BAR_OFF + 16);
    const uint32_t sbase = smem_u32(smem);

    // coefficients as tf32 hi / lo (staged in stage 0 until the first plane)
    constexpr int D3 = C::D * C::D * C::D;
    float *chi = reinterpret_cast<float *>(smem);
    float *clo = chi + D3;
    for (int k = tid; k < D3; k += kMmaThreads) {
        const double c = a.cd[k];
        const float h = tf32_rna(static_cast<float>(c));
        chi[k] = h;
        clo[k] = tf32_rna(static_cast<float>(c - static_cast<double>(h)));
    }
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(tslot)),
                     "r"(C::NCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    __syncthreads();
    // Toeplitz images: pair p = dzi*D + dyi, half (hi, lo), entry (k, n) at
    // (k/4)*256 + n*16 + (k%4)*4; one 16-byte chunk of 4 k per item.
    for (int e = tid; e < C::D * C::D * 2 * 16 * 6; e += kMmaThreads) {
        const int c4 = e % 6, n = (e / 6) % 16, half = (e / 96) % 2, p = e / 192;
        const float *src = half ? clo : chi;
        float q[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int dx = 4 * c4 + u - 4 - n;
            q[u] = (dx >= -R && dx <= R) ? src[p * C::D + dx + R] : 0.0f;
        }
        *reinterpret_cast<float4 *>(smem + C::B_OFF + p * C::BPAIR + half * C::BMAT + c4 * 256 + n * 16) =
            make_float4(q[0], q[1], q[2], q[3]);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;
    const uint32_t b_addr = sbase + C::B_OFF;

    unsigned ph[2] = {0u, 0u};
    bool bad = false;
    long long lo = a.work * blockIdx.x / gridDim.x;
    const long long hi = a.work * (blockIdx.x + 1) / gridDim.x;
    float v[C::NQ];
    while (lo < hi && !bad) {
        const long long tile = lo / a.nz;
        const int z0 = static_cast<int>(lo - tile * a.nz);
        const int len = static_cast<int>(hi - lo < a.nz - z0 ? hi - lo : a.nz - z0);
        lo += len;
        const int x0 = a.lb2 + static_cast<int>(tile % a.tiles_x) * C::XT;
        const int y0 = a.lb1 + static_cast<int>(tile / a.tiles_x) * kMmaM;
        const int zs = a.lb0 + z0, ze = zs + len;
        const int nin = len + 2 * R;
        load_plane<C, R>(v, a, zs - R, x0, y0);
        for (int i = 0; i < nin; ++i) {
            const int zi = zs - R + i, s = i & 1;
            // stage s was last read by plane i-2's MMAs, awaited in iteration i-1
            store_plane<C>(v, smem + s * C::STG);
            if (i + 1 < nin) load_plane<C, R>(v, a, zi + 1, x0, y0);
            fence_async_smem();
            tc_fence_before();
            __syncthreads();
            if (tid == 0) {
                tc_fence_after();
                // A in tensor memory is single-buffered: plane i's copies
                // overwrite what plane i-1's MMAs read, so they wait for
                // those MMAs (the drain below waits on the same phase).
                bool aok = true;
                if constexpr (ATMEM)
                    if (i >= 1) aok = mbar_wait(&bar[s ^ 1], ph[s ^ 1]);
                if (aok) issue_plane<C, R, NS, ATMEM>(sbase + s * C::STG, b_addr, tbase, zi, zs, ze);
                mma_commit(&bar[s]);
            }
            if (i >= 1) {
                // plane i-1's MMAs: frees stage s^1, completes output zi-1-R
                const int sp = s ^ 1;
                const bool ok = mbar_wait(&bar[sp], ph[sp]);
                ph[sp] ^= 1u;
                if (__syncthreads_or(!ok)) {
                    if (tid == 0) record_timeout(a, zi - 1, sp, ph[sp] ^ 1u);
                    (void)mbar_wait(&bar[s], ph[s]);  // this plane's MMAs, bounded
                    bad = true;
                    break;
                }
                tc_fence_after();
                if (zi - 1 - R >= zs) drain<C, NS>(a, tbase, zi - 1 - R, zs, x0, y0);
                tc_fence_before();
            }
        }
        if (bad) break;
        const int sl = (nin - 1) & 1;
        const bool ok = mbar_wait(&bar[sl], ph[sl]);
        ph[sl] ^= 1u;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) record_timeout(a, ze - 1 + R, sl, ph[sl] ^ 1u);
            bad = true;
            break;
        }
        tc_fence_after();
        drain<C, NS>(a, tbase, ze - 1, zs, x0, y0);
        tc_fence_before();
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tbase), "r"(C::NCOLS)
                     : "memory");
    }
}

template <int R, int NS, bool ATMEM>
cudaError_t launch_t(const MmaCall &c) {
    using C = MmaCfg<R, NS, ATMEM>;
    auto kern = k_box_mma<R, NS, ATMEM>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
    if (e != cudaSuccess) return e;
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kMmaThreads, C::SMEM);
    if (e != cudaSuccess) return e;
    if (c.occ_out) {
        *c.occ_out = occ;
        return cudaSuccess;
    }
    MmaArgs a{};
    a.in = static_cast<const float *>(c.in.data);
    a.out = static_cast<float *>(c.out.data);
    a.si0 = c.in.s[0];
    a.so0 = c.out.s[0];
    a.si1 = static_cast<int>(c.in.s[1]);
    a.so1 = static_cast<int>(c.out.s[1]);
    a.lb0 = static_cast<int>(c.lb[0]);
    a.lb1 = static_cast<int>(c.lb[1]);
    a.lb2 = static_cast<int>(c.lb[2]);
    a.ub0 = static_cast<int>(c.ub[0]);
    a.ub1 = static_cast<int>(c.ub[1]);
    a.ub2 = static_cast<int>(c.ub[2]);
    const int64_t nx = c.ub[2] - c.lb[2], ny = c.ub[1] - c.lb[1], nz = c.ub[0] - c.lb[0];
    if (nx <= 0 || ny <= 0 || nz <= 0) return cudaSuccess;
    a.tiles_x = static_cast<int>((nx + C::XT - 1) / C::XT);
    const int64_t tiles = a.tiles_x * ((ny + kMmaM - 1) / kMmaM);
    a.nz = static_cast<int>(nz);
    a.work = tiles * nz;
    a.err = c.err;
    constexpr int D3 = C::D * C::D * C::D;
    for (int k = 0; k < D3; ++k) a.cd[k] = c.coef[k];
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t grid = std::min<int64_t>(a.work, static_cast<int64_t>(sms) * std::max(occ, 1));
    kern<<<static_cast<unsigned>(grid), kMmaThreads, C::SMEM, c.stream>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_box_mma(const MmaCall &c) {
    if (c.a_tmem) {
        if (c.R == 3 && c.xtile == 16) return launch_t<3, 1, true>(c);
        if (c.R == 2 && c.xtile == 16) return launch_t<2, 1, true>(c);
        return cudaErrorInvalidValue;
    }
    if (c.R == 3 && c.xtile == 16) return launch_t<3, 1, false>(c);
    if (c.R == 2 && c.xtile == 16) return launch_t<2, 1, false>(c);
    if (c.R == 2 && c.xtile == 32) return launch_t<2, 2, false>(c);
    return cudaErrorInvalidValue;
}

}  // namespace uhs
