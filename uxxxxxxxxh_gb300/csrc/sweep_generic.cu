// Generic sweep: any linear stencil expression (up to UHS_MAX_TERMS terms,
// |offset| <= UHS_MAX_RADIUS), evaluated term by term in the order the .dsl
// expression writes them.
//
// This is the kernel shape UHStencil's GPU lowering emits
// (examples/2d5pt_star/2d5pt_gpu.mlir:10-102; its hand-written twin
// examples/3d27pt_box/3d27pt.cu:20-129): a shared-memory input tile with the
// halo around it, one output per thread.  What differs is the schedule:
//   * each CTA streams a chunk of planes along the slowest axis and keeps the
//     2*rz+1 planes a point needs in a ring of shared-memory slots, so every
//     input plane is fetched from global memory once per CTA instead of once
//     per neighbouring plane;
//   * planes arrive by cp.async one plane ahead of the compute, so the fetch
//     of plane z+rz+1 overlaps the sums for plane z;
//   * results go straight from registers to global memory (no output tile).
// With UHS_ARITH_EXACT every product and sum is rounded separately in
// expression order, which makes the result bit-identical to the serial CPU
// loops (UH-SW/*/stencil_*_driver.serial.c mpe_verify).
#include "uhs_kernels.h"

#include <algorithm>

namespace uhs {
namespace {

template <int MAXT>
struct GenericTerms {
    int32_t plane[MAXT];    // dz + rz
    int32_t inplane[MAXT];  // dy * W + dx
    double coef[MAXT];
};

template <class T, int MAXT>
struct GenericArgs {
    const T *in;
    T *out;
    int64_t in_s0, in_s1, out_s0, out_s1;
    int64_t n0, n1, n2;
    int64_t lb0, lb1, lb2, ub0, ub1, ub2;
    int rz, ry, rx;
    int W, H, NS;
    int zchunk;
    int nterms;
    GenericTerms<MAXT> t;
};

__device__ __forceinline__ void cp_async_elem(void *smem, const void *gmem, bool valid, int bytes) {
    unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    int src_size = valid ? bytes : 0;
    if (bytes == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(src_size));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(gmem), "r"(src_size));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;\n" ::); }

template <class T>
__device__ __forceinline__ T mul_rn(T a, T b);
template <>
__device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <>
__device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <class T>
__device__ __forceinline__ T add_rn(T a, T b);
template <>
__device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <>
__device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }

// blockDim = (TX, TY); one output point per thread per plane.
template <class T, int MAXT, bool EXACT>
__global__ void __launch_bounds__(256) k_generic(const __grid_constant__ GenericArgs<T, MAXT> a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *ring = reinterpret_cast<T *>(smem_raw);
    __shared__ int plane_base[2 * UHS_MAX_RADIUS + 1];

    const int TX = blockDim.x, TY = blockDim.y;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t x0 = a.lb2 + (int64_t)blockIdx.x * TX;
    const int64_t y0 = a.lb1 + (int64_t)blockIdx.y * TY;
    const int64_t zs = a.lb0 + (int64_t)blockIdx.z * a.zchunk;
    const int64_t ze = min(zs + (int64_t)a.zchunk, a.ub0);
    const int plane_elems = a.W * a.H;

    // Ring slot of plane p.  Planes below 0 occur when the program reaches
    // only upwards in z from a domain starting at 0; they are zero-filled
    // and must still land in a slot of the ring, so the modulo is floored.
    auto slot_of = [&](int64_t p) { return static_cast<int>(((p % a.NS) + a.NS) % a.NS); };
    auto load_plane = [&](int64_t p) {
        T *dst = ring + slot_of(p) * plane_elems;
        const bool zin = (p >= 0) && (p < a.n0);
        for (int r = ty; r < a.H; r += TY) {
            const int64_t gy = y0 - a.ry + r;
            const bool yin = zin && gy >= 0 && gy < a.n1;
            for (int c = tx; c < a.W; c += TX) {
                const int64_t gx = x0 - a.rx + c;
                const bool ok = yin && gx >= 0 && gx < a.n2;
                const T *src = ok ? a.in + p * a.in_s0 + gy * a.in_s1 + gx : a.in;
                cp_async_elem(dst + r * a.W + c, src, ok, (int)sizeof(T));
            }
        }
    };

    // Prologue: planes zs-rz .. zs+rz, then one plane of look-ahead.
    for (int64_t p = zs - a.rz; p <= zs + a.rz; ++p) {
        load_plane(p);
        cp_async_commit();
    }
    const int64_t last_needed = ze - 1 + a.rz;
    if (zs + a.rz + 1 <= last_needed) load_plane(zs + a.rz + 1);
    cp_async_commit();

    const int64_t y = y0 + ty, x = x0 + tx;
    const bool active = (y < a.ub1) && (x < a.ub2);
    const int center = (ty + a.ry) * a.W + (tx + a.rx);

    for (int64_t z = zs; z < ze; ++z) {
        cp_async_wait_1();
        if (ty == 0 && tx <= 2 * a.rz) plane_base[tx] = slot_of(z - a.rz + tx) * plane_elems;
        __syncthreads();
        if (active) {
            const T *c0 = ring + center;
            T acc;
            {
                const T v = c0[plane_base[a.t.plane[0]] + a.t.inplane[0]];
                const T c = static_cast<T>(a.t.coef[0]);
                acc = EXACT ? mul_rn<T>(c, v) : c * v;
            }
            for (int k = 1; k < a.nterms; ++k) {
                const T v = c0[plane_base[a.t.plane[k]] + a.t.inplane[k]];
                const T c = static_cast<T>(a.t.coef[k]);
                if (EXACT)
                    acc = add_rn<T>(acc, mul_rn<T>(c, v));
                else
                    acc = fma(c, v, acc);
            }
            a.out[z * a.out_s0 + y * a.out_s1 + x] = acc;
        }
        __syncthreads();
        if (z + a.rz + 2 <= last_needed) load_plane(z + a.rz + 2);
        cp_async_commit();
    }
}

template <class T, int MAXT, bool EXACT>
cudaError_t launch_t(const SweepSpec &sp, const LaunchCfg &cfg, const GridView &in, const GridView &out,
                     cudaStream_t st) {
    GenericArgs<T, MAXT> a{};
    a.in = static_cast<const T *>(in.data);
    a.out = static_cast<T *>(out.data);
    a.in_s0 = in.s[0];
    a.in_s1 = in.s[1];
    a.out_s0 = out.s[0];
    a.out_s1 = out.s[1];
    a.n0 = in.n[0];
    a.n1 = in.n[1];
    a.n2 = in.n[2];
    a.lb0 = sp.lb[0];
    a.lb1 = sp.lb[1];
    a.lb2 = sp.lb[2];
    a.ub0 = sp.ub[0];
    a.ub1 = sp.ub[1];
    a.ub2 = sp.ub[2];
    a.rz = sp.rz;
    a.ry = sp.ry;
    a.rx = sp.rx;
    const int TX = cfg.tile_x > 0 ? cfg.tile_x : 32;
    const int TY = cfg.tile_y > 0 ? cfg.tile_y : 8;
    a.W = TX + 2 * sp.rx;
    a.H = TY + 2 * sp.ry;
    a.NS = 2 * sp.rz + 2;
    a.nterms = sp.nterms;
    for (int k = 0; k < sp.nterms; ++k) {
        a.t.plane[k] = sp.dz[k] + sp.rz;
        a.t.inplane[k] = sp.dy[k] * a.W + sp.dx[k];
        a.t.coef[k] = sp.coef[k];
    }
    const int64_t nz = sp.ub[0] - sp.lb[0], ny = sp.ub[1] - sp.lb[1], nx = sp.ub[2] - sp.lb[2];
    if (nz <= 0 || ny <= 0 || nx <= 0) return cudaSuccess;
    const int64_t tiles = ((nx + TX - 1) / TX) * ((ny + TY - 1) / TY);
    int zchunk = cfg.tile_z;
    if (zchunk <= 0) {
        // Enough CTAs to fill the SMs several times over, chunks long enough
        // that the 2*rz warm-up planes stay a small fraction.
        const int64_t want = static_cast<int64_t>(device_sm_count()) * 16;
        const int64_t want_chunks = std::max<int64_t>(1, (want + tiles - 1) / tiles);
        zchunk = (int)std::max<int64_t>(std::max(8, 4 * sp.rz), (nz + want_chunks - 1) / want_chunks);
    }
    a.zchunk = (int)std::min<int64_t>(zchunk, nz);
    const size_t smem = (size_t)a.NS * a.W * a.H * sizeof(T);
    auto kern = k_generic<T, MAXT, EXACT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((nx + TX - 1) / TX), (unsigned)((ny + TY - 1) / TY),
              (unsigned)((nz + a.zchunk - 1) / a.zchunk));
    dim3 block(TX, TY);
    kern<<<grid, block, smem, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_generic(const SweepSpec &sp, const LaunchCfg &cfg, const GridView &in, const GridView &out,
                           cudaStream_t st) {
    const bool exact = cfg.arith == UHS_ARITH_EXACT;
    const int tx = cfg.tile_x > 0 ? cfg.tile_x : 32, ty = cfg.tile_y > 0 ? cfg.tile_y : 8;
    if (tx * ty > 256 || tx <= 0 || ty <= 0) return cudaErrorInvalidValue;
    if (sp.dtype == UHS_F64) {
        if (sp.nterms <= 64)
            return exact ? launch_t<double, 64, true>(sp, cfg, in, out, st)
                         : launch_t<double, 64, false>(sp, cfg, in, out, st);
        return exact ? launch_t<double, UHS_MAX_TERMS, true>(sp, cfg, in, out, st)
                     : launch_t<double, UHS_MAX_TERMS, false>(sp, cfg, in, out, st);
    }
    if (sp.dtype == UHS_F32) {
        if (sp.nterms <= 64)
            return exact ? launch_t<float, 64, true>(sp, cfg, in, out, st)
                         : launch_t<float, 64, false>(sp, cfg, in, out, st);
        return exact ? launch_t<float, UHS_MAX_TERMS, true>(sp, cfg, in, out, st)
                     : launch_t<float, UHS_MAX_TERMS, false>(sp, cfg, in, out, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace uhs
