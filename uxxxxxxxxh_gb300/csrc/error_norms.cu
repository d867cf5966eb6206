// FP64 error reduction on the GPU: how far a grid is from a reference grid
// over a stencil's domain.  This is the comparison the reference's drivers
// make on the host after every run (UH-GPU/3d1r_star/3d7pt_main.cpp:84-96,
// |cpu - gpu| <= 1e-6 per point), done here in FP64 on the device for grids
// of any element type so that FP32 and float-pair results can be scored
// against an FP64 result without copying either grid back.
//
// Two launches: k_err_partial has each of at most kErrBlocks CTAs reduce its
// share of the domain's work units (kErrRowsPerUnit rows, or an x-chunk of
// them when the rows are few and long) into one slot of a partials array
// (sum of squared differences, sum of squared reference values,
// max |difference|, max |reference|); k_err_final reduces the slots into the
// result.  The partials array is scratch memory owned by the runtime (grown
// on demand, one per device) or, for the allocation-free entry, a fixed array
// in the library's device memory.
//
// The sums stay in FP64 (3 FP64 operations per point: the difference and two
// squares), which bounds the kernel by GB300's FP64 pipe rather than HBM;
// the maxima run on the integer pipes.
#include <cuda.h>

#include <mutex>

#include "uhs_kernels.h"

// Scratch of uhs_error_norms_noalloc: partial sums of up to
// UHS_NOALLOC_MAX_PARTIALS CTAs (a reduction uses at most kErrBlocks) plus
// the 4-double result.  Lives in the
// library's device memory on every GPU that loads it; host code must not use
// this name as an address (it is a host-side stand-in): the device address
// comes from cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[4 * (UHS_NOALLOC_MAX_PARTIALS + 1)];
static_assert(uhs::kErrBlocks <= UHS_NOALLOC_MAX_PARTIALS, "every reduction fits the allocation-free scratch");

namespace uhs {
int set_error(int code, const char *fmt, ...);
int prepare_error_norms(const uhs_stencil_desc *d, const uhs_memref *x, const uhs_memref *ref, ErrNormsCall *c,
                        bool *empty);

namespace {

constexpr int kErrThreads = 256;

// Exact float -> double.  Normal floats and zeros are widened by bit
// construction on the integer pipes; subnormals, infinities and NaNs (rare)
// take the conversion instruction.  Same value as static_cast in every case.
__device__ __forceinline__ double widen(float v) {
    const unsigned b = __float_as_uint(v), m = b & 0x7fffffffu, s = b & 0x80000000u;
    if (m - 0x00800000u < 0x7f000000u)
        return __hiloint2double(static_cast<int>(s | ((m >> 3) + (896u << 20))), static_cast<int>(b << 29));
    if (m == 0u) return __hiloint2double(static_cast<int>(s), 0);
    return static_cast<double>(v);
}

template <class T>
__device__ __forceinline__ double load_val(const T *p);
template <>
__device__ __forceinline__ double load_val<double>(const double *p) {
    return *p;
}
template <>
__device__ __forceinline__ double load_val<float>(const float *p) {
    return widen(*p);
}
template <>
__device__ __forceinline__ double load_val<float2>(const float2 *p) {
    const float2 v = *p;
    return widen(v.x) + widen(v.y);
}

// max |v| on the integer pipes.  The bit patterns of non-negative doubles
// order as their values, so |v| is kept as its (high, low) 32-bit words and
// compared lexicographically; 64-bit integer compares, and the FP64 min/max,
// would load the FP64 pipe (a small fraction of the FP32 rate on this part),
// which then does only the subtraction and the two squares.  A NaN's high
// word is above kInfHi, or equal to it with a nonzero fraction.
constexpr unsigned kInfHi = 0x7ff00000u;
struct AbsMax {
    unsigned h = 0, l = 0;
    __device__ __forceinline__ void add(unsigned vh, unsigned vl) {
        const bool gt = vh > h, eq = vh == h;
        l = gt ? vl : (eq ? max(l, vl) : l);
        h = max(h, vh);
    }
    __device__ __forceinline__ double value() const {
        return __hiloint2double(static_cast<int>(h), static_cast<int>(l));
    }
};
__device__ __forceinline__ bool is_nan_words(unsigned h, unsigned l) { return h > kInfHi || (h == kInfHi && l); }

struct ErrArgs {
    const void *x;
    const double *r;
    int64_t xs0, xs1, rs0, rs1;
    int64_t lb0, lb1, lb2, ub0, ub1, ub2;
    int64_t rows;   // (ub0 - lb0) * (ub1 - lb1)
    int64_t units;  // row units x xchunks (err_split)
    int xchunks;
    double *partials;
    double *result;
};

__device__ __forceinline__ void block_reduce(double &s2, double &r2, double &md, double &mr, double *sh) {
    for (int o = 16; o > 0; o >>= 1) {
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
        mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sh[4 * w] = s2;
        sh[4 * w + 1] = r2;
        sh[4 * w + 2] = md;
        sh[4 * w + 3] = mr;
    }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        s2 = lane < nw ? sh[4 * lane] : 0.0;
        r2 = lane < nw ? sh[4 * lane + 1] : 0.0;
        md = lane < nw ? sh[4 * lane + 2] : 0.0;
        mr = lane < nw ? sh[4 * lane + 3] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
            r2 += __shfl_xor_sync(0xffffffffu, r2, o);
            md = fmax(md, __shfl_xor_sync(0xffffffffu, md, o));
            mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
        }
    }
}

// Each CTA takes work units blockIdx.x, blockIdx.x + gridDim.x, ...; a unit
// is kErrRowsPerUnit consecutive (z, y) rows of the domain over one x-chunk.
// One warp per row at a time, lanes striding along x.  max |x - r| counts a
// NaN difference as +inf; a NaN reference value does not raise max |r|.
template <class T>
__global__ void __launch_bounds__(kErrThreads) k_err_partial(const ErrArgs a) {
    __shared__ double sh[4 * (kErrThreads / 32)];
    double s2 = 0.0, r2 = 0.0;
    AbsMax kd, kr;
    const int64_t ny = a.ub1 - a.lb1;
    const int64_t cw = ((a.ub2 - a.lb2 + a.xchunks - 1) / a.xchunks + 31) & ~int64_t(31);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const T *x = static_cast<const T *>(a.x);
    for (int64_t u = blockIdx.x; u < a.units; u += gridDim.x) {
        const int64_t row0 = (u / a.xchunks) * kErrRowsPerUnit, row1 = min(row0 + kErrRowsPerUnit, a.rows);
        const int64_t x0 = a.lb2 + (u % a.xchunks) * cw, x1 = min(x0 + cw, a.ub2);
        for (int64_t row = row0 + warp; row < row1; row += kErrThreads / 32) {
            const int64_t z = a.lb0 + row / ny, y = a.lb1 + row % ny;
            const T *xr = x + z * a.xs0 + y * a.xs1;
            const double *rr = a.r + z * a.rs0 + y * a.rs1;
#pragma unroll 4
            for (int64_t i = x0 + lane; i < x1; i += 32) {
                const double rv = rr[i];
                const double d = load_val<T>(xr + i) - rv;
                s2 = fma(d, d, s2);
                r2 = fma(rv, rv, r2);
                const unsigned dh = static_cast<unsigned>(__double2hiint(d)) & 0x7fffffffu;
                const unsigned dl = static_cast<unsigned>(__double2loint(d));
                const unsigned rh = static_cast<unsigned>(__double2hiint(rv)) & 0x7fffffffu;
                const unsigned rl = static_cast<unsigned>(__double2loint(rv));
                if (is_nan_words(dh, dl)) kd.add(kInfHi, 0u);
                else kd.add(dh, dl);
                if (!is_nan_words(rh, rl)) kr.add(rh, rl);
            }
        }
    }
    double md = kd.value(), mr = kr.value();
    block_reduce(s2, r2, md, mr, sh);
    if (threadIdx.x == 0) {
        double *p = a.partials + 4 * static_cast<int64_t>(blockIdx.x);
        p[0] = s2;
        p[1] = r2;
        p[2] = md;
        p[3] = mr;
    }
}

__global__ void __launch_bounds__(kErrThreads) k_err_final(const double *partials, int n, double *result) {
    __shared__ double sh[4 * (kErrThreads / 32)];
    double s2 = 0.0, r2 = 0.0, md = 0.0, mr = 0.0;
    for (int i = threadIdx.x; i < n; i += kErrThreads) {
        s2 += partials[4 * i];
        r2 += partials[4 * i + 1];
        md = fmax(md, partials[4 * i + 2]);
        mr = fmax(mr, partials[4 * i + 3]);
    }
    block_reduce(s2, r2, md, mr, sh);
    if (threadIdx.x == 0) {
        result[0] = r2 > 0.0 ? sqrt(s2 / r2) : sqrt(s2);
        result[1] = md;
        result[2] = mr > 0.0 ? md / mr : md;
        result[3] = mr;
    }
}

}  // namespace

cudaError_t launch_error_norms(const ErrNormsCall &c) {
    ErrArgs a{};
    a.x = c.x.data;
    a.r = static_cast<const double *>(c.r.data);
    a.xs0 = c.x.s[0];
    a.xs1 = c.x.s[1];
    a.rs0 = c.r.s[0];
    a.rs1 = c.r.s[1];
    a.lb0 = c.lb[0];
    a.lb1 = c.lb[1];
    a.lb2 = c.lb[2];
    a.ub0 = c.ub[0];
    a.ub1 = c.ub[1];
    a.ub2 = c.ub[2];
    a.rows = (c.ub[0] - c.lb[0]) * (c.ub[1] - c.lb[1]);
    a.units = c.units;
    a.xchunks = c.xchunks > 0 ? c.xchunks : 1;
    a.partials = c.scratch;
    a.result = c.scratch + 4 * static_cast<int64_t>(c.nblocks);
    if (c.dtype == UHS_F64) k_err_partial<double><<<c.nblocks, kErrThreads, 0, c.stream>>>(a);
    else if (c.dtype == UHS_F32) k_err_partial<float><<<c.nblocks, kErrThreads, 0, c.stream>>>(a);
    else k_err_partial<float2><<<c.nblocks, kErrThreads, 0, c.stream>>>(a);
    k_err_final<<<1, kErrThreads, 0, c.stream>>>(a.partials, c.nblocks, a.result);
    count_launch(2);
    return cudaGetLastError();
}

}  // namespace uhs

// Identity of the calling thread's current CUDA context (the device's
// primary context once the runtime has set the device), through the driver
// entry points; 0 when they are unavailable.  cudaDeviceReset destroys the
// primary context and the next runtime call creates another with a new id,
// in which the array has a new device address.
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

static unsigned long long current_context_id() {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<CtxGetCurrentFn>(p);
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(p);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Set-up, once per device and context, with that device current: the device
// address of g_noalloc_scratch (a lookup: it allocates nothing).  The
// address is kept with the id of the context it belongs to and looked up
// again when the device's context has changed (after cudaDeviceReset), or on
// every call when the context id cannot be read.  Returns nullptr (and sets
// the error) on failure.
static double *noalloc_scratch(int dev) {
    static std::mutex mu;
    static double *addr[64] = {};
    static unsigned long long ctx_of[64] = {};
    if (dev < 0 || dev >= 64) {
        uhs::set_error(UHS_EUNSUPPORTED, "device ordinal %d is beyond the 64 this library tracks", dev);
        return nullptr;
    }
    // make the device's primary context current on this thread (cudaSetDevice
    // initialises it), so the id read below is the one the launches will use
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) {
        uhs::set_error(UHS_ECUDA, "cudaSetDevice(%d): %s", dev, cudaGetErrorString(e));
        return nullptr;
    }
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev] || ctx == 0 || ctx != ctx_of[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            uhs::set_error(UHS_ECUDA, "cudaGetSymbolAddress of the reduction scratch: %s", cudaGetErrorString(e));
            return nullptr;
        }
        addr[dev] = static_cast<double *>(p);
        ctx_of[dev] = ctx;
    }
    return addr[dev];
}

extern "C" int uhs_error_norms_noalloc(const uhs_stencil_desc *d, const uhs_memref *x, const uhs_memref *ref,
                                       double out[4], void *stream) {
    uhs::ErrNormsCall c;
    bool empty = false;
    int rc = uhs::prepare_error_norms(d, x, ref, &c, &empty);
    if (rc) return rc;
    if (!out) return uhs::set_error(UHS_EINVAL, "out is NULL");
    if (empty) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return UHS_OK;
    }
    if (c.nblocks > UHS_NOALLOC_MAX_PARTIALS)  // cannot happen: err_split caps CTAs at kErrBlocks
        return uhs::set_error(UHS_EUNSUPPORTED, "the reduction needs %d partial slots; the allocation-free "
                              "scratch holds %d", c.nblocks, UHS_NOALLOC_MAX_PARTIALS);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return uhs::set_error(UHS_ECUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
    double *scratch = noalloc_scratch(dev);
    if (!scratch) return UHS_ECUDA;
    c.scratch = scratch;
    c.stream = static_cast<cudaStream_t>(stream);
    e = uhs::launch_error_norms(c);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, scratch + 4 * static_cast<int64_t>(c.nblocks), 4 * sizeof(double),
                            cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return uhs::set_error(UHS_ECUDA, "allocation-free error reduction: %s", cudaGetErrorString(e));
    return UHS_OK;
}
