// Host runtime behind the C ABI (include/uhs.h): descriptor validation, the
// pass planner and the launch sequence that replaces the reference's generated
// <name>_iteration entry.
//
// Reference behaviour mirrored here:
//  * T == 1 is a single sweep in -> out; an even T runs T/2 pairs
//    (a -> b, b -> a) and leaves the result in a
//    (UHStencil/lib/Parser/MLIRGen.cpp:317-352,
//     lib/Conversion/StencilToStandard/ConvertStencilToStandard.cpp:298-337);
//    any other T is rejected (MLIRGen.cpp:317-321).
//  * Only domain points [lb, ub) are written; the halo of both grids is read
//    as it stands (ConvertStencilToStandard.cpp:91-149, 339-381).
//  * The entry is synchronous for the caller (the MLIR CUDA runtime wrappers
//    synchronise after each launch); UHS_FLAG_NO_SYNC lifts that.
#include "stream_call.h"
#include "uhs_kernels.h"

#include <algorithm>
#include <map>
#include <memory>
#include <tuple>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace uhs {

static std::atomic<int64_t> g_launches{0};
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static std::atomic<int64_t> g_alloc_cap{0};  // 0: no cap

cudaError_t dev_alloc(void **p, size_t bytes) {
    const int64_t cap = g_alloc_cap.load(std::memory_order_relaxed);
    if (cap > 0 && static_cast<int64_t>(bytes) > cap) {
        *p = nullptr;
        return cudaErrorMemoryAllocation;
    }
    return cudaMalloc(p, bytes);
}

static thread_local std::string t_err = "no error";

int set_error(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_err = buf;
    return code;
}

// Keeps the thread's last-error message across an optional step whose
// failure the caller works around (the message then still describes the last
// call that failed).
struct ErrorMessageGuard {
    std::string saved = t_err;
    ~ErrorMessageGuard() { t_err = saved; }
};

static int cuda_error(cudaError_t e, const char *what) {
    return set_error(UHS_ECUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

// Status words (kStatusWords x unsigned, layout in uhs_kernels.h) in device
// memory, one per (device, stream), allocated at first use and kept for the
// process.  Calls on different streams (or host threads with their own streams) never
// share a word, so one call's errors and scan results cannot leak into
// another's.
unsigned *stream_error_word(int device, cudaStream_t stream) {
    static std::mutex mu;
    static std::map<std::pair<int, uintptr_t>, unsigned *> words;
    const auto key = std::make_pair(device, reinterpret_cast<uintptr_t>(stream));
    std::lock_guard<std::mutex> lk(mu);
    auto it = words.find(key);
    if (it != words.end()) return it->second;
    void *p = nullptr;
    if (dev_alloc(&p, kStatusWords * sizeof(unsigned)) != cudaSuccess) return nullptr;
    if (cudaMemset(p, 0, kStatusWords * sizeof(unsigned)) != cudaSuccess) {
        cudaFree(p);
        return nullptr;
    }
    words[key] = static_cast<unsigned *>(p);
    return static_cast<unsigned *>(p);
}

static size_t elem_bytes(int dtype) { return dtype == UHS_F32 ? 4 : 8; }

// Validate one memref against the descriptor; fill the view.
static int view_of(const uhs_stencil_desc *d, const uhs_memref *m, const char *name, GridView *v) {
    if (!m) return set_error(UHS_EINVAL, "%s: memref is NULL", name);
    if (!m->aligned) return set_error(UHS_EINVAL, "%s: aligned pointer is NULL", name);
    if (m->offset < 0) return set_error(UHS_EINVAL, "%s: negative offset %lld", name, (long long)m->offset);
    for (int i = 0; i < 3; ++i) {
        if (m->sizes[i] <= 0)
            return set_error(UHS_EINVAL, "%s: sizes[%d] = %lld must be positive", name, i, (long long)m->sizes[i]);
    }
    if (m->strides[2] != 1)
        return set_error(UHS_EUNSUPPORTED, "%s: the fastest axis must have unit stride (got %lld)", name,
                         (long long)m->strides[2]);
    if (m->strides[1] < m->sizes[2] || m->strides[0] < m->strides[1] * m->sizes[1])
        return set_error(UHS_EINVAL, "%s: strides (%lld, %lld, 1) overlap rows or planes of sizes (%lld, %lld, %lld)",
                         name, (long long)m->strides[0], (long long)m->strides[1], (long long)m->sizes[0],
                         (long long)m->sizes[1], (long long)m->sizes[2]);
    if (d->rank == 2 && m->sizes[0] != 1)
        return set_error(UHS_EINVAL, "%s: a rank-2 grid is passed with sizes[0] == 1 (got %lld)", name,
                         (long long)m->sizes[0]);
    const size_t eb = elem_bytes(d->dtype);
    char *base = static_cast<char *>(m->aligned) + (size_t)m->offset * eb;
    if (reinterpret_cast<uintptr_t>(base) % eb != 0)
        return set_error(UHS_EINVAL, "%s: element pointer is not %zu-byte aligned", name, eb);
    v->data = base;
    for (int i = 0; i < 3; ++i) {
        v->n[i] = m->sizes[i];
        v->s[i] = m->strides[i];
    }
    return UHS_OK;
}

static int validate_desc(const uhs_stencil_desc *d) {
    if (!d) return set_error(UHS_EINVAL, "descriptor is NULL");
    if (d->rank != 2 && d->rank != 3) return set_error(UHS_EINVAL, "rank must be 2 or 3 (got %d)", d->rank);
    if (d->dtype != UHS_F64 && d->dtype != UHS_F32 && d->dtype != UHS_F32X2)
        return set_error(UHS_EINVAL, "unknown dtype %d", d->dtype);
    if (d->nterms < 1 || d->nterms > UHS_MAX_TERMS)
        return set_error(UHS_EUNSUPPORTED, "nterms = %d outside [1, %d]", d->nterms, UHS_MAX_TERMS);
    if (!d->terms) return set_error(UHS_EINVAL, "terms is NULL");
    for (int k = 0; k < d->nterms; ++k) {
        const uhs_term &t = d->terms[k];
        if (std::abs(t.dz) > UHS_MAX_RADIUS || std::abs(t.dy) > UHS_MAX_RADIUS || std::abs(t.dx) > UHS_MAX_RADIUS)
            return set_error(UHS_EUNSUPPORTED, "term %d offset (%d, %d, %d) exceeds radius %d", k, t.dz, t.dy, t.dx,
                             UHS_MAX_RADIUS);
        if (d->rank == 2 && t.dz != 0)
            return set_error(UHS_EINVAL, "term %d of a rank-2 stencil has dz = %d", k, t.dz);
        if (t.param >= 0) {
            if (!d->params || t.param >= d->nparams)
                return set_error(UHS_EINVAL, "term %d uses parameter %d but %d parameters are given", k, t.param,
                                 d->params ? d->nparams : 0);
        }
    }
    if (d->rank == 2 && (d->lb[0] != 0 || d->ub[0] != 1))
        return set_error(UHS_EINVAL, "rank-2 domain must have lb[0] = 0, ub[0] = 1");
    for (int i = 0; i < 3; ++i)
        if (d->lb[i] > d->ub[i])
            return set_error(UHS_EINVAL, "domain axis %d: lb %lld > ub %lld", i, (long long)d->lb[i],
                             (long long)d->ub[i]);
    if (d->iterations < 0 || (d->iterations != 1 && d->iterations % 2 != 0))
        return set_error(UHS_EINVAL, "expect iteration num is 1 or a multiple of 2 (got %d)", d->iterations);
    return UHS_OK;
}

// Domain plus reach of the terms must stay inside the grid.
static int check_reach(const uhs_stencil_desc *d, const GridView &v) {
    if (d->lb[0] == d->ub[0] || d->lb[1] == d->ub[1] || d->lb[2] == d->ub[2]) return UHS_OK;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int k = 0; k < d->nterms; ++k) {
        const int o[3] = {d->terms[k].dz, d->terms[k].dy, d->terms[k].dx};
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], o[i]);
            hi[i] = std::max(hi[i], o[i]);
        }
    }
    for (int i = 0; i < 3; ++i) {
        if (d->lb[i] + lo[i] < 0 || d->ub[i] - 1 + hi[i] > v.n[i] - 1)
            return set_error(UHS_EINVAL,
                             "domain [%lld, %lld) on axis %d with offsets [%d, %d] reaches outside the grid extent %lld",
                             (long long)d->lb[i], (long long)d->ub[i], i, lo[i], hi[i], (long long)v.n[i]);
    }
    return UHS_OK;
}

static void make_spec(const uhs_stencil_desc *d, SweepSpec *sp) {
    std::memset(sp, 0, sizeof *sp);
    sp->rank = d->rank;
    sp->dtype = d->dtype;
    for (int i = 0; i < 3; ++i) {
        sp->lb[i] = d->lb[i];
        sp->ub[i] = d->ub[i];
    }
    sp->nterms = d->nterms;
    for (int k = 0; k < d->nterms; ++k) {
        const uhs_term &t = d->terms[k];
        sp->dz[k] = t.dz;
        sp->dy[k] = t.dy;
        sp->dx[k] = t.dx;
        sp->coef[k] = t.param >= 0 ? d->params[t.param] : t.coef;
        sp->rz = std::max(sp->rz, std::abs(t.dz));
        sp->ry = std::max(sp->ry, std::abs(t.dy));
        sp->rx = std::max(sp->rx, std::abs(t.dx));
    }
    sp->shape = kShapeGeneric;
}

// ---------------------------------------------------------------------------
// Planning: which kernel family, arithmetic, loader and tile run a sweep.
// ---------------------------------------------------------------------------
struct Plan {
    int kernel;  // UHS_KERNEL_GENERIC / UHS_KERNEL_STREAM
    LaunchCfg cfg;
    // streaming kernel
    int shape = -1, R = 0, st = 0, ar = 0, ld = kLdCpAsync, tile = 0, zchunk = 0;
    int zcap = 0;              // default launches: upper bound on the automatic z-chunk (0: none)
    int pd = 0;                // planes (rows) the streaming kernel loads ahead: built into its variant
    std::vector<double> coef;  // coef_slot order
    bool auto_df32 = false;    // df32 chosen by UHS_ARITH_AUTO, subject to range_ok()
    int pair_shift = 0;        // FP64 grids in float pairs: the pairs hold x * 2^pair_shift (range_ok)
    bool factored = false;     // separable box run as 1D passes
    bool a_tmem = false;       // tensor-core path: A operand staged in tensor memory
    bool xshuffle = false;     // rank-2 stars: x-neighbours by warp shuffles
};

int device_sm_count() {
    static std::atomic<int> cached[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return 1;
    if (dev < 64 && cached[dev].load(std::memory_order_relaxed) > 0) return cached[dev].load(std::memory_order_relaxed);
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        return 1;
    }
    if (dev < 64) cached[dev].store(sms, std::memory_order_relaxed);
    return sms;
}

static int device_sms() { return device_sm_count(); }

static int coef_slot_rt(int shape, int R, int dz, int dy, int dx) {
    const int D = 2 * R + 1;
    if (shape == kBox3) return ((dz + R) * D + (dy + R)) * D + (dx + R);
    if (shape == kBox2) return (dz + R) * D + (dx + R);
    const int axes = shape == kStar3 ? 3 : 2;
    if (dz == 0 && dy == 0 && dx == 0) return axes * 2 * R;
    int axis, d;
    if (dz != 0) {
        axis = 0;
        d = dz;
    } else if (dy != 0) {
        axis = 1;
        d = dy;
    } else {
        axis = shape == kStar3 ? 2 : 1;
        d = dx;
    }
    return axis * 2 * R + (std::abs(d) - 1) * 2 + (d > 0 ? 1 : 0);
}

static int nterms_of(int shape, int R) {
    const int D = 2 * R + 1;
    switch (shape) {
        case kStar3: return 6 * R + 1;
        case kStar2: return 4 * R + 1;
        case kBox3: return D * D * D;
        default: return D * D;
    }
}

// Star if every offset lies on an axis, box otherwise; radius 1..3.  Rank-2
// programs are streamed along y, so (dy, dx) become the kernel's (dz, dx).
// Star or box of radius R for the templated kernels.  Those kernels read
// every cell within R of the domain on every axis of the rank, so the
// program must reach exactly -R..+R on each of them: a one-sided or shorter
// reach on some axis (which check_reach would accept with a thinner halo)
// would send them outside the grid, or into cells the program never reads.
// Such programs run on the generic kernel.
static bool classify(const SweepSpec &sp, int *shape, int *R) {
    int r = 0;
    bool on_axes = true;
    int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int k = 0; k < sp.nterms; ++k) {
        const int o[3] = {sp.dz[k], sp.dy[k], sp.dx[k]};
        const int a[3] = {std::abs(o[0]), std::abs(o[1]), std::abs(o[2])};
        r = std::max({r, a[0], a[1], a[2]});
        if ((a[0] != 0) + (a[1] != 0) + (a[2] != 0) > 1) on_axes = false;
        for (int i = 0; i < 3; ++i) {
            lo[i] = std::min(lo[i], o[i]);
            hi[i] = std::max(hi[i], o[i]);
        }
    }
    if (r < 1 || r > 3) return false;
    for (int i = (sp.rank == 3 ? 0 : 1); i < 3; ++i)
        if (lo[i] != -r || hi[i] != r) return false;
    *R = r;
    if (sp.rank == 3) *shape = on_axes ? kStar3 : kBox3;
    else *shape = on_axes ? kStar2 : kBox2;
    return true;
}

// Rank-1 factorisation of a box stencil's coefficient tensor, C = a (x) b (x) c
// (rank 3) or a (x) c (rank 2; a on the streamed axis).  Exact to a few ulp
// of max |C| or rejected.  Output: [a | b | c] or [a | c].
static bool factor_box(const SweepSpec &sp, int R, std::vector<double> *out) {
    const int D = 2 * R + 1;
    const bool is2d = sp.rank == 2;
    std::vector<double> C(is2d ? D * D : D * D * D, 0.0);
    for (int k = 0; k < sp.nterms; ++k) {
        const int i = (is2d ? sp.dy[k] : sp.dz[k]) + R, j = sp.dy[k] + R, l = sp.dx[k] + R;
        C[is2d ? i * D + l : (i * D + j) * D + l] += sp.coef[k];
    }
    int piv = 0;
    for (int n = 1; n < (int)C.size(); ++n)
        if (std::fabs(C[n]) > std::fabs(C[piv])) piv = n;
    const double m = C[piv];
    if (m == 0.0) return false;
    out->clear();
    if (is2d) {
        const int i0 = piv / D, l0 = piv % D;
        for (int i = 0; i < D; ++i) out->push_back(C[i * D + l0]);
        for (int l = 0; l < D; ++l) out->push_back(C[i0 * D + l] / m);
        for (int i = 0; i < D; ++i)
            for (int l = 0; l < D; ++l)
                if (std::fabs(C[i * D + l] - (*out)[i] * (*out)[D + l]) > 1e-15 * std::fabs(m)) return false;
    } else {
        const int i0 = piv / (D * D), j0 = (piv / D) % D, l0 = piv % D;
        for (int i = 0; i < D; ++i) out->push_back(C[(i * D + j0) * D + l0]);
        for (int j = 0; j < D; ++j) out->push_back(C[(i0 * D + j) * D + l0] / m);
        for (int l = 0; l < D; ++l) out->push_back(C[(i0 * D + j0) * D + l] / m);
        for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j)
                for (int l = 0; l < D; ++l)
                    if (std::fabs(C[(i * D + j) * D + l] - (*out)[i] * (*out)[D + j] * (*out)[2 * D + l]) >
                        1e-15 * std::fabs(m))
                        return false;
    }
    return true;
}

// UHS_ARITH_AUTO after range_ok() vetoed float pairs: native arithmetic.
// The two-points-along-x tiles of rank-2 stars are built for float
// arithmetic only; native FP64 takes the 128-column one-point tile.
static void fall_back_native(Plan &pl) {
    pl.ar = kArNative;
    pl.cfg.arith = UHS_ARITH_FMA;
    if (pl.kernel == UHS_KERNEL_STREAM && pl.st == kStF64 && is_rank2_shape(pl.shape) &&
        tile_shape(true, pl.tile).vx == 2)
        pl.tile = 0;
}

static int plan_sweep(const SweepSpec &sp, const uhs_params *p, const GridView &view, Plan *pl) {
    uhs_params dflt;
    uhs_params_default(&dflt);
    if (!p) p = &dflt;
    LaunchCfg &cfg = pl->cfg;
    cfg.arith = p->arith;
    cfg.tile_x = p->tile_x;
    cfg.tile_y = p->tile_y;
    cfg.tile_z = p->tile_z;
    cfg.k_temporal = p->k_temporal > 0 ? p->k_temporal : 1;
    cfg.use_tma = p->use_tma;
    if (p->arith < UHS_ARITH_AUTO || p->arith > UHS_ARITH_DF32)
        return set_error(UHS_EINVAL, "unknown arithmetic mode %d", p->arith);
    if (p->kernel < UHS_KERNEL_AUTO || p->kernel > UHS_KERNEL_MMA)
        return set_error(UHS_EINVAL, "unknown kernel family %d", p->kernel);
    if (cfg.k_temporal != 1 && cfg.k_temporal != 2 && cfg.k_temporal != 4)
        return set_error(UHS_EUNSUPPORTED, "temporal fusion depth %d: depths 1, 2 and 4 are available", cfg.k_temporal);

    int shape = -1, R = 0;
    const bool shaped = classify(sp, &shape, &R);
    int arith = p->arith;
    pl->auto_df32 = false;
    if (arith == UHS_ARITH_AUTO) {
        if (sp.dtype == UHS_F32X2) arith = UHS_ARITH_DF32;
        else if (sp.dtype == UHS_F64 && shaped) {
            // FP64 on the streaming kernel: float pairs unless the range check
            // in range_ok() vetoes them for this run's data.
            arith = UHS_ARITH_DF32;
            pl->auto_df32 = true;
        } else arith = UHS_ARITH_FMA;
    }
    if (sp.dtype == UHS_F32 && arith == UHS_ARITH_DF32)
        return set_error(UHS_EUNSUPPORTED, "float-pair arithmetic needs F64 or F32X2 grids");
    if (sp.dtype == UHS_F32X2 && arith != UHS_ARITH_DF32)
        return set_error(UHS_EUNSUPPORTED, "F32X2 grids are swept in float-pair arithmetic only");
    cfg.arith = arith;

    int kernel = p->kernel;
    const bool stream_ok = shaped && arith != UHS_ARITH_EXACT;
    if (kernel == UHS_KERNEL_AUTO) kernel = stream_ok ? UHS_KERNEL_STREAM : UHS_KERNEL_GENERIC;
    if (kernel == UHS_KERNEL_MMA) {
        // tcgen05 kind::tf32 with split operands: FP32 3D boxes of radius 2 and 3
        if (!(sp.dtype == UHS_F32 && shaped && shape == kBox3 && (R == 2 || R == 3)))
            return set_error(UHS_EUNSUPPORTED, "the tensor-core path covers FP32 3D box stencils of radius 2 and 3");
        if (arith != UHS_ARITH_FMA)
            return set_error(UHS_EUNSUPPORTED, "the tensor-core path computes in split-tf32 FMA arithmetic");
        if (cfg.k_temporal > 1) return set_error(UHS_EUNSUPPORTED, "the tensor-core path sweeps one step per pass");
        const bool want_tmem_a = (p->flags & UHS_FLAG_MMA_TMEM_A) != 0;
        int xt = cfg.tile_x > 0 ? cfg.tile_x : (R == 2 && !want_tmem_a ? 32 : 16);
        if (!(xt == 16 || (xt == 32 && R == 2)))
            return set_error(UHS_EINVAL, "tensor-core tiles are 16 columns wide (32 for radius 2), got %d", xt);
        if (view.s[0] >= (int64_t(1) << 31) || view.n[0] >= (int64_t(1) << 31))
            return set_error(UHS_EUNSUPPORTED, "planes of 2^31 elements or more need the generic kernel");
        if (p->prefetch != 0)
            return set_error(UHS_EUNSUPPORTED, "the tensor-core kernel's load-ahead is fixed (prefetch must be 0)");
        if (cfg.use_tma > 0) return set_error(UHS_EUNSUPPORTED, "the tensor-core kernel stages planes without TMA");
        pl->kernel = cfg.kernel = UHS_KERNEL_MMA;
        cfg.tile_x = xt;
        cfg.tile_y = 128;
        cfg.use_tma = -1;
        pl->shape = shape;
        pl->R = R;
        pl->st = kStF32;
        pl->ar = kArNative;
        pl->tile = xt;
        if (want_tmem_a && xt != 16)
            return set_error(UHS_EINVAL, "the tensor-memory A operand takes 16-column tiles");
        pl->a_tmem = want_tmem_a;
        pl->coef.assign(nterms_of(shape, R), 0.0);
        for (int k = 0; k < sp.nterms; ++k) pl->coef[coef_slot_rt(shape, R, sp.dz[k], sp.dy[k], sp.dx[k])] += sp.coef[k];
        return UHS_OK;
    }
    if (kernel == UHS_KERNEL_STREAM && !stream_ok)
        return set_error(UHS_EUNSUPPORTED, "the streaming kernel covers star and box stencils of radius 1-3 in "
                                           "FMA or float-pair arithmetic");
    if (kernel == UHS_KERNEL_GENERIC) {
        if (cfg.k_temporal > 1) return set_error(UHS_EUNSUPPORTED, "the generic kernel sweeps one step per pass");
        if (arith != UHS_ARITH_FMA && arith != UHS_ARITH_EXACT)
            return set_error(UHS_EUNSUPPORTED, "the generic kernel runs FMA or EXACT arithmetic");
        const int tx = cfg.tile_x > 0 ? cfg.tile_x : 32, ty = cfg.tile_y > 0 ? cfg.tile_y : 8;
        if (tx * ty > 256) return set_error(UHS_EINVAL, "tile %d x %d exceeds 256 threads", tx, ty);
        if (tx % 32 != 0) return set_error(UHS_EINVAL, "tile_x must be a multiple of 32 (got %d)", tx);
        if (p->prefetch != 0 && p->prefetch != 1)
            return set_error(UHS_EUNSUPPORTED, "the generic kernel loads one plane ahead (prefetch 0 or 1)");
        if (cfg.use_tma > 0) return set_error(UHS_EUNSUPPORTED, "the generic kernel loads by cp.async, not TMA");
        pl->kernel = kernel;
        cfg.kernel = kernel;
        return UHS_OK;
    }
    // temporal fusion (stream_fused.cuh): star and box stencils on FP32/FP64
    // grids, depths 2 and 4 (4 in 3D for radius 1 only: deeper 3D tiles of
    // radius 2-3 do not fit shared memory)
    if (cfg.k_temporal > 1) {
        if (sp.dtype == UHS_F32X2)
            return set_error(UHS_EUNSUPPORTED, "temporal fusion covers FP32 and FP64 grids (not float-pair grids)");
        if (cfg.k_temporal == 4 && sp.rank == 3 && R > 1)
            return set_error(UHS_EUNSUPPORTED, "temporal fusion of depth 4 covers radius 1 in 3D (depth 2 for radius %d)", R);
        if (p->vx == 2) return set_error(UHS_EUNSUPPORTED, "temporal fusion takes one point per thread along x");
    }
    pl->kernel = cfg.kernel = UHS_KERNEL_STREAM;
    pl->shape = shape;
    pl->R = R;
    pl->st = sp.dtype == UHS_F64 ? kStF64 : sp.dtype == UHS_F32 ? kStF32 : kStF32x2;
    pl->ar = arith == UHS_ARITH_DF32 ? kArDf32 : kArNative;
    const bool is2d = sp.rank == 2;
    // separable boxes run as 1D passes unless the caller opts out
    std::vector<double> fac;
    // (fused passes sum boxes term by term)
    const bool sep = (shape == kBox3 || shape == kBox2) && !(p->flags & UHS_FLAG_NO_FACTOR) && cfg.k_temporal <= 1 &&
                     factor_box(sp, R, &fac);
    // whether the grid allows TMA loads: 16-byte aligned base, row and plane pitches
    const int eb = sp.dtype == UHS_F32 ? 4 : 8;
    const int64_t row_b = view.s[1] * eb, plane_b = (is2d ? view.s[1] : view.s[0]) * eb;
    const bool tma_aligned = !(reinterpret_cast<uintptr_t>(view.data) % 16 || row_b % 16 || plane_b % 16);
    // tile variant from (tile_x, tile_y, vy, vx)
    int tile = 0;
    pl->zcap = 0;
    if (p->vx < 0 || p->vx > 2 || (p->vx == 2 && !is2d))
        return set_error(UHS_EUNSUPPORTED, "points per thread along x: 1, or 2 for rank-2 stars (got %d)", p->vx);
    if (is2d && p->vx == 2) {
        // two points per thread along x: tile 3 (64 threads, 128 columns) or 4 (128 threads, 256)
        const bool f32 = sp.dtype == UHS_F32 && arith == UHS_ARITH_FMA;
        if (shape != kStar2 || !(f32 || arith == UHS_ARITH_DF32))
            return set_error(UHS_EUNSUPPORTED, "two points per thread along x: rank-2 stars on FP32 grids or in "
                                               "float pairs");
        if (cfg.tile_x == 128) tile = 3;
        else if (cfg.tile_x == 0 || cfg.tile_x == 256) tile = 4;
        else return set_error(UHS_EINVAL, "two points per thread along x: tiles are 128 or 256 wide (got %d)", cfg.tile_x);
    } else if (is2d) {
        if (cfg.tile_x == 64) tile = 1;
        else if (cfg.tile_x == 256) tile = 2;
        else if (cfg.tile_x != 0 && cfg.tile_x != 128)
            return set_error(UHS_EINVAL, "rank-2 streaming tiles are 64, 128 or 256 wide (got %d)", cfg.tile_x);
        // FP32 rows: 256-wide strips (cp.async), 2-30 % over 128 on the
        // twelve reference shapes at 8192^2; float pairs keep 128
        if (cfg.tile_x == 0 && sp.dtype == UHS_F32 && arith != UHS_ARITH_DF32) tile = 2;
        // Stars, two points per thread along x (vx 0 = planner's choice),
        // GStencil/s per sweep at 8192^2 against the one-point default: in
        // float pairs (packed sums) 128 columns by TMA, r1/r2/r3 366/253/184
        // vs 310/214/163, or 256 by cp.async where TMA cannot load the grid
        // (358/242/177); FP32 radius 2 by TMA 622 vs 581 (radius 1 even, 3
        // slower).
        if (cfg.tile_x == 0 && p->vx == 0 && shape == kStar2 && !(p->flags & UHS_FLAG_XSHUFFLE)) {
            const bool tma = tma_aligned && cfg.use_tma >= 0;
            // (FP64 grids swept in place, bounded sums, at 8192^2: 256 columns
            // by cp.async 229 / 194 GStencil/s for r1 / r2 against 217 / 190
            // at 128 by TMA; radius 3 one point per thread, 129 vs 122)
            if (arith == UHS_ARITH_DF32) {
                if (sp.dtype == UHS_F32X2 || cfg.use_tma > 0) tile = tma ? 3 : 4;
                else tile = R == 3 ? 2 : 4;
            }
            else if (sp.dtype == UHS_F32 && R == 2 && tma) tile = 3;
        }
    } else if (cfg.tile_x == 0 && cfg.tile_y == 0 && p->vy == 0) {
        // Defaults from planner-against-exhaustive-tuning runs on GB300 at
        // 512^3 (studies.py shapes, reference and random coefficients).
        // Tiles: 0 = 32 x 32 points, 4 per thread along y; 1 = 32 x 16, 4 per
        // thread; 2 = 64 x 8, 2 per thread (big boxes, r2-3 term by term,
        // have one fixed tile).  GStencil/s new vs old default, z-chunk caps
        // (below) included.
        if (arith == UHS_ARITH_DF32) {
            // with packed sums (stream_kernel.cuh PACKED), GStencil/s per
            // sweep at 512^3: float-pair grids of a 3d1r star 341 at 32 x 16
            // (4 per thread) vs 311 at 64 x 8 (FP64 grids swept in place:
            // 189 vs 191); 3d2r/3d3r stars 186/134 vs 181/127 at 64 x 8;
            // separable boxes r1/r2/r3 235/125/79 (FP64 in place 163/102/68)
            // vs 231/122/76 (162/98/60) at 32 x 32
            // (with bounded sums FP64 grids swept in place prefer it too:
            // 3d1r star 190 vs 177 GStencil/s at 64 x 8)
            if (shape == kStar3) tile = 1;
            else tile = 1;  // separable and term-by-term boxes (3d1r box 81.6 vs 75.9 at 32 x 32)
        } else if (sp.dtype == UHS_F32) {
            // 3d1r/2r/3r 632/659/438 vs 596/625/410; 32-row tiles for r2 only
            // when they do not leave more than 2 % of the rows idle (a
            // 194 x 294 x 343 grid: 32 x 16 is 1.15x faster)
            const int64_t ny = sp.ub[1] - sp.lb[1];
            const bool rows32 = ((ny + 31) / 32) * 32 <= ny + ny / 50;
            if (shape == kStar3) tile = (R == 2 && rows32) ? 0 : 1;
            else if (sep) tile = 1;                      // 3d1r/2r/3r 626/563/297 vs 588/548/270 at 32 x 32
        }  // non-separable FP32 boxes and native FP64 keep tile 0
    } else {
        if (cfg.tile_x == 64) tile = 2;
        else if (cfg.tile_x != 0 && cfg.tile_x != 32)
            return set_error(UHS_EINVAL, "rank-3 streaming tiles are 32 or 64 wide (got %d)", cfg.tile_x);
        else if (cfg.tile_y == 16) tile = p->vy == 2 ? 3 : 1;
        else if (p->vy == 2) tile = 3;
        else if (p->vy == 8) {
            if (!(sp.dtype == UHS_F32 && shape == kStar3))
                return set_error(UHS_EUNSUPPORTED, "8 points per thread along y: FP32 3D stars only");
            tile = 4;
        }
    }
    // Lane-shuffle variant (UHS_FLAG_XSHUFFLE): rank-2 stars, built for the
    // default strips of FP32 grids (256 wide) and float-pair grids (128)
    pl->xshuffle = false;
    // (FP64 grids in float pairs: the flag applies to the sweeps of their
    // pair-resident runs, on float-pair grids)
    const bool xs_pairs_later = sp.dtype == UHS_F64 && arith == UHS_ARITH_DF32 && is2d && shape == kStar2;
    if ((p->flags & UHS_FLAG_XSHUFFLE) && !xs_pairs_later) {
        const bool f32 = sp.dtype == UHS_F32 && arith == UHS_ARITH_FMA, f32x2 = sp.dtype == UHS_F32X2;
        if (!(is2d && shape == kStar2 && (f32 || f32x2)))
            return set_error(UHS_EUNSUPPORTED, "lane shuffles cover rank-2 stars on FP32 or float-pair grids");
        if (p->vx == 2) return set_error(UHS_EUNSUPPORTED, "lane shuffles take one point per thread along x");
        const int want = f32 ? 2 : 0;
        if (cfg.tile_x != 0 && tile != want)
            return set_error(UHS_EUNSUPPORTED, "lane shuffles run %d-wide strips on this element type", f32 ? 256 : 128);
        tile = want;
        pl->xshuffle = true;
    }
    pl->tile = tile;
    // Load-ahead depth: built into each variant (2D strips 4 rows; 3D 3
    // planes, 2 for radius 2-3 boxes swept term by term; temporal fusion 2).
    // A caller may state it, not choose another.
    pl->pd = cfg.k_temporal > 1 ? 2 : is2d ? 4 : (shape == kBox3 && R >= 2 && !sep) ? 2 : 3;
    if (p->prefetch != 0 && p->prefetch != pl->pd)
        return set_error(UHS_EUNSUPPORTED, "this streaming variant loads %d %s ahead (prefetch %d)", pl->pd,
                         is2d ? "rows" : "planes", p->prefetch);
    // Upper bound on the automatic z-chunk (about four waves of CTAs) for 3D
    // sweeps: shorter chunks measured faster in these classes (FP32 3d1r
    // star 632 vs 596 GStencil/s at 16 planes; float-pair 3d3r box 6.8 vs
    // 6.3 at 16; float-pair 3d2r star 118.4 vs 114.7 at 64).  A caller's
    // tile_z overrides it.
    if (!is2d) {
        const bool df = arith == UHS_ARITH_DF32, f32 = sp.dtype == UHS_F32 && !df;
        // (float-pair 3d1r star with bounded sums: 374 vs 363 GStencil/s at 16 planes)
        // (FP64 grids swept in place: 64 planes)
        if (shape == kStar3) pl->zcap = df ? ((R >= 2 || sp.dtype == UHS_F64) ? 64 : 16) : f32 ? (R == 3 ? 64 : 16) : 0;
        else if (sep) pl->zcap = (df || f32) ? (R >= 2 ? 64 : f32 ? 16 : 0) : 0;
        else pl->zcap = df ? (R >= 2 ? 16 : 64) : f32 ? (R >= 2 ? 64 : 0) : 0;
    }
    // the kernel keeps in-plane offsets in 32 bits
    const int64_t plane_elems = is2d ? view.s[1] : view.s[0];
    if (plane_elems >= (int64_t(1) << 31) || view.n[2] >= (int64_t(1) << 31)) {
        if (p->kernel == UHS_KERNEL_STREAM)
            return set_error(UHS_EUNSUPPORTED, "planes of 2^31 elements or more need the generic kernel");
        pl->kernel = cfg.kernel = UHS_KERNEL_GENERIC;
        if (arith != UHS_ARITH_FMA && arith != UHS_ARITH_EXACT)
            return set_error(UHS_EUNSUPPORTED, "planes of 2^31 elements or more run FMA or EXACT arithmetic only");
        return UHS_OK;
    }
    // loader
    bool tma_ok = cfg.use_tma >= 0 && !(is2d && (tile == 2 || tile == 4));
    // float-pair 2D boxes term by term load faster by cp.async (2d2r box at
    // 8192^2: 71.8 vs 65.6 GStencil/s with TMA)
    if (cfg.use_tma == 0 && is2d && shape == kBox2 && !sep && arith == UHS_ARITH_DF32) tma_ok = false;
    if (!tma_aligned) tma_ok = false;
    if (cfg.use_tma > 0 && is2d && (tile == 2 || tile == 4))
        return set_error(UHS_EUNSUPPORTED, "256-column rank-2 tiles load by cp.async (a TMA box is at most 256 wide)");
    if (cfg.use_tma > 0 && !tma_ok)
        return set_error(UHS_EUNSUPPORTED, "TMA needs 16-byte aligned grids and row/plane strides");
    pl->ld = tma_ok ? kLdTma : kLdCpAsync;
    if (sep) {
        pl->shape = shape = (shape == kBox3) ? kSep3 : kSep2;
        pl->coef = fac;
        pl->factored = true;
        return UHS_OK;
    }
    // coefficients in slot order
    pl->coef.assign(nterms_of(shape, R), 0.0);
    for (int k = 0; k < sp.nterms; ++k) {
        const int dz = is2d ? sp.dy[k] : sp.dz[k], dy = is2d ? 0 : sp.dy[k];
        pl->coef[coef_slot_rt(shape, R, dz, dy, sp.dx[k])] += sp.coef[k];
    }
    return UHS_OK;
}

// ---- TMA tensor maps (encoded through the driver entry point) -------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(ptr);
    });
    return fn;
}

// Map of the kernel-frame view (z, y, x) with box {W, H, 1}.
static bool make_tmap(const GridView &v, int eb, int W, int H, CUtensorMap *m) {
    static std::mutex mu;
    static std::map<std::tuple<uintptr_t, int64_t, int64_t, int64_t, int64_t, int64_t, int, int, int>, CUtensorMap>
        cache;
    const auto key = std::make_tuple(reinterpret_cast<uintptr_t>(v.data), v.n[0], v.n[1], v.n[2], v.s[0], v.s[1],
                                     eb, W, H);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
        *m = it->second;
        return true;
    }
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {static_cast<cuuint64_t>(v.n[2]), static_cast<cuuint64_t>(v.n[1]),
                                static_cast<cuuint64_t>(v.n[0])};
    const cuuint64_t strides[2] = {static_cast<cuuint64_t>(v.s[1] * eb), static_cast<cuuint64_t>(v.s[0] * eb)};
    const cuuint32_t box[3] = {static_cast<cuuint32_t>(W), static_cast<cuuint32_t>(H), 1};
    const cuuint32_t es[3] = {1, 1, 1};
    CUresult r = fn(m, eb == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, v.data, dims,
                    strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return false;
    if (cache.size() > 256) cache.clear();
    cache[key] = *m;
    return true;
}

static cudaError_t stream_dispatch(const StreamCall &c) {
    const bool is2d = is_rank2_shape(c.shape);
    if (c.st == kStF64 && c.ar == kArNative) return is2d ? launch_stream_f64n_2d(c) : launch_stream_f64n_3d(c);
    if (c.st == kStF64) return is2d ? launch_stream_f64df_2d(c) : launch_stream_f64df_3d(c);
    if (c.st == kStF32) return is2d ? launch_stream_f32_2d(c) : launch_stream_f32_3d(c);
    return is2d ? launch_stream_f32x2_2d(c) : launch_stream_f32x2_3d(c);
}

// Kernel-frame view: rank-2 grids (1, Y, X) stream along Y -> (Y, 1, X).
static GridView kernel_view(const SweepSpec &sp, const GridView &v) {
    if (sp.rank == 3) return v;
    GridView k = v;
    k.n[0] = v.n[1];
    k.n[1] = 1;
    k.s[0] = v.s[1];
    k.s[1] = v.s[1];
    return k;
}

// UHS_ARITH_AUTO on FP64 grids.  A float pair holds a value to 2^-48 of
// itself between 2^-74 and 2^128 (df32.cuh), and a run may keep every value
// scaled by 2^s, which moves that window anywhere in the FP64 range (a linear
// sweep commutes with the scale exactly).  Scan both grids (their whole
// spans, halo included) for their exponent range and keep float pairs only
// when
//   * no cell holds Inf or NaN;
//   * with s chosen so that the largest magnitude grown by (sum |c|)^T over
//     the run stays below 2^120 (8 binades under the float range), every
//     nonzero magnitude, scaled, is at least 2^(-74 + kPairLowMargin): each
//     input value splits exactly to 48 bits, and values the run brings down
//     by up to 2^kPairLowMargin still do.
// Otherwise the run computes in native FP64.  A field spanning more than
// about 2^169 between its largest (grown) and smallest nonzero magnitudes is
// the case left to native arithmetic: in float pairs its small cells would
// keep 24 bits or flush to zero, which a max-normalised error would not show.
constexpr int kPairLowMargin = 24;
static bool range_ok(const SweepSpec &sp, const GridView &a, const GridView &b, int T, cudaStream_t st,
                     int *shift) {
    *shift = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    unsigned *w = stream_error_word(dev, st);
    if (!w) return false;
    unsigned *emax = w + 1, *emin = w + 8;
    if (cudaMemsetAsync(emax, 0, sizeof(unsigned), st) != cudaSuccess) return false;
    if (cudaMemsetAsync(emin, 0xff, sizeof(unsigned), st) != cudaSuccess) return false;
    for (const GridView *g : {&a, &b}) {
        const int64_t span = (g->n[0] - 1) * g->s[0] + (g->n[1] - 1) * g->s[1] + g->n[2];
        if (launch_exponent_range(g->data, span, emax, emin, device_sms(), st) != cudaSuccess) return false;
    }
    unsigned e[2] = {0u, 0u};
    if (cudaMemcpyAsync(&e[0], emax, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess) return false;
    if (cudaMemcpyAsync(&e[1], emin, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess) return false;
    if (cudaStreamSynchronize(st) != cudaSuccess) return false;
    if (e[0] >= 0x7ffu) return false;  // Inf or NaN somewhere
    if (e[1] == 0xffffffffu) return true;  // every cell zero
    double csum = 0.0;
    for (int k = 0; k < sp.nterms; ++k) csum += std::fabs(sp.coef[k]);
    const double growth = csum > 1.0 ? std::max(T, 1) * std::log2(csum) : 0.0;
    // log2 bound of every magnitude during the run, and the largest scale
    // that keeps it below 2^120 (kept within +-800 so scaled exponents and
    // their joins stay inside the FP64 range)
    const double top = static_cast<double>(static_cast<int>(e[0]) - 1023) + 1.0 + growth;
    const double sd = std::floor(119.0 - top);
    if (!(sd >= -800.0)) return false;
    const int sh = static_cast<int>(std::min(sd, 800.0));
    if (static_cast<int>(e[1]) - 1023 + sh < -74 + kPairLowMargin) return false;
    *shift = sh;
    return true;
}

// CTAs per SM of a streaming launch's kernel variant (1 when the query fails;
// its error is cleared so the launch does not report it).
static int stream_occupancy(const StreamCall &c) {
    int occ = 0;
    StreamCall q = c;
    q.occ_out = &occ;
    if (stream_dispatch(q) != cudaSuccess || occ <= 0) {
        cudaGetLastError();
        occ = 1;
    }
    return occ;
}

// z-chunk of a streaming launch: the caller's tile_z, else enough CTAs for
// about four waves over the SMs, at most the planner's cap; at least 32 rows
// for rank-2 strips (2048^2 to 4096^2 FP32 5-point: 340 / 507 GStencil/s at
// 32 rows against 291 / 454 at the 8 rows four waves would give).  *occ_out,
// when given, receives the variant's CTAs per SM.
static int stream_zchunk(const SweepSpec &sp, const Plan &pl, const StreamCall &c, int *occ_out) {
    int bx, by;
    stream_tile_xy(c, &bx, &by);
    const int64_t nz = c.ub[0] - c.lb[0];
    const int64_t tiles = ((c.ub[2] - c.lb[2] + bx - 1) / bx) * ((c.ub[1] - c.lb[1] + by - 1) / by);
    int zchunk = pl.cfg.tile_z;
    int occ = 0;
    if (occ_out || (zchunk <= 0 && nz > 0 && tiles > 0)) occ = stream_occupancy(c);
    if (zchunk <= 0 && nz > 0 && tiles > 0) {
        const int64_t slots = static_cast<int64_t>(device_sms()) * occ;
        const int64_t want = slots * 4;
        const int64_t chunks = std::max<int64_t>(1, (want + tiles - 1) / tiles);
        int floor_z = std::max(sp.rank == 2 ? 32 : 8, 4 * c.R);
        // Float-pair rank-2 strips: 16-row chunks where those still make two
        // waves (GStencil/s per sweep, 2d1r float pairs at 4096^2: 319 at 16
        // rows vs 279 at 32, whose 1.1 waves leave most SMs idle in the
        // second; at 3072^2, where 16 rows give 1.3 waves, 32 rows stay
        // faster, 281 vs 239)
        if (sp.rank == 2 && c.ar == kArDf32 && tiles * ((nz + 15) / 16) >= 2 * slots)
            floor_z = std::max(16, 4 * c.R);
        zchunk = static_cast<int>(std::max<int64_t>(floor_z, (nz + chunks - 1) / chunks));
        if (pl.zcap > 0) zchunk = std::min(zchunk, std::max(pl.zcap, floor_z));
    }
    if (occ_out) *occ_out = occ;
    return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(zchunk > 0 ? zchunk : 1, std::max<int64_t>(nz, 1))));
}

// The launch-frame description of a streaming sweep (no grids or stream).
static StreamCall stream_call_of(const SweepSpec &sp, const Plan &pl) {
    StreamCall c{};
    c.xshuffle = pl.xshuffle ? 1 : 0;
    c.shape = pl.shape;
    c.R = pl.R;
    c.st = pl.st;
    c.ar = pl.ar;
    c.ld = pl.ld;
    c.tile = pl.tile;
    c.coef = pl.coef.data();
    const bool is2d = sp.rank == 2;
    c.lb[0] = is2d ? sp.lb[1] : sp.lb[0];
    c.ub[0] = is2d ? sp.ub[1] : sp.ub[0];
    c.lb[1] = is2d ? 0 : sp.lb[1];
    c.ub[1] = is2d ? 1 : sp.ub[1];
    c.lb[2] = sp.lb[2];
    c.ub[2] = sp.ub[2];
    return c;
}

static int launch_sweep(const SweepSpec &sp, const Plan &pl, const GridView &in, const GridView &out,
                        cudaStream_t st, unsigned *err_word = nullptr) {
    if (pl.kernel == UHS_KERNEL_GENERIC) {
        cudaError_t e = launch_generic(sp, pl.cfg, in, out, st);
        if (e != cudaSuccess) return cuda_error(e, "generic sweep launch");
        return UHS_OK;
    }
    if (pl.kernel == UHS_KERNEL_MMA) {
        MmaCall m{};
        m.in = in;
        m.out = out;
        for (int i = 0; i < 3; ++i) {
            m.lb[i] = sp.lb[i];
            m.ub[i] = sp.ub[i];
        }
        m.R = pl.R;
        m.xtile = pl.tile;
        m.a_tmem = pl.a_tmem ? 1 : 0;
        m.coef = pl.coef.data();
        m.stream = st;
        int dev = 0;
        cudaGetDevice(&dev);
        m.err = stream_error_word(dev, st);
        if (!m.err) return set_error(UHS_ENOMEM, "device error word allocation failed");
        cudaError_t e = launch_box_mma(m);
        if (e != cudaSuccess) return cuda_error(e, "tensor-core box sweep launch");
        return UHS_OK;
    }
    StreamCall c{};
    c.shape = pl.shape;
    c.R = pl.R;
    c.st = pl.st;
    c.ar = pl.ar;
    c.ld = pl.ld;
    c.tile = pl.tile;
    c.coef = pl.coef.data();
    c.in = kernel_view(sp, in);
    c.out = kernel_view(sp, out);
    const bool is2d = sp.rank == 2;
    c.lb[0] = is2d ? sp.lb[1] : sp.lb[0];
    c.ub[0] = is2d ? sp.ub[1] : sp.ub[0];
    c.lb[1] = is2d ? 0 : sp.lb[1];
    c.ub[1] = is2d ? 1 : sp.ub[1];
    c.lb[2] = sp.lb[2];
    c.ub[2] = sp.ub[2];
    c.stream = st;
    int dev = 0;
    cudaGetDevice(&dev);
    c.err = err_word ? err_word : stream_error_word(dev, st);
    c.pair_shift = pl.pair_shift;
    c.xshuffle = pl.xshuffle ? 1 : 0;
    if (!c.err) return set_error(UHS_ENOMEM, "device error word allocation failed");
    const int eb = sp.dtype == UHS_F32 ? 4 : 8;
    // two points per thread along x: start the tiles on an even element of
    // the output's first row (vector stores of each thread's pair)
    c.xoff = 0;
    if (is2d && tile_shape(true, c.tile).vx == 2) {
        const int64_t e0 = static_cast<int64_t>(reinterpret_cast<uintptr_t>(c.out.data) / eb) + c.lb[0] * c.out.s[0] +
                           c.lb[2];
        c.xoff = static_cast<int>(e0 & 1);
    }
    const int64_t tile_x0 = c.lb[2] - c.xoff;  // first column of the first tile
    CUtensorMap tmap;
    if (c.ld == kLdTma) {
        int W, H;
        stream_box(c, eb, &W, &H);
        if (make_tmap(c.in, eb, W, H, &tmap)) {
            c.tmap = &tmap;
            const int q = 16 / eb;
            c.shift = static_cast<int>(((tile_x0 - c.R) % q + q) % q);
        } else {
            c.ld = kLdCpAsync;
        }
    }
    c.zchunk = stream_zchunk(sp, pl, c, nullptr);
    // 4-byte grids: copy in 8-byte pairs when every row start of the tile is 8-byte aligned
    if (eb == 4 && c.ld == kLdCpAsync) {
        const bool even = ((tile_x0 - c.R) % 2 == 0) && c.in.s[0] % 2 == 0 && c.in.s[1] % 2 == 0 &&
                          c.in.n[2] % 2 == 0 && reinterpret_cast<uintptr_t>(c.in.data) % 8 == 0;
        c.pair_loads = even ? 1 : 0;
    }
    cudaError_t e = stream_dispatch(c);
    if (e != cudaSuccess) return cuda_error(e, "streaming sweep launch");
    return UHS_OK;
}

// Pass depths for T steps with fusion depth k (1, 2 or 4).  Passes alternate
// a -> b, b -> a, so an even pass count leaves step T in a; the last pass is a
// single step so b ends holding step T-1, as the reference's ping-pong does.
static std::vector<int> plan_passes(int T, int k) {
    std::vector<int> out;
    if (T <= 0) return out;
    if (T == 1 || k <= 1) return std::vector<int>(static_cast<size_t>(T), 1);
    const int rest = T - 1;  // steps before the final single-step pass (odd count of passes)
    int best_n = -1, b4 = 0, b2 = 0, b1 = 0;
    for (int n4 = (k >= 4 ? rest / 4 : 0); n4 >= 0; --n4) {
        for (int n2 = (rest - 4 * n4) / 2; n2 >= 0; --n2) {
            const int n1 = rest - 4 * n4 - 2 * n2;
            const int n = n4 + n2 + n1;
            if (n % 2 == 1 && (best_n < 0 || n < best_n)) {
                best_n = n;
                b4 = n4;
                b2 = n2;
                b1 = n1;
            }
        }
    }
    out.insert(out.end(), static_cast<size_t>(b4), 4);
    out.insert(out.end(), static_cast<size_t>(b2), 2);
    out.insert(out.end(), static_cast<size_t>(b1), 1);
    out.push_back(1);
    return out;
}

// Device check that both grids hold byte-identical cells outside the domain.
static int halos_equal(const SweepSpec &sp, const GridView &a, const GridView &b, cudaStream_t st, bool *eq) {
    int dev = 0;
    cudaGetDevice(&dev);
    unsigned *w = stream_error_word(dev, st);
    if (!w) return set_error(UHS_ENOMEM, "device status word allocation failed");
    unsigned *cnt = w + 1;
    cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(unsigned), st);
    const int eb = sp.dtype == UHS_F32 ? 4 : 8;
    if (e == cudaSuccess) e = launch_halo_diff(a, b, eb, sp.lb, sp.ub, cnt, device_sms(), st);
    unsigned h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, cnt, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "halo comparison");
    *eq = h == 0;
    return UHS_OK;
}

static int launch_fused_pass(const SweepSpec &sp, const Plan &pl, const GridView &in, const GridView &out, int K,
                             cudaStream_t st) {
    StreamCall c{};
    c.shape = pl.shape;
    c.R = pl.R;
    c.st = pl.st;
    c.ar = pl.ar;
    c.coef = pl.coef.data();
    // the kernel's (z, y, x) frame: rank-2 rows stream as planes
    const bool is2d = sp.rank == 2;
    c.in = kernel_view(sp, in);
    c.out = kernel_view(sp, out);
    c.lb[0] = is2d ? sp.lb[1] : sp.lb[0];
    c.ub[0] = is2d ? sp.ub[1] : sp.ub[0];
    c.lb[1] = is2d ? 0 : sp.lb[1];
    c.ub[1] = is2d ? 1 : sp.ub[1];
    c.lb[2] = sp.lb[2];
    c.ub[2] = sp.ub[2];
    c.stream = st;
    int dev = 0;
    cudaGetDevice(&dev);
    c.err = stream_error_word(dev, st);
    if (!c.err) return set_error(UHS_ENOMEM, "device error word allocation failed");
    c.pair_shift = pl.pair_shift;
    // output tile of the fused kernel: 256 - 2KR columns of a row (2D),
    // 32 x 16 (radius 1) or 32 x 8 cells (3D)
    const int bx = is2d ? 256 - 2 * K * pl.R : 32, by = is2d ? 1 : (pl.R >= 2 ? 8 : 16);
    const int64_t nz = c.ub[0] - c.lb[0];
    const int64_t tiles = ((c.ub[2] - c.lb[2] + bx - 1) / bx) * ((c.ub[1] - c.lb[1] + by - 1) / by);
    int zchunk = pl.cfg.tile_z;
    if (zchunk <= 0 && nz > 0 && tiles > 0) {
        int occ = 0;
        StreamCall q = c;
        q.occ_out = &occ;
        if (launch_fused(q, K) != cudaSuccess || occ <= 0) occ = 1;
        const int64_t want = static_cast<int64_t>(device_sms()) * occ * 3;
        const int64_t chunks = std::max<int64_t>(1, (want + tiles - 1) / tiles);
        zchunk = static_cast<int>(std::max<int64_t>(8 * K * pl.R, (nz + chunks - 1) / chunks));
    }
    c.zchunk = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(zchunk, std::max<int64_t>(nz, 1))));
    cudaError_t e = launch_fused(c, K);
    if (e != cudaSuccess) return cuda_error(e, "fused sweep launch");
    return UHS_OK;
}

// Read and clear the device error word after the stream drained.
static int check_status_word(unsigned *w, cudaStream_t st) {
    if (!w) return UHS_OK;
    unsigned h[8] = {};
    cudaError_t e = cudaMemcpyAsync(h, w, sizeof h, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "device status read");
    if (!h[0]) return UHS_OK;
    cudaMemsetAsync(w, 0, sizeof h, st);
    cudaStreamSynchronize(st);
    if (h[0] & kDevErrTimeout)
        return set_error(UHS_ETIMEOUT,
                         "a kernel's bounded wait for its plane loads ran out (block %u,%u, plane %u, slot %u, "
                         "phase %u)",
                         h[3], h[4], h[5], h[6], h[7]);
    return set_error(UHS_ERANGE, "a grid value is outside the float-pair range [2^-126, 2^128); "
                                 "run this grid with UHS_ARITH_FMA");
}

static int check_device_errors(cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    return check_status_word(stream_error_word(dev, st), st);
}

static int finish(const uhs_params *p, cudaStream_t st) {
    if (p && (p->flags & UHS_FLAG_NO_SYNC)) return UHS_OK;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "stream synchronise");
    return check_device_errors(st);
}

static int prepare(const uhs_stencil_desc *d, const uhs_memref *a, const uhs_memref *b, GridView *va,
                   GridView *vb) {
    int rc = validate_desc(d);
    if (rc) return rc;
    if ((rc = view_of(d, a, "a", va))) return rc;
    if ((rc = view_of(d, b, "b", vb))) return rc;
    for (int i = 0; i < 3; ++i)
        if (va->n[i] != vb->n[i])
            return set_error(UHS_EINVAL, "a and b differ in sizes[%d] (%lld vs %lld)", i, (long long)va->n[i],
                             (long long)vb->n[i]);
    if (va->data == vb->data) return set_error(UHS_EINVAL, "a and b are the same grid");
    // The sweeps read one grid while writing the other: their address spans
    // must not intersect (a grid's span runs from its first to its last cell).
    {
        const auto span_end = [&](const GridView &v) {
            return reinterpret_cast<uintptr_t>(v.data) +
                   static_cast<uintptr_t>(((v.n[0] - 1) * v.s[0] + (v.n[1] - 1) * v.s[1] + v.n[2]) *
                                          static_cast<int64_t>(elem_bytes(d->dtype)));
        };
        const uintptr_t a0 = reinterpret_cast<uintptr_t>(va->data), b0 = reinterpret_cast<uintptr_t>(vb->data);
        if (a0 < span_end(*vb) && b0 < span_end(*va))
            return set_error(UHS_EINVAL, "a and b overlap in memory");
    }
    return check_reach(d, *va);
}

// Validation and launch description shared by error-reduction entry points
// that bring their own scratch (the caller fills c->scratch and c->stream).
int prepare_error_norms(const uhs_stencil_desc *d, const uhs_memref *x, const uhs_memref *ref, ErrNormsCall *c,
                        bool *empty) {
    int rc = validate_desc(d);
    if (rc) return rc;
    GridView vx, vr;
    if ((rc = view_of(d, x, "x", &vx))) return rc;
    uhs_stencil_desc d64 = *d;
    d64.dtype = UHS_F64;
    if ((rc = view_of(&d64, ref, "ref", &vr))) return rc;
    for (int i = 0; i < 3; ++i) {
        if (vx.n[i] != vr.n[i])
            return set_error(UHS_EINVAL, "x and ref differ in sizes[%d] (%lld vs %lld)", i, (long long)vx.n[i],
                             (long long)vr.n[i]);
        if (d->lb[i] < 0 || d->ub[i] > vx.n[i])
            return set_error(UHS_EINVAL, "domain axis %d [%lld, %lld) lies outside the grid", i, (long long)d->lb[i],
                             (long long)d->ub[i]);
    }
    const int64_t rows = (d->ub[0] - d->lb[0]) * (d->ub[1] - d->lb[1]);
    *empty = rows <= 0 || d->ub[2] <= d->lb[2];
    std::memset(c, 0, sizeof *c);
    c->dtype = d->dtype;
    c->x = vx;
    c->r = vr;
    for (int i = 0; i < 3; ++i) {
        c->lb[i] = d->lb[i];
        c->ub[i] = d->ub[i];
    }
    if (!*empty) err_split(rows, d->ub[2] - d->lb[2], &c->units, &c->xchunks, &c->nblocks);
    return UHS_OK;
}


// ---------------------------------------------------------------------------
// Batches (stream_batch.cu): one persistent launch per timestep, replayed
// from a CUDA graph.
// ---------------------------------------------------------------------------
struct BatchGridHost {
    int pack, kind, T, order;
    int bx, by, zc;    // item tile and z-chunk
    int64_t items;
    double item_cost;  // estimated cost of one item, for the list order
};

// Relative cost of one work item: points per item x (per-point overhead +
// terms x per-term cost of the arithmetic).  Per-term costs follow the
// measured rates of the streaming kernels (FP32 FFMA 1, float pairs about
// 6 FP32 operations' worth, native FP64 bound by the FP64 pipe).
static double batch_item_cost(int bx, int by, int zc, int nterms, int st, int ar) {
    const double per_term = st == kStF32 ? 1.0 : ar == kArDf32 ? 6.0 : 14.0;
    return static_cast<double>(bx) * by * zc * (20.0 + per_term * nterms);
}

// Grids of at least kSoloPoints interior points run in a batch as their own
// sweep launches -- the standalone plan: tuner-database or default tile,
// separable passes for rank-1 boxes -- in up to kSoloBranches parallel
// branches of the batch's graph, beside the persistent kernel that takes the
// smaller grids.  On the 64-grid mixed suite (2D sides 256-8192, 3D 64-512)
// that runs 42 grids solo: 143.9 ms per replay, against 188 ms for the
// persistent kernel alone and 164 ms for the grids launched one after
// another.  Thresholds 2^20 / 2^22 / 2^23 gave 144.4 / 149.9 / 155.2 ms;
// two branches 147.5 ms, eight 144.3 ms.
constexpr int64_t kSoloPoints = int64_t(1) << 21;
constexpr int kSoloBranches = 4;
// Float-pair FP64 programs that run pair-resident (uhs_run in uhs.h; the
// batches' solo grids): T >= kPairMinT sweeps on the streaming kernel.  The
// conversions cost a fixed ~1.8 ms per 512^3 grid pair (two splits, two
// joins, two range scans), and a float-pair sweep saves the split of every
// loaded value: GB300 at 512^3, T = 10, in place -> pair-resident, ms:
// 3d7pt 7.42 -> 5.82, 3d13pt 10.69 -> 9.10, 3d19pt 14.23 -> ~11.9 (sweeps
// 10.05 + conversions), 3d27pt box 16.15 -> ~15.2.  Below T = 8 the
// conversions would cost more than they save.
constexpr int kPairMinT = 8;
static bool pair_eligible(const Plan &pl, int T, const uhs_params *p) {
    return pl.kernel == UHS_KERNEL_STREAM && pl.st == kStF64 && pl.ar == kArDf32 && T >= kPairMinT &&
           !(p && (p->flags & UHS_FLAG_IN_PLACE));
}

struct BatchSolo {
    SweepSpec sp;
    Plan pl;
    GridView va, vb;
    int T;
    double work;  // points x T x (overhead + terms): the branch balance
    // pair-resident: float-pair copies owned by the batch, and their plan
    bool pairs = false;
    SweepSpec sp2;
    Plan pl2;
    GridView pa{}, pb{};
};

static const uhs_params *effective_params(const uhs_stencil_desc *d, const uhs_params *p, uhs_params *buf);

struct uhs_batch_impl {
    int dev = 0;
    int n = 0;
    int n_solo = 0;
    int steps = 0;
    int64_t launches = 0, items0 = 0;
    BatchGrid *d_grids = nullptr;
    int4 *d_items[kNumPacks] = {nullptr, nullptr};
    int *d_counters = nullptr;  // one item counter per (timestep, pack), zeroed at each replay
    unsigned *d_status = nullptr;  // the batch's own status word (its graph may replay on any stream)
    std::vector<void *> scratch;   // float-pair copies of pair-resident solo grids
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

static void batch_free(uhs_batch_impl *b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_grids) cudaFree(b->d_grids);
    if (b->d_counters) cudaFree(b->d_counters);
    if (b->d_status) cudaFree(b->d_status);
    for (auto *p : b->d_items)
        if (p) cudaFree(p);
    for (auto *p : b->scratch) cudaFree(p);
    delete b;
}

static int batch_create(const uhs_stencil_desc *descs, const uhs_memref *as, const uhs_memref *bs, int32_t n,
                        const uhs_params *params, uhs_batch_impl **out) {
    if (!descs || !as || !bs || !out || n < 0) return set_error(UHS_EINVAL, "batch arguments must be non-NULL");
    auto *B = new uhs_batch_impl();
    std::unique_ptr<uhs_batch_impl, void (*)(uhs_batch_impl *)> guard(B, batch_free);
    cudaGetDevice(&B->dev);
    B->n = n;
    std::vector<BatchGrid> host(static_cast<size_t>(n));
    std::vector<BatchGridHost> info(static_cast<size_t>(n));
    std::vector<BatchSolo> solo;
    std::vector<std::vector<int4>> items(kNumPacks);
    {
        void *q = nullptr;
        if (dev_alloc(&q, kStatusWords * sizeof(unsigned)) != cudaSuccess ||
            cudaMemset(q, 0, kStatusWords * sizeof(unsigned)) != cudaSuccess)
            return set_error(UHS_ENOMEM, "batch status word allocation failed");
        B->d_status = static_cast<unsigned *>(q);
    }
    unsigned *err = B->d_status;
    cudaStream_t scan_stream = nullptr;
    if (cudaStreamCreateWithFlags(&scan_stream, cudaStreamNonBlocking) != cudaSuccess)
        return set_error(UHS_ECUDA, "stream creation failed");
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{scan_stream};
    for (int32_t i = 0; i < n; ++i) {
        GridView va, vb;
        int rc = prepare(&descs[i], &as[i], &bs[i], &va, &vb);
        if (rc) return set_error(rc, "program %d: %s", i, uhs_last_error());
        SweepSpec sp;
        make_spec(&descs[i], &sp);
        Plan pl;
        const int64_t points = (sp.ub[0] - sp.lb[0]) * (sp.ub[1] - sp.lb[1]) * (sp.ub[2] - sp.lb[2]);
        if (points >= kSoloPoints) {
            uhs_params tuned, sparams;
            const uhs_params *ep = effective_params(&descs[i], params, &tuned);
            if (ep) sparams = *ep;
            else uhs_params_default(&sparams);
            sparams.k_temporal = 0;  // one step per launch
            if ((rc = plan_sweep(sp, &sparams, va, &pl)) || pl.kernel != UHS_KERNEL_STREAM) {
                // a tuned entry for another kernel family: the caller's own parameters
                if (params) sparams = *params;
                else uhs_params_default(&sparams);
                sparams.k_temporal = 0;
                if ((rc = plan_sweep(sp, &sparams, va, &pl))) return set_error(rc, "program %d: %s", i, uhs_last_error());
            }
            if (pl.kernel != UHS_KERNEL_STREAM)
                return set_error(UHS_EUNSUPPORTED, "program %d is not a star/box stencil the batched kernel covers", i);
            if (pl.auto_df32 && descs[i].iterations > 0 &&
                !range_ok(sp, va, vb, descs[i].iterations, scan_stream, &pl.pair_shift)) {
                fall_back_native(pl);
            }
            const int nt = pl.factored ? 3 * (2 * pl.R + 1) : sp.nterms;
            const double per_term = pl.st == kStF32 ? 1.0 : pl.ar == kArDf32 ? 6.0 : 14.0;
            BatchSolo g;
            g.sp = sp;
            g.pl = pl;
            g.va = va;
            g.vb = vb;
            g.T = descs[i].iterations;
            g.work = static_cast<double>(points) * descs[i].iterations * (20.0 + per_term * nt);
            if (pair_eligible(pl, g.T, &sparams)) {
                const int64_t n0 = va.n[0], n1 = va.n[1], n2 = va.n[2];
                const size_t bytes = static_cast<size_t>(n0 * n1 * n2) * sizeof(double);
                void *buf = nullptr;
                if (dev_alloc(&buf, 2 * bytes) == cudaSuccess) {
                    B->scratch.push_back(buf);
                    g.pa = GridView{buf, {n0, n1, n2}, {n1 * n2, n2, 1}};
                    g.pb = GridView{static_cast<char *>(buf) + bytes, {n0, n1, n2}, {n1 * n2, n2, 1}};
                    g.sp2 = sp;
                    g.sp2.dtype = UHS_F32X2;
                    uhs_params q = sparams;
                    q.arith = UHS_ARITH_DF32;
                    ErrorMessageGuard keep;
                    g.pairs = plan_sweep(g.sp2, &q, g.pa, &g.pl2) == UHS_OK && g.pl2.kernel == UHS_KERNEL_STREAM;
                } else {
                    cudaGetLastError();  // no copies: this grid sweeps in place
                }
            }
            solo.push_back(g);
            info[i] = BatchGridHost{-1, 0, 0, i, 1, 1, 1, 0, 0.0};
            continue;
        }
        uhs_params bp;
        if (params) bp = *params;
        else uhs_params_default(&bp);
        bp.flags |= UHS_FLAG_NO_FACTOR;  // the batched packs sweep boxes term by term
        if ((rc = plan_sweep(sp, &bp, va, &pl))) return set_error(rc, "program %d: %s", i, uhs_last_error());
        if (pl.kernel != UHS_KERNEL_STREAM)
            return set_error(UHS_EUNSUPPORTED, "program %d is not a star/box stencil the batched kernel covers", i);
        if (pl.auto_df32 && descs[i].iterations > 0 &&
            !range_ok(sp, va, vb, descs[i].iterations, scan_stream, &pl.pair_shift)) {
            fall_back_native(pl);
        }
        int pack = kPackMain, kind = batch_kind(kPackMain, pl.shape, pl.R, pl.st, pl.ar);
        if (kind < 0) {
            pack = kPackF64Native;
            kind = batch_kind(pack, pl.shape, pl.R, pl.st, pl.ar);
        }
        if (kind < 0) return set_error(UHS_EUNSUPPORTED, "program %d: no batched variant for its element type", i);
        StreamCall c{};
        c.shape = pl.shape;
        c.R = pl.R;
        c.st = pl.st;
        c.ar = pl.ar;
        c.ld = kLdCpAsync;
        c.coef = pl.coef.data();
        const bool is2d = sp.rank == 2;
        c.lb[0] = is2d ? sp.lb[1] : sp.lb[0];
        c.ub[0] = is2d ? sp.ub[1] : sp.ub[0];
        c.lb[1] = is2d ? 0 : sp.lb[1];
        c.ub[1] = is2d ? 1 : sp.ub[1];
        c.lb[2] = sp.lb[2];
        c.ub[2] = sp.ub[2];
        c.err = err;
        c.pair_shift = pl.pair_shift;
        int bx, by, zc;
        batch_tile(pl.shape, pl.R, pl.st, &bx, &by, &zc);
        const int eb = sp.dtype == UHS_F32 ? 4 : 8;
        for (int d = 0; d < 2; ++d) {
            c.in = kernel_view(sp, d == 0 ? va : vb);
            c.out = kernel_view(sp, d == 0 ? vb : va);
            c.pair_loads = 0;
            if (eb == 4)
                c.pair_loads = ((c.lb[2] - c.R) % 2 == 0) && c.in.s[0] % 2 == 0 && c.in.s[1] % 2 == 0 &&
                               c.in.n[2] % 2 == 0 && reinterpret_cast<uintptr_t>(c.in.data) % 8 == 0;
            batch_fill_args(&host[i].dir[d], c, static_cast<int>(pl.coef.size()));
        }
        host[i].kind = kind;
        info[i] = BatchGridHost{pack, kind, descs[i].iterations, i, bx, by, zc, 0,
                                batch_item_cost(bx, by, 1, static_cast<int>(pl.coef.size()), pl.st, pl.ar)};
    }
    // z-chunks: the batch's estimated work shared by every resident CTA sets
    // a target item cost; grids whose 32-plane items would exceed a quarter of
    // a CTA's share get shorter chunks (down to 8 planes), so no single long
    // item holds up the end of a timestep.
    {
        double work = 0.0;
        for (int i = 0; i < n; ++i) {
            if (info[i].pack < 0) continue;  // solo grid
            const BatchArgs &a0 = host[i].dir[0];
            work += info[i].item_cost * static_cast<double>((a0.ub2 - a0.lb2) * (a0.ub1 - a0.lb1)) /
                    (static_cast<double>(info[i].bx) * info[i].by) * static_cast<double>(a0.ub0 - a0.lb0);
        }
        const double target = work / (4.0 * device_sms() * 3);
        for (int i = 0; i < n; ++i) {
            BatchGridHost &g = info[i];
            if (g.pack < 0) continue;
            int zc = g.zc;
            while (zc > 8 && g.item_cost * zc > target) zc /= 2;
            g.zc = zc;
            g.item_cost *= zc;
            for (int d = 0; d < 2; ++d) host[i].dir[d].zchunk = zc;
            const BatchArgs &a0 = host[i].dir[0];
            const int64_t tx = (a0.ub2 - a0.lb2 + g.bx - 1) / g.bx, ty = (a0.ub1 - a0.lb1 + g.by - 1) / g.by,
                          tz = (a0.ub0 - a0.lb0 + zc - 1) / zc;
            g.items = tx * ty * tz;
            if (g.items > (int64_t(1) << 28)) return set_error(UHS_EUNSUPPORTED, "program %d has too many tiles", i);
        }
    }
    // Items of each pack, grids in decreasing T so a timestep's active items
    // are a prefix of the list; within one T, costliest items first.
    std::vector<int> order(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        if (info[x].T != info[y].T) return info[x].T > info[y].T;
        return info[x].item_cost > info[y].item_cost;
    });
    std::vector<std::vector<int64_t>> prefix(kNumPacks);  // prefix[pack][step] = active items
    int steps = 0;
    for (int i = 0; i < n; ++i) steps = std::max(steps, info[i].T);
    B->steps = steps;
    for (int p = 0; p < kNumPacks; ++p) prefix[p].assign(static_cast<size_t>(steps), 0);
    for (int i : order) {
        const int p = info[i].pack;
        if (p < 0) continue;
        const int bx = info[i].bx, by = info[i].by, zc = info[i].zc;
        const BatchArgs &a0 = host[i].dir[0];
        const int64_t tx = (a0.ub2 - a0.lb2 + bx - 1) / bx, ty = (a0.ub1 - a0.lb1 + by - 1) / by,
                      tz = (a0.ub0 - a0.lb0 + zc - 1) / zc;
        for (int64_t z = 0; z < tz; ++z)
            for (int64_t y = 0; y < ty; ++y)
                for (int64_t x = 0; x < tx; ++x)
                    items[p].push_back(make_int4(i, static_cast<int>(x), static_cast<int>(y), static_cast<int>(z)));
        for (int s = 0; s < info[i].T; ++s) prefix[p][s] = static_cast<int64_t>(items[p].size());
    }
    if (items[0].size() + items[1].size() > static_cast<size_t>(INT32_MAX))
        return set_error(UHS_EUNSUPPORTED, "batch has too many work items");
    // Upload.
    if (n > 0) {
        void *p = nullptr;
        if (dev_alloc(&p, sizeof(BatchGrid) * static_cast<size_t>(n)) != cudaSuccess)
            return set_error(UHS_ENOMEM, "batch argument upload: allocation failed");
        B->d_grids = static_cast<BatchGrid *>(p);
        if (cudaMemcpy(B->d_grids, host.data(), sizeof(BatchGrid) * static_cast<size_t>(n), cudaMemcpyHostToDevice) !=
            cudaSuccess)
            return set_error(UHS_ECUDA, "batch argument upload failed");
    }
    int ctas[kNumPacks] = {0, 0};
    for (int p = 0; p < kNumPacks; ++p) {
        if (items[p].empty()) continue;
        void *q = nullptr;
        if (dev_alloc(&q, sizeof(int4) * items[p].size()) != cudaSuccess)
            return set_error(UHS_ENOMEM, "batch item list: allocation failed");
        B->d_items[p] = static_cast<int4 *>(q);
        if (cudaMemcpy(q, items[p].data(), sizeof(int4) * items[p].size(), cudaMemcpyHostToDevice) != cudaSuccess)
            return set_error(UHS_ECUDA, "batch item upload failed");
        BatchPackInfo bi;
        cudaError_t e = batch_prepare(p, &bi);
        if (e != cudaSuccess) return cuda_error(e, "batch kernel set-up");
        const int64_t want = static_cast<int64_t>(device_sms()) * std::max(1, bi.occ);
        ctas[p] = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(want, static_cast<int64_t>(items[p].size()))));
    }
    B->items0 = 0;
    for (int p = 0; p < kNumPacks; ++p)
        if (steps > 0) B->items0 += prefix[p][0];
    const size_t n_counters = static_cast<size_t>(steps) * kNumPacks;
    if (n_counters > 0) {
        void *q = nullptr;
        if (dev_alloc(&q, sizeof(int) * n_counters) != cudaSuccess)
            return set_error(UHS_ENOMEM, "batch item counters: allocation failed");
        B->d_counters = static_cast<int *>(q);
    }
    // Solo grids: costliest first onto the least-loaded of up to
    // kSoloBranches branches.
    const int nbr = std::min<int>(kSoloBranches, static_cast<int>(solo.size()));
    std::vector<std::vector<int>> branch(static_cast<size_t>(nbr));
    {
        std::vector<int> so(solo.size());
        for (size_t k = 0; k < solo.size(); ++k) so[k] = static_cast<int>(k);
        std::stable_sort(so.begin(), so.end(), [&](int x, int y) { return solo[x].work > solo[y].work; });
        std::vector<double> load(static_cast<size_t>(nbr), 0.0);
        for (int k : so) {
            const int bi = static_cast<int>(std::min_element(load.begin(), load.end()) - load.begin());
            branch[bi].push_back(k);
            load[bi] += solo[k].work;
        }
    }
    B->n_solo = static_cast<int>(solo.size());
    for (const BatchSolo &g : solo) B->steps = std::max(B->steps, g.T);
    // Capture the timestep loop of the persistent kernel and the solo grids'
    // sweeps (forked branches joined back at the end).
    if (steps > 0 || !solo.empty()) {
        cudaStream_t cs;
        if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess)
            return set_error(UHS_ECUDA, "capture stream creation failed");
        StreamGuard cg{cs};
        std::vector<cudaStream_t> bs_(static_cast<size_t>(nbr), nullptr);
        std::vector<cudaEvent_t> evs(static_cast<size_t>(nbr) + 1, nullptr);
        struct BranchGuard {
            std::vector<cudaStream_t> &s;
            std::vector<cudaEvent_t> &e;
            ~BranchGuard() {
                for (auto x : s)
                    if (x) cudaStreamDestroy(x);
                for (auto x : e)
                    if (x) cudaEventDestroy(x);
            }
        } bg{bs_, evs};
        for (int k = 0; k < nbr; ++k)
            if (cudaStreamCreateWithFlags(&bs_[k], cudaStreamNonBlocking) != cudaSuccess)
                return set_error(UHS_ECUDA, "branch stream creation failed");
        for (auto &ev : evs)
            if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess)
                return set_error(UHS_ECUDA, "branch event creation failed");
        if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return set_error(UHS_ECUDA, "graph capture could not start");
        cudaError_t e = cudaSuccess;
        int rc = UHS_OK;
        int64_t launches = 0;
        if (nbr > 0) {
            e = cudaEventRecord(evs[nbr], cs);
            for (int k = 0; k < nbr && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(bs_[k], evs[nbr], 0);
            for (int k = 0; k < nbr && e == cudaSuccess && rc == UHS_OK; ++k) {
                for (int gi : branch[k]) {
                    const BatchSolo &g = solo[gi];
                    if (g.pairs) {  // split a, and b's halo, into the copies
                        const int sh = g.pl.pair_shift;
                        e = launch_to_pairs(g.va, g.pa, g.sp.lb, g.sp.ub, false, sh, err, bs_[k]);
                        if (e == cudaSuccess) e = launch_to_pairs(g.vb, g.pb, g.sp.lb, g.sp.ub, true, sh, err, bs_[k]);
                        launches += 2;
                        if (e != cudaSuccess) break;
                    }
                    const SweepSpec &ssp = g.pairs ? g.sp2 : g.sp;
                    const Plan &spl = g.pairs ? g.pl2 : g.pl;
                    const GridView &ga = g.pairs ? g.pa : g.va, &gb = g.pairs ? g.pb : g.vb;
                    for (int t = 0; t < g.T && rc == UHS_OK; ++t) {
                        // T = 1: a -> b; even T: pairs a -> b, b -> a (as uhs_run)
                        const bool fwd = (t % 2) == 0;
                        rc = launch_sweep(ssp, spl, fwd ? ga : gb, fwd ? gb : ga, bs_[k], err);
                        ++launches;
                    }
                    if (rc) break;
                    if (g.pairs) {  // both domains back (T >= 8 sweeps wrote both grids)
                        const int sh = g.pl.pair_shift;
                        e = launch_from_pairs(g.pa, g.va, g.sp.lb, g.sp.ub, sh, err, bs_[k]);
                        if (e == cudaSuccess) e = launch_from_pairs(g.pb, g.vb, g.sp.lb, g.sp.ub, sh, err, bs_[k]);
                        launches += 2;
                        if (e != cudaSuccess) break;
                    }
                }
                if (rc == UHS_OK && e == cudaSuccess) e = cudaEventRecord(evs[k], bs_[k]);
            }
        }
        // every replay zeroes the persistent kernel's item counters (a memset node)
        if (e == cudaSuccess && rc == UHS_OK && n_counters > 0)
            e = cudaMemsetAsync(B->d_counters, 0, sizeof(int) * n_counters, cs);
        for (int s = 0; s < steps && e == cudaSuccess && rc == UHS_OK; ++s) {
            for (int p = 0; p < kNumPacks && e == cudaSuccess; ++p) {
                const int64_t m = prefix[p][s];
                if (m <= 0) continue;
                e = batch_launch(p, B->d_grids, B->d_items[p], static_cast<int>(m), s & 1, ctas[p],
                                 B->d_counters + static_cast<size_t>(s) * kNumPacks + p, cs);
                ++launches;
            }
        }
        for (int k = 0; k < nbr && e == cudaSuccess && rc == UHS_OK; ++k) e = cudaStreamWaitEvent(cs, evs[k], 0);
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        if (rc != UHS_OK || e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            if (rc != UHS_OK) return rc;
            return cuda_error(e != cudaSuccess ? e : e2, "batch graph capture");
        }
        B->graph = g;
        if ((e = cudaGraphInstantiate(&B->exec, g, 0)) != cudaSuccess) return cuda_error(e, "batch graph instantiate");
        B->launches = launches;
    }
    *out = guard.release();
    return UHS_OK;
}

// ---------------------------------------------------------------------------
// Tuner database (include/uhs.h): best launch parameters per program class.
// ---------------------------------------------------------------------------
struct TuneKey {
    int rank, shape, R, dtype;
    int64_t ext[3];
    bool operator<(const TuneKey &o) const {
        return std::tie(rank, shape, R, dtype, ext[0], ext[1], ext[2]) <
               std::tie(o.rank, o.shape, o.R, o.dtype, o.ext[0], o.ext[1], o.ext[2]);
    }
};
struct TuneEntry {
    uhs_params p;
    double gst;
};
static std::mutex g_tune_mu;
static std::map<TuneKey, TuneEntry> g_tune;

static bool tune_key(const uhs_stencil_desc *d, TuneKey *k) {
    SweepSpec sp;
    make_spec(d, &sp);
    int shape = -1, R = 0;
    if (!classify(sp, &shape, &R)) return false;
    k->rank = d->rank;
    k->shape = shape;
    k->R = R;
    k->dtype = d->dtype;
    for (int i = 0; i < 3; ++i) k->ext[i] = d->ub[i] - d->lb[i];
    return true;
}

static bool tune_lookup(const uhs_stencil_desc *d, uhs_params *out, bool *exact) {
    TuneKey k;
    if (!tune_key(d, &k)) return false;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(k);
    if (it != g_tune.end()) {
        *out = it->second.p;
        *exact = true;
        return true;
    }
    double best = 1e300;
    const TuneEntry *hit = nullptr;
    for (const auto &kv : g_tune) {
        const TuneKey &e = kv.first;
        if (e.rank != k.rank || e.shape != k.shape || e.R != k.R || e.dtype != k.dtype) continue;
        double dist = 0.0;
        for (int i = 0; i < 3; ++i)
            dist += std::fabs(std::log2(static_cast<double>(std::max<int64_t>(1, e.ext[i]))) -
                              std::log2(static_cast<double>(std::max<int64_t>(1, k.ext[i]))));
        if (dist < best) {
            best = dist;
            hit = &kv.second;
        }
    }
    if (!hit) return false;
    *out = hit->p;
    *exact = false;
    return true;
}

static bool params_are_auto(const uhs_params *p) {
    if (!p) return true;
    return p->kernel == 0 && p->arith == 0 && p->tile_x == 0 && p->tile_y == 0 && p->tile_z == 0 &&
           p->k_temporal == 0 && p->use_tma == 0 && p->vy == 0 && p->prefetch == 0 && p->vx == 0;
}

// The parameters a call runs with: the caller's, or the database's when the
// caller left everything on auto.
static const uhs_params *effective_params(const uhs_stencil_desc *d, const uhs_params *p, uhs_params *buf) {
    if (!params_are_auto(p) || (p && (p->flags & UHS_FLAG_NO_TUNE_DB))) return p;
    if (validate_desc(d) != UHS_OK) return p;  // the caller's own validation reports it
    bool exact = false;
    if (!tune_lookup(d, buf, &exact)) return p;
    if (buf->arith == UHS_ARITH_DF32) buf->arith = UHS_ARITH_AUTO;
    buf->flags = p ? p->flags : 0;
    return buf;
}
// Stream-ordered scratch from a memory pool the library creates on each
// device, set to keep freed memory for reuse (later runs then allocate
// without a device-wide synchronisation).  The device's default pool, which
// the host application may use, is left as it is.  uhs_release_scratch trims
// these pools.  Honours the diagnostic cap.
static std::mutex g_pool_mu;
static cudaMemPool_t g_pools[64] = {};

static cudaMemPool_t scratch_pool(int dev) {
    if (dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pools[dev] = pool;
    }
    return g_pools[dev];
}

static cudaError_t dev_alloc_async(void **p, size_t bytes, cudaStream_t st) {
    const int64_t cap = g_alloc_cap.load(std::memory_order_relaxed);
    if (cap > 0 && static_cast<int64_t>(bytes) > cap) return cudaErrorMemoryAllocation;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaMemPool_t pool = scratch_pool(dev);
    if (!pool) return cudaErrorMemoryAllocation;
    const cudaError_t e = cudaMallocFromPoolAsync(p, bytes, pool, st);
    if (e != cudaSuccess) cudaGetLastError();  // not sticky: the caller falls back
    return e;
}

// Pair-resident run of a float-pair FP64 program (see uhs_run in uhs.h):
// *ran stays false when the scratch could not be had or planned, and the
// caller then sweeps the FP64 grids in place.
static int run_pair_resident(const SweepSpec &sp, const uhs_params *p, const GridView &va, const GridView &vb,
                             int T, int shift, cudaStream_t st, bool *ran) {
    *ran = false;
    int dev = 0;
    cudaGetDevice(&dev);
    unsigned *err = stream_error_word(dev, st);
    if (!err) {
        *ran = true;  // report the failure instead of sweeping in place
        return set_error(UHS_ENOMEM, "device error word allocation failed");
    }
    const int64_t n0 = va.n[0], n1 = va.n[1], n2 = va.n[2];
    const size_t bytes = static_cast<size_t>(n0 * n1 * n2) * sizeof(double);
    void *buf = nullptr;
    if (dev_alloc_async(&buf, 2 * bytes, st) != cudaSuccess) return UHS_OK;
    const GridView pa{buf, {n0, n1, n2}, {n1 * n2, n2, 1}};
    const GridView pb{static_cast<char *>(buf) + bytes, {n0, n1, n2}, {n1 * n2, n2, 1}};
    SweepSpec sp2 = sp;
    sp2.dtype = UHS_F32X2;
    uhs_params q;
    if (p) q = *p;
    else uhs_params_default(&q);
    q.arith = UHS_ARITH_DF32;
    Plan pl2;
    bool planned;
    {
        ErrorMessageGuard keep;
        planned = plan_sweep(sp2, &q, pa, &pl2) == UHS_OK && pl2.kernel == UHS_KERNEL_STREAM;
    }
    if (!planned) {
        cudaFreeAsync(buf, st);
        return UHS_OK;
    }
    *ran = true;
    int rc = UHS_OK;
    cudaError_t e = launch_to_pairs(va, pa, sp.lb, sp.ub, false, shift, err, st);
    if (e == cudaSuccess) e = launch_to_pairs(vb, pb, sp.lb, sp.ub, true, shift, err, st);
    if (e != cudaSuccess) rc = cuda_error(e, "float-pair conversion");
    for (int it = 0; it < T / 2 && rc == UHS_OK; ++it) {
        if ((rc = launch_sweep(sp2, pl2, pa, pb, st))) break;
        rc = launch_sweep(sp2, pl2, pb, pa, st);
    }
    if (rc == UHS_OK) {
        e = launch_from_pairs(pa, va, sp.lb, sp.ub, shift, err, st);
        if (e == cudaSuccess) e = launch_from_pairs(pb, vb, sp.lb, sp.ub, shift, err, st);
        if (e != cudaSuccess) rc = cuda_error(e, "float-pair conversion");
    }
    cudaFreeAsync(buf, st);
    return rc;
}

}  // namespace uhs

using namespace uhs;

extern "C" {

const char *uhs_last_error(void) { return t_err.c_str(); }

int uhs_abi_version(void) { return UHS_ABI_VERSION; }

void uhs_params_default(uhs_params *p) {
    if (p) std::memset(p, 0, sizeof *p);
}

int64_t uhs_launch_count(void) { return g_launches.load(); }

int uhs_release_scratch(void) {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (int dev = 0; dev < 64; ++dev) {
        if (!g_pools[dev]) continue;
        const cudaError_t e = cudaMemPoolTrimTo(g_pools[dev], 0);
        if (e != cudaSuccess) return cuda_error(e, "scratch pool trim");
    }
    return UHS_OK;
}

int uhs_probe_wait_timeout(int64_t cycles, void *stream) {
    if (cycles < 1 || cycles > (int64_t(1) << 31))
        return set_error(UHS_EINVAL, "cycles must be in [1, 2^31] (got %lld)", static_cast<long long>(cycles));
    int dev = 0;
    cudaGetDevice(&dev);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned *w = stream_error_word(dev, st);
    if (!w) return set_error(UHS_ENOMEM, "device status word allocation failed");
    cudaError_t e = launch_wait_probe(w, static_cast<long long>(cycles), st);
    if (e != cudaSuccess) return cuda_error(e, "wait probe launch");
    return finish(nullptr, st);
}

int uhs_probe_dfma_rate(double *per_second, void *stream) {
    if (!per_second) return set_error(UHS_EINVAL, "per_second is NULL");
    const cudaError_t e = probe_dfma_rate(per_second, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_error(e, "FP64 rate probe");
    return UHS_OK;
}

int uhs_error_norms(const uhs_stencil_desc *d, const uhs_memref *x, const uhs_memref *ref, double out[4],
                    void *stream) {
    int rc = validate_desc(d);
    if (rc) return rc;
    if (!out) return set_error(UHS_EINVAL, "out is NULL");
    GridView vx, vr;
    if ((rc = view_of(d, x, "x", &vx))) return rc;
    uhs_stencil_desc d64 = *d;
    d64.dtype = UHS_F64;
    if ((rc = view_of(&d64, ref, "ref", &vr))) return rc;
    for (int i = 0; i < 3; ++i) {
        if (vx.n[i] != vr.n[i])
            return set_error(UHS_EINVAL, "x and ref differ in sizes[%d] (%lld vs %lld)", i, (long long)vx.n[i],
                             (long long)vr.n[i]);
        if (d->lb[i] < 0 || d->ub[i] > vx.n[i])
            return set_error(UHS_EINVAL, "domain axis %d [%lld, %lld) lies outside the grid", i, (long long)d->lb[i],
                             (long long)d->ub[i]);
    }
    const int64_t rows = (d->ub[0] - d->lb[0]) * (d->ub[1] - d->lb[1]);
    if (rows <= 0 || d->ub[2] <= d->lb[2]) {
        out[0] = out[1] = out[2] = out[3] = 0.0;
        return UHS_OK;
    }
    int64_t units = 0;
    int xchunks = 1, nblocks = 0;
    err_split(rows, d->ub[2] - d->lb[2], &units, &xchunks, &nblocks);
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return set_error(UHS_EUNSUPPORTED, "device ordinal %d", dev);
    // Runtime-owned scratch: one growable buffer per device, used under a lock
    // for the whole call so concurrent callers cannot share it.
    static std::mutex mu[64];
    static double *buf[64] = {};
    static int64_t cap[64] = {};
    std::lock_guard<std::mutex> lk(mu[dev]);
    const int64_t need = 4 * (nblocks + 1);
    if (cap[dev] < need) {
        if (buf[dev]) cudaFree(buf[dev]);
        buf[dev] = nullptr;
        cap[dev] = 0;
        void *p = nullptr;
        if (dev_alloc(&p, need * sizeof(double)) != cudaSuccess)
            return set_error(UHS_ENOMEM, "scratch allocation of %lld doubles failed", (long long)need);
        buf[dev] = static_cast<double *>(p);
        cap[dev] = need;
    }
    ErrNormsCall c{};
    c.dtype = d->dtype;
    c.x = vx;
    c.r = vr;
    for (int i = 0; i < 3; ++i) {
        c.lb[i] = d->lb[i];
        c.ub[i] = d->ub[i];
    }
    c.nblocks = nblocks;
    c.xchunks = xchunks;
    c.units = units;
    c.scratch = buf[dev];
    c.stream = static_cast<cudaStream_t>(stream);
    cudaError_t e = launch_error_norms(c);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, c.scratch + 4 * nblocks, 4 * sizeof(double), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e != cudaSuccess) return cuda_error(e, "error-norm reduction");
    return UHS_OK;
}

int uhs_validate(const uhs_stencil_desc *d, const uhs_memref *a, const uhs_memref *b) {
    GridView va, vb;
    return prepare(d, a, b, &va, &vb);
}

int uhs_plan(const uhs_stencil_desc *d, const uhs_memref *a, const uhs_params *p, uhs_params *out) {
    int rc = validate_desc(d);
    if (rc) return rc;
    uhs_params tuned;
    p = effective_params(d, p, &tuned);
    if (!out) return set_error(UHS_EINVAL, "out is NULL");
    SweepSpec sp;
    make_spec(d, &sp);
    GridView v{};
    if (a && (rc = view_of(d, a, "a", &v))) return rc;
    Plan pl;
    if ((rc = plan_sweep(sp, p, v, &pl))) return rc;
    uhs_params_default(out);
    out->kernel = pl.kernel;
    out->arith = pl.cfg.arith;
    if (pl.kernel == UHS_KERNEL_STREAM) {
        StreamCall c{};
        c.shape = pl.shape;
        c.R = pl.R;
        c.tile = pl.tile;
        c.ld = pl.ld;
        int bx, by;
        stream_tile_xy(c, &bx, &by);
        out->tile_x = bx;
        out->tile_y = sp.rank == 3 ? by : 1;
        out->vy = sp.rank == 3 ? tile_shape(false, (pl.shape == kBox3 && pl.R >= 2) ? 3 : pl.tile).vy : 1;
        out->vx = sp.rank == 2 ? tile_shape(true, pl.tile).vx : 1;
        out->use_tma = pl.ld == kLdTma ? 1 : -1;
        out->factored = pl.factored ? 1 : 0;
        out->prefetch = pl.pd;
    } else {
        out->tile_x = pl.cfg.tile_x > 0 ? pl.cfg.tile_x : 32;
        out->tile_y = pl.cfg.tile_y > 0 ? pl.cfg.tile_y : 8;
        out->use_tma = -1;
    }
    out->tile_z = pl.cfg.tile_z;
    out->k_temporal = pl.cfg.k_temporal;
    return UHS_OK;
}

int uhs_launch_geometry(const uhs_stencil_desc *d, const uhs_memref *a, const uhs_params *p, int64_t out[4]) {
    int rc = validate_desc(d);
    if (rc) return rc;
    if (!out) return set_error(UHS_EINVAL, "out is NULL");
    uhs_params tuned;
    p = effective_params(d, p, &tuned);
    SweepSpec sp;
    make_spec(d, &sp);
    GridView v{};
    if (a && (rc = view_of(d, a, "a", &v))) return rc;
    Plan pl;
    if ((rc = plan_sweep(sp, p, v, &pl))) return rc;
    out[0] = out[1] = out[2] = 0;
    out[3] = device_sms();
    if (pl.kernel != UHS_KERNEL_STREAM) return UHS_OK;
    StreamCall c = stream_call_of(sp, pl);
    int occ = 1;
    const int zc = stream_zchunk(sp, pl, c, &occ);
    int bx, by;
    stream_tile_xy(c, &bx, &by);
    const int64_t tiles = ((c.ub[2] - c.lb[2] + bx - 1) / bx) * ((c.ub[1] - c.lb[1] + by - 1) / by);
    const int64_t nz = c.ub[0] - c.lb[0];
    out[0] = zc;
    out[1] = occ;
    out[2] = tiles * ((nz + zc - 1) / zc);
    return UHS_OK;
}

int uhs_sweep(const uhs_stencil_desc *d, const uhs_memref *in, const uhs_memref *out, const uhs_params *p,
              void *stream) {
    uhs_params tuned;
    if (d) p = effective_params(d, p, &tuned);
    GridView vi, vo;
    int rc = prepare(d, in, out, &vi, &vo);
    if (rc) return rc;
    SweepSpec sp;
    make_spec(d, &sp);
    Plan pl;
    if ((rc = plan_sweep(sp, p, vi, &pl))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (pl.auto_df32 && !range_ok(sp, vi, vo, 1, st, &pl.pair_shift)) {
        fall_back_native(pl);
    }
    if ((rc = launch_sweep(sp, pl, vi, vo, st))) return rc;
    return finish(p, st);
}

int uhs_run(const uhs_stencil_desc *d, const uhs_memref *a, const uhs_memref *b, const uhs_params *p,
            void *stream) {
    uhs_params tuned;
    if (d) p = effective_params(d, p, &tuned);
    GridView va, vb;
    int rc = prepare(d, a, b, &va, &vb);
    if (rc) return rc;
    SweepSpec sp;
    make_spec(d, &sp);
    Plan pl;
    if ((rc = plan_sweep(sp, p, va, &pl))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (pl.auto_df32 && d->iterations > 0 && !range_ok(sp, va, vb, d->iterations, st, &pl.pair_shift)) {
        fall_back_native(pl);
    }
    if (pl.kernel == UHS_KERNEL_STREAM && pl.cfg.k_temporal > 1 && d->iterations > 1) {
        bool eq = false;
        if ((rc = halos_equal(sp, va, vb, st, &eq))) return rc;
        if (!eq)
            return set_error(UHS_EINVAL, "temporal fusion needs both grids to hold the same values outside the "
                                         "domain (the halo); run with k_temporal = 1");
        const std::vector<int> passes = plan_passes(d->iterations, pl.cfg.k_temporal);
        bool fwd = true;
        for (int depth : passes) {
            const GridView &in = fwd ? va : vb, &out = fwd ? vb : va;
            rc = depth == 1 ? launch_sweep(sp, pl, in, out, st) : launch_fused_pass(sp, pl, in, out, depth, st);
            if (rc) return rc;
            fwd = !fwd;
        }
        return finish(p, st);
    }
    if (pair_eligible(pl, d->iterations, p)) {
        bool ran = false;
        rc = run_pair_resident(sp, p, va, vb, d->iterations, pl.pair_shift, st, &ran);
        if (ran) return rc ? rc : finish(p, st);
    }
    if (d->iterations == 1) {
        if ((rc = launch_sweep(sp, pl, va, vb, st))) return rc;
    } else {
        for (int it = 0; it < d->iterations / 2; ++it) {
            if ((rc = launch_sweep(sp, pl, va, vb, st))) return rc;
            if ((rc = launch_sweep(sp, pl, vb, va, st))) return rc;
        }
    }
    return finish(p, st);
}

struct uhs_batch {
    uhs_batch_impl *impl;
};

int uhs_batch_create(const uhs_stencil_desc *descs, const uhs_memref *a, const uhs_memref *b, int32_t n,
                     const uhs_params *params, uhs_batch **out) {
    if (!out) return set_error(UHS_EINVAL, "out is NULL");
    *out = nullptr;
    uhs_batch_impl *impl = nullptr;
    int rc = batch_create(descs, a, b, n, params, &impl);
    if (rc) return rc;
    *out = new uhs_batch{impl};
    return UHS_OK;
}

int uhs_batch_run(uhs_batch *batch, void *stream, int32_t flags) {
    if (!batch || !batch->impl) return set_error(UHS_EINVAL, "batch is NULL");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (batch->impl->exec) {
        cudaError_t e = cudaGraphLaunch(batch->impl->exec, st);
        if (e != cudaSuccess) return cuda_error(e, "batch graph launch");
        count_launch(static_cast<int>(batch->impl->launches));
    }
    if (flags & UHS_FLAG_NO_SYNC) return UHS_OK;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "stream synchronise");
    return check_status_word(batch->impl->d_status, st);
}

int uhs_batch_stats(const uhs_batch *batch, int64_t *launches, int64_t *steps, int64_t *items) {
    if (!batch || !batch->impl) return set_error(UHS_EINVAL, "batch is NULL");
    if (launches) *launches = batch->impl->launches;
    if (steps) *steps = batch->impl->steps;
    if (items) *items = batch->impl->items0;
    return UHS_OK;
}

void uhs_batch_destroy(uhs_batch *batch) {
    if (!batch) return;
    batch_free(batch->impl);
    delete batch;
}

int uhs_run_batch(const uhs_stencil_desc *descs, const uhs_memref *a, const uhs_memref *b, int32_t n,
                  const uhs_params *params, void *stream) {
    uhs_batch *bt = nullptr;
    int rc = uhs_batch_create(descs, a, b, n, params, &bt);
    if (rc) return rc;
    rc = uhs_batch_run(bt, stream, params ? params->flags & ~UHS_FLAG_NO_SYNC : 0);
    uhs_batch_destroy(bt);
    return rc;
}

int uhs_tune_put(const uhs_stencil_desc *d, const uhs_params *best, double gst) {
    int rc = validate_desc(d);
    if (rc) return rc;
    if (!best) return set_error(UHS_EINVAL, "best is NULL");
    TuneKey k;
    if (!tune_key(d, &k)) return set_error(UHS_EUNSUPPORTED, "only star and box programs of radius 1-3 are tuned");
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[k] = TuneEntry{*best, gst};
    return UHS_OK;
}

int uhs_tune_get(const uhs_stencil_desc *d, uhs_params *out, int32_t *exact) {
    int rc = validate_desc(d);
    if (rc) return rc;
    if (!out) return set_error(UHS_EINVAL, "out is NULL");
    bool ex = false;
    if (!tune_lookup(d, out, &ex)) return set_error(UHS_EINVAL, "the tuner database has no entry for this class");
    if (exact) *exact = ex ? 1 : 0;
    return UHS_OK;
}

// File format: a header line "uhs-tune 2", then one entry per line:
//   rank shape R dtype ext0 ext1 ext2 kernel arith tile_x tile_y tile_z
//   k_temporal use_tma flags vy prefetch vx gstencil_per_s
// (files of version 1, written before vx, have no vx column and still load)
int uhs_tune_save(const char *path) {
    if (!path) return set_error(UHS_EINVAL, "path is NULL");
    std::map<TuneKey, TuneEntry> snap;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        snap = g_tune;
    }
    const std::string tmp = std::string(path) + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "w");
    if (!f) return set_error(UHS_EINVAL, "cannot write %s", tmp.c_str());
    bool ok = std::fprintf(f, "uhs-tune 2\n") > 0;
    for (const auto &kv : snap) {
        const TuneKey &k = kv.first;
        const uhs_params &q = kv.second.p;
        ok = ok && std::fprintf(f, "%d %d %d %d %lld %lld %lld %d %d %d %d %d %d %d %d %d %d %d %.9g\n", k.rank,
                                k.shape, k.R, k.dtype, static_cast<long long>(k.ext[0]),
                                static_cast<long long>(k.ext[1]), static_cast<long long>(k.ext[2]), q.kernel, q.arith,
                                q.tile_x, q.tile_y, q.tile_z, q.k_temporal, q.use_tma, q.flags, q.vy, q.prefetch, q.vx,
                                kv.second.gst) > 0;
    }
    ok = (std::fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return set_error(UHS_EINVAL, "writing %s failed", path);
    }
    return UHS_OK;
}

// Entries are read into a scratch table and merged only when the whole file
// parses and every field is in range: a truncated or corrupted file changes
// nothing.
int uhs_tune_load(const char *path) {
    if (!path) return set_error(UHS_EINVAL, "path is NULL");
    FILE *f = std::fopen(path, "r");
    if (!f) return set_error(UHS_EINVAL, "cannot read %s", path);
    std::map<TuneKey, TuneEntry> got;
    char line[512];
    int lineno = 0;
    int rc = UHS_OK;
    int version = 0;
    while (std::fgets(line, sizeof line, f)) {
        ++lineno;
        if (lineno == 1) {
            if (std::strncmp(line, "uhs-tune 1", 10) == 0) version = 1;
            else if (std::strncmp(line, "uhs-tune 2", 10) == 0) version = 2;
            else {
                rc = set_error(UHS_EPARSE, "%s: not a tuner database (header)", path);
                break;
            }
            continue;
        }
        if (line[0] == '\n' || line[0] == '\0') continue;
        TuneKey k{};
        uhs_params q;
        uhs_params_default(&q);
        long long e0, e1, e2;
        double gst = 0.0;
        char extra[2];
        int n;
        if (version == 1) {
            n = std::sscanf(line, "%d %d %d %d %lld %lld %lld %d %d %d %d %d %d %d %d %d %d %lf %1s", &k.rank, &k.shape,
                            &k.R, &k.dtype, &e0, &e1, &e2, &q.kernel, &q.arith, &q.tile_x, &q.tile_y, &q.tile_z,
                            &q.k_temporal, &q.use_tma, &q.flags, &q.vy, &q.prefetch, &gst, extra);
        } else {
            n = std::sscanf(line, "%d %d %d %d %lld %lld %lld %d %d %d %d %d %d %d %d %d %d %d %lf %1s", &k.rank,
                            &k.shape, &k.R, &k.dtype, &e0, &e1, &e2, &q.kernel, &q.arith, &q.tile_x, &q.tile_y,
                            &q.tile_z, &q.k_temporal, &q.use_tma, &q.flags, &q.vy, &q.prefetch, &q.vx, &gst, extra);
            n -= 1;  // the vx column
        }
        k.ext[0] = e0;
        k.ext[1] = e1;
        k.ext[2] = e2;
        const bool shape_ok = k.rank == 3 ? (k.shape == kStar3 || k.shape == kBox3)
                                          : (k.rank == 2 && (k.shape == kStar2 || k.shape == kBox2));
        const bool in_range = n == 18 && shape_ok &&
                              k.R >= 1 && k.R <= 3 && k.dtype >= UHS_F64 && k.dtype <= UHS_F32X2 && e0 >= 1 &&
                              e1 >= 1 && e2 >= 1 && q.kernel >= UHS_KERNEL_AUTO && q.kernel <= UHS_KERNEL_MMA &&
                              q.arith >= UHS_ARITH_AUTO && q.arith <= UHS_ARITH_DF32 && q.tile_x >= 0 &&
                              q.tile_x <= 1024 && q.tile_y >= 0 && q.tile_y <= 1024 && q.tile_z >= 0 &&
                              q.k_temporal >= 0 && q.k_temporal <= 4 && q.use_tma >= -1 && q.use_tma <= 1 &&
                              q.vy >= 0 && q.vy <= 8 && q.prefetch >= 0 && q.prefetch <= 8 && q.vx >= 0 &&
                              q.vx <= 2 && std::isfinite(gst);
        if (!in_range) {
            rc = set_error(UHS_EPARSE, "%s:%d: malformed tuner entry", path, lineno);
            break;
        }
        got[k] = TuneEntry{q, gst};
    }
    if (rc == UHS_OK && lineno == 0) rc = set_error(UHS_EPARSE, "%s: empty file", path);
    std::fclose(f);
    if (rc != UHS_OK) return rc;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const auto &kv : got) g_tune[kv.first] = kv.second;
    return UHS_OK;
}

int uhs_set_alloc_cap(int64_t bytes) {
    if (bytes < 0) return set_error(UHS_EINVAL, "the cap must be >= 0 (0: none)");
    g_alloc_cap.store(bytes);
    return UHS_OK;
}

void uhs_tune_clear(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
}

int64_t uhs_tune_size(void) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return static_cast<int64_t>(g_tune.size());
}

}  // extern "C"
