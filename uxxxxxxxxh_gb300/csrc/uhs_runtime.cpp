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
#include "uhs_kernels.h"

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

namespace uhs {

static std::atomic<int64_t> g_launches{0};
void count_launch(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

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

static int cuda_error(cudaError_t e, const char *what) {
    return set_error(UHS_ECUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

// Per-device error word (see uhs_kernels.h).  Allocated on first use.
unsigned *device_error_word(int device) {
    static std::mutex mu;
    static unsigned *words[64] = {};
    if (device < 0 || device >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    if (!words[device]) {
        void *p = nullptr;
        if (cudaMalloc(&p, sizeof(unsigned)) != cudaSuccess) return nullptr;
        cudaMemset(p, 0, sizeof(unsigned));
        words[device] = static_cast<unsigned *>(p);
    }
    return words[device];
}

static size_t elem_bytes(int dtype) { return dtype == UHS_F64 ? 8 : 4; }

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

static int plan_cfg(const SweepSpec &sp, const uhs_params *p, LaunchCfg *cfg) {
    uhs_params dflt;
    uhs_params_default(&dflt);
    if (!p) p = &dflt;
    cfg->kernel = p->kernel == UHS_KERNEL_AUTO ? UHS_KERNEL_GENERIC : p->kernel;
    cfg->arith = p->arith == UHS_ARITH_AUTO ? UHS_ARITH_FMA : p->arith;
    cfg->tile_x = p->tile_x;
    cfg->tile_y = p->tile_y;
    cfg->tile_z = p->tile_z;
    cfg->k_temporal = p->k_temporal > 0 ? p->k_temporal : 1;
    cfg->use_tma = p->use_tma;
    if (cfg->kernel != UHS_KERNEL_GENERIC)
        return set_error(UHS_EUNSUPPORTED, "kernel family %d is not available for this stencil", cfg->kernel);
    if (cfg->arith != UHS_ARITH_FMA && cfg->arith != UHS_ARITH_EXACT)
        return set_error(UHS_EUNSUPPORTED, "arithmetic mode %d is not available for the generic kernel", cfg->arith);
    if (sp.dtype == UHS_F32X2)
        return set_error(UHS_EUNSUPPORTED, "float-pair grids need the streaming kernel");
    const int tx = cfg->tile_x > 0 ? cfg->tile_x : 32, ty = cfg->tile_y > 0 ? cfg->tile_y : 8;
    if (tx * ty > 256) return set_error(UHS_EINVAL, "tile %d x %d exceeds 256 threads", tx, ty);
    if (tx % 32 != 0) return set_error(UHS_EINVAL, "tile_x must be a multiple of 32 (got %d)", tx);
    return UHS_OK;
}

static int launch_sweep(const SweepSpec &sp, const LaunchCfg &cfg, const GridView &in, const GridView &out,
                        cudaStream_t st) {
    cudaError_t e = launch_generic(sp, cfg, in, out, st);
    if (e != cudaSuccess) return cuda_error(e, "sweep launch");
    return UHS_OK;
}

static int finish(const uhs_params *p, cudaStream_t st) {
    if (p && (p->flags & UHS_FLAG_NO_SYNC)) return UHS_OK;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "stream synchronise");
    return UHS_OK;
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
    return check_reach(d, *va);
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

int uhs_validate(const uhs_stencil_desc *d, const uhs_memref *a, const uhs_memref *b) {
    GridView va, vb;
    return prepare(d, a, b, &va, &vb);
}

int uhs_plan(const uhs_stencil_desc *d, const uhs_memref *a, const uhs_params *p, uhs_params *out) {
    int rc = validate_desc(d);
    if (rc) return rc;
    if (!out) return set_error(UHS_EINVAL, "out is NULL");
    SweepSpec sp;
    make_spec(d, &sp);
    LaunchCfg cfg;
    if ((rc = plan_cfg(sp, p, &cfg))) return rc;
    (void)a;
    uhs_params_default(out);
    out->kernel = cfg.kernel;
    out->arith = cfg.arith;
    out->tile_x = cfg.tile_x > 0 ? cfg.tile_x : 32;
    out->tile_y = cfg.tile_y > 0 ? cfg.tile_y : 8;
    out->tile_z = cfg.tile_z;
    out->k_temporal = cfg.k_temporal;
    out->use_tma = cfg.use_tma;
    return UHS_OK;
}

int uhs_sweep(const uhs_stencil_desc *d, const uhs_memref *in, const uhs_memref *out, const uhs_params *p,
              void *stream) {
    GridView vi, vo;
    int rc = prepare(d, in, out, &vi, &vo);
    if (rc) return rc;
    SweepSpec sp;
    make_spec(d, &sp);
    LaunchCfg cfg;
    if ((rc = plan_cfg(sp, p, &cfg))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if ((rc = launch_sweep(sp, cfg, vi, vo, st))) return rc;
    return finish(p, st);
}

int uhs_run(const uhs_stencil_desc *d, const uhs_memref *a, const uhs_memref *b, const uhs_params *p,
            void *stream) {
    GridView va, vb;
    int rc = prepare(d, a, b, &va, &vb);
    if (rc) return rc;
    SweepSpec sp;
    make_spec(d, &sp);
    LaunchCfg cfg;
    if ((rc = plan_cfg(sp, p, &cfg))) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (d->iterations == 1) {
        if ((rc = launch_sweep(sp, cfg, va, vb, st))) return rc;
    } else {
        for (int it = 0; it < d->iterations / 2; ++it) {
            if ((rc = launch_sweep(sp, cfg, va, vb, st))) return rc;
            if ((rc = launch_sweep(sp, cfg, vb, va, st))) return rc;
        }
    }
    return finish(p, st);
}

}  // extern "C"
