/*
 * uhs.h -- C ABI of the GB300 stencil backend for UHStencil.
 *
 * The backend replaces what UHStencil's GPU lowering produces for one stencil
 * program: the generated sweep kernel (one stencil.apply over the domain) and
 * the generated program entry _mlir_ciface_<name>_iteration that runs T/2
 * ping-pong pairs of sweeps.  Callers hand in device memory exactly as the
 * reference's drivers do (UH-GPU/3d1r_star/3d7pt_main.cpp:117-150): two
 * caller-allocated grids described by MLIR memref descriptors, result in the
 * first one.  Everything here is plain C: pointers, sizes, status codes.
 *
 * Grid layout: row-major, slowest axis first, unit stride on the fastest axis,
 * halo cells included in the extents (a 512^3 interior with a 1-cell halo is
 * a 514^3 memref).  A rank-2 grid is passed as rank 3 with sizes[0] == 1.
 *
 * Status: every entry returns an int status; uhs_last_error() gives the
 * message of the last failing call on the calling thread.
 */
#ifndef UHS_H_
#define UHS_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UHS_ABI_VERSION 1

/* Largest expression the sweep kernels accept: 343 terms (7^3 box) plus room
 * for hand-written programs. */
#define UHS_MAX_TERMS 512
/* Largest |offset| on any axis. */
#define UHS_MAX_RADIUS 4

/* ---- status codes ------------------------------------------------------ */
enum {
    UHS_OK = 0,
    UHS_EINVAL = 1,       /* malformed descriptor, memref or parameters */
    UHS_EUNSUPPORTED = 2, /* well-formed but outside what the kernels cover */
    UHS_ECUDA = 3,        /* a CUDA call failed; the message names it */
    UHS_ETIMEOUT = 4,     /* a device-side wait ran out of its bound */
    UHS_ENOMEM = 5,       /* a runtime-owned allocation failed */
    UHS_ERANGE = 6,       /* a value is outside what the chosen arithmetic represents */
    UHS_EPARSE = 7        /* DSL text did not parse */
};

/* ---- element types and arithmetic -------------------------------------- */
enum {
    UHS_F64 = 0,  /* double grids (the reference's type in every case) */
    UHS_F32 = 1,  /* float grids, float arithmetic */
    UHS_F32X2 = 2 /* compensated pair: each 8-byte element is {float hi, float lo},
                     value = hi + lo (about 48 significant bits) */
};

enum {
    UHS_ARITH_AUTO = 0,  /* the backend picks: for F64 grids on the streaming kernel,
                            float pairs scaled by a power of two chosen from a device
                            scan of both grids (one extra read of each grid and one
                            host round trip per call), unless the grids hold Inf/NaN
                            or span more than about 2^169 between the largest
                            magnitude grown by (sum|c|)^T and the smallest nonzero
                            one; then UHS_ARITH_FMA */
    UHS_ARITH_FMA = 1,   /* native arithmetic, products fused into the sum */
    UHS_ARITH_EXACT = 2, /* separately rounded products and sums in expression
                            order: bit-identical to the serial CPU loops */
    UHS_ARITH_DF32 = 3   /* F64 grids computed in float-pair arithmetic on the FP32
                            pipes, unscaled: 48-bit significands in the float exponent
                            range (a value between 2^-74 and 2^128 is held to 2^-48 of
                            itself; below 2^-74 a pair keeps 24 bits, below 2^-126 it
                            flushes to zero; 2^128 or more returns UHS_ERANGE).  Star
                            and separable sums are error-free on a power-of-two grid set
                            per point from sum |c_k x_k| (bounded sums); each point's
                            error stays within about n^2 2^-46 of that sum for n terms */
};

/* ---- MLIR memref descriptor (rank-3 layout) ---------------------------- */
/* Same field order as MLIR's StridedMemRefType<T, 3>; strides and offset
 * count elements.  The element address of (z, y, x) is
 *   aligned + offset + z*strides[0] + y*strides[1] + x*strides[2]. */
typedef struct uhs_memref {
    void *allocated;
    void *aligned;
    int64_t offset;
    int64_t sizes[3];
    int64_t strides[3];
} uhs_memref;

/* ---- stencil descriptor ------------------------------------------------ */
/* One term of the linear form  out[p] = sum_k coef_k * in[p + (dz,dy,dx)_k].
 * Terms are kept in the order the .dsl expression writes them.  A term whose
 * param >= 0 takes its coefficient from the parameter array of the program
 * (the DSL's `c[2]*U[x-1]...` form); coef is ignored for it. */
typedef struct uhs_term {
    int32_t dz, dy, dx;
    int32_t param;
    double coef;
} uhs_term;

typedef struct uhs_stencil_desc {
    int32_t rank;         /* 2 or 3 */
    int32_t dtype;        /* UHS_F64 / UHS_F32 / UHS_F32X2 */
    int64_t lb[3];        /* domain, slowest first; rank 2: lb[0]=0, ub[0]=1 */
    int64_t ub[3];
    int32_t nterms;
    const uhs_term *terms;
    int32_t iterations;   /* T: 1 (single sweep a -> b) or even (T/2 pairs, result in a) */
    const double *params; /* host copy of the parameter array, or NULL */
    int32_t nparams;
} uhs_stencil_desc;

/* ---- tuning parameters ------------------------------------------------- */
/* The launch parameters UHStencil fixes at compile time through pass options
 * (tile_sizes_l0/l1, inner_tile, use smem: include/Conversion/UHAffineToParallel/
 * Passes.td:6-101) become run-time values.  Zero means "let the backend choose":
 * the tuner database entry for the program when there is one (filled by the
 * exhaustive tuner or by the learned cost model's picks, uhs_tune_put), else
 * the planner's defaults, which are set per sweep class from GB300 timings. */
enum {
    UHS_KERNEL_AUTO = 0,
    UHS_KERNEL_GENERIC = 1, /* any term list, smem plane ring, expression order */
    UHS_KERNEL_STREAM = 2,  /* 2.5D register streaming, templated star/box shapes */
    UHS_KERNEL_MMA = 3      /* box radius 2/3: contraction on tensor cores */
};

typedef struct uhs_params {
    int32_t kernel;       /* UHS_KERNEL_* */
    int32_t arith;        /* UHS_ARITH_* */
    int32_t tile_x;       /* CTA tile along x (fastest axis) */
    int32_t tile_y;       /* CTA tile along y (rank 3) */
    int32_t tile_z;       /* planes (rows, rank 2) streamed per CTA along the slowest axis;
                             0: about four waves of CTAs, at least 8 planes / 32 rows, capped
                             for some sweep classes */
    int32_t k_temporal;   /* timesteps fused per pass over HBM */
    int32_t use_tma;      /* -1 off (cp.async loads), 0 auto, 1 on */
    int32_t flags;        /* UHS_FLAG_* */
    int32_t vy;           /* points per thread along y (streaming kernel, rank 3) */
    int32_t prefetch;     /* planes (rows) loaded ahead of the one computed: fixed per kernel
                             variant (streaming: 3 planes, 2 for radius 2-3 boxes swept term
                             by term and for temporal fusion, 4 rows in 2D; generic: 1).
                             0 or the built depth; uhs_plan reports it */
    int32_t factored;     /* set by uhs_plan: 1 when a separable box runs as 1D passes */
    int32_t vx;           /* points per thread along x: 0 or 1, or 2 for rank-2 stars on FP32
                             grids or in float pairs (tile_x 128 or 256, the CTA's columns;
                             256 loads by cp.async) */
} uhs_params;

enum {
    UHS_FLAG_NO_SYNC = 1,    /* return without synchronising the stream */
    UHS_FLAG_NO_TUNE_DB = 2, /* ignore the tuner database for this call */
    UHS_FLAG_NO_FACTOR = 4,  /* sweep a separable box term by term, not as 1D passes */
    UHS_FLAG_MMA_TMEM_A = 8, /* tensor-core path: stage the A operand in tensor memory
                                (tcgen05.cp) instead of reading it from shared memory */
    UHS_FLAG_IN_PLACE = 16,  /* FP64 grids in float pairs: sweep the FP64 grids themselves,
                                not pair-resident copies (no scratch; see uhs_run) */
    UHS_FLAG_XSHUFFLE = 32   /* rank-2 stars on FP32 grids (256-wide strips, cp.async) or
                                float-pair grids (128-wide; for FP64 grids, the sweeps of
                                pair-resident runs): x-neighbours from the adjacent lanes by
                                warp shuffles instead of shared memory (an evaluated
                                alternative, kept for comparison) */
};

/* ---- entry points ------------------------------------------------------ */

/* Thread-local message for the last failing call (never NULL). */
const char *uhs_last_error(void);

/* Version of this ABI (UHS_ABI_VERSION). */
int uhs_abi_version(void);

/* Fill *p with the defaults (all zero / auto). */
void uhs_params_default(uhs_params *p);

/* Check a descriptor and its two grids without touching the GPU. */
int uhs_validate(const uhs_stencil_desc *desc, const uhs_memref *a, const uhs_memref *b);

/* Run the program: desc->iterations == 1 sweeps a -> b; an even count runs
 * iterations/2 pairs (a -> b, b -> a), leaving step T in a and step T-1 in b,
 * like the reference's generated <name>_iteration
 * (UHStencil/lib/Conversion/StencilToStandard/ConvertStencilToStandard.cpp:298-337).
 * a and b are device grids of identical shape; cells outside the domain are
 * read, never written, in both.  stream is a cudaStream_t (NULL = legacy
 * default stream).  Unless UHS_FLAG_NO_SYNC is set the call returns after the
 * stream has drained, which is what the reference's entry does.
 *
 * Pair-resident runs: FP64 grids swept in float-pair arithmetic (UHS_ARITH_AUTO
 * after its range check, or UHS_ARITH_DF32) with T >= 8 sweeps on the
 * streaming kernel (star and box stencils) run on float-pair copies of the grids.  Each value is split into its {hi, lo}
 * floats once, the T sweeps read and write pairs, and the domain of both grids
 * is joined back to FP64 at the end.  The halo is read from the FP64 grids and
 * never written, so it stays bit-exact.  The copies (16 bytes per grid cell)
 * are stream-ordered allocations from a memory pool the library owns on each
 * device, which keeps freed memory for the next run (uhs_release_scratch
 * returns it; the device's default pool is not touched).  When that
 * allocation fails, or with UHS_FLAG_IN_PLACE, the sweeps run on the FP64
 * grids directly, splitting on every load.
 *
 * Range: under UHS_ARITH_AUTO the pairs hold every value times 2^s, with s
 * chosen from a scan of both grids so that the largest magnitude, grown by
 * (sum|c|)^T, stays below 2^120 (a linear sweep commutes with the scale
 * exactly); the run keeps float pairs when every nonzero magnitude, scaled,
 * is at least 2^-50, and computes in native FP64 otherwise (or when a grid
 * holds Inf/NaN).  With either float-pair mode, a value that leaves the
 * float range during the run makes the call return UHS_ERANGE. */
int uhs_run(const uhs_stencil_desc *desc, const uhs_memref *a, const uhs_memref *b,
            const uhs_params *params, void *stream);

/* One sweep in -> out (the compute function MLIRGen emits beside the
 * iteration entry, UHStencil/lib/Parser/MLIRGen.cpp:183-273). */
int uhs_sweep(const uhs_stencil_desc *desc, const uhs_memref *in, const uhs_memref *out,
              const uhs_params *params, void *stream);

/* Pass plan the backend would use: fills kernel/arith/tiles/k of *out. */
int uhs_plan(const uhs_stencil_desc *desc, const uhs_memref *a, const uhs_params *params,
             uhs_params *out);

/* Geometry of the streaming launch uhs_plan describes, for cost models:
 *   out[0] = z-chunk (planes, or rows of a rank-2 grid, per CTA)
 *   out[1] = resident CTAs per SM of the kernel variant
 *   out[2] = CTAs in the launch            out[3] = SMs of the current device
 * out[0..2] are 0 when the plan is not a streaming launch.  Occupancy comes
 * from the CUDA runtime's query (1 where it cannot answer, e.g. without a
 * GPU).  The z-chunk the reference fixes at compile time through its
 * tile_sizes_l0 (include/Conversion/UHAffineToParallel/Passes.td:6-101) is
 * chosen here at run time. */
int uhs_launch_geometry(const uhs_stencil_desc *desc, const uhs_memref *a, const uhs_params *params,
                        int64_t out[4]);

/* FP64 error of grid x against the FP64 grid ref over desc's domain, reduced
 * on the GPU (the comparison the reference's drivers do on the host after a
 * run, UH-GPU/3d1r_star/3d7pt_main.cpp:84-96, here for x of any element type):
 *   out[0] = ||x - ref||_2 / ||ref||_2    out[1] = max |x - ref|
 *   out[2] = out[1] / max |ref|            out[3] = max |ref|
 * x has desc->dtype (F64, F32 or F32X2 pairs); ref is F64 of the same sizes.
 * Returns after the stream drained, with out filled.  Partial sums use
 * scratch memory the library allocates on first use (4 doubles per CTA, at
 * most 608 CTAs: under 20 KiB, one buffer per device, serialised by a lock).
 * The sums are FP64; the result does not depend on the device. */
int uhs_error_norms(const uhs_stencil_desc *desc, const uhs_memref *x, const uhs_memref *ref, double out[4],
                    void *stream);

/* Partial-sum slots of the allocation-free reduction below.  A reduction
 * uses at most 608 (one per CTA), so every domain fits. */
#define UHS_NOALLOC_MAX_PARTIALS 8192

/* No counterpart in the reference.  The same reduction as uhs_error_norms
 * (same kernels, bit-identical results) for callers that cannot allocate
 * device memory: a plugin hosted by an application that owns every device
 * allocation and forbids its plugins cudaMalloc, a service that must not grow
 * its device footprint or risk an allocation failure after start-up, a
 * latency-bound loop where cudaMalloc/cudaFree would stall on a device-wide
 * synchronisation.  Instead of runtime-owned scratch it uses a fixed array in
 * the library's device memory: 4 * (UHS_NOALLOC_MAX_PARTIALS + 1) doubles,
 * 256 KiB, held on every GPU that loads the library until the process exits.
 * The call allocates and frees nothing.  Its first call on a device looks up the
 * array's device address (a set-up that loads the library's device code on
 * that device if it is not loaded yet), so make that first call before any
 * stream capture.  The address is kept for the device's context and looked
 * up again after the context is destroyed and re-created (cudaDeviceReset).  All calls on a device share the one array; each call
 * rewrites every slot it reads, so nothing carries over between calls, but
 * calls whose kernels overlap on the GPU (other streams, other host threads)
 * race on it: serialise them.  Returns after the stream drained, out filled. */
int uhs_error_norms_noalloc(const uhs_stencil_desc *desc, const uhs_memref *x, const uhs_memref *ref,
                            double out[4], void *stream);

/* ---- batches: many programs advanced together -------------------------- */
/* A batch runs n programs (each its own grids a[i], b[i], descriptor and T)
 * with one persistent kernel launch per timestep.  Every grid is cut into
 * work items (tile x z-chunk; the z-chunks sized from the batch's total
 * work so that no item is much longer than a CTA's share), the items are
 * listed costliest first, and the launch's CTAs take them through an atomic
 * counter.  Each item is swept by its grid's variant (star/box, radius 1-3,
 * rank 2/3, FP64 in float pairs or native, FP32; boxes term by term, not as
 * separable passes).  Grids of 2^21 interior points or more run instead as
 * their own sweep launches with their standalone plan (tuner database or
 * default tile, separable passes for rank-1 boxes), in up to four parallel
 * branches of the same graph, concurrent with the persistent kernel.
 * uhs_batch_create plans the batch, uploads the per-grid arguments, and
 * captures the whole timestep loop (max T launches; a program stops after
 * its own T) and the large grids' sweeps into one CUDA graph; uhs_batch_run
 * replays it on any stream and reports through the batch's own status word.
 * Programs the streaming kernels do not cover (generic shapes,
 * UHS_ARITH_EXACT) are rejected with UHS_EUNSUPPORTED.  The grids must stay
 * allocated for the batch's lifetime.  params (may be NULL) applies to every
 * program; the persistent kernel uses only its arith field. */
typedef struct uhs_batch uhs_batch;

int uhs_batch_create(const uhs_stencil_desc *descs, const uhs_memref *a, const uhs_memref *b, int32_t n,
                     const uhs_params *params, uhs_batch **out);
/* Replay the captured timestep loop on stream; synchronous unless flags has
 * UHS_FLAG_NO_SYNC. */
int uhs_batch_run(uhs_batch *batch, void *stream, int32_t flags);
/* Launches per replay (persistent and large-grid sweeps), timesteps (max
 * T), persistent-kernel work items in the first timestep. */
int uhs_batch_stats(const uhs_batch *batch, int64_t *launches, int64_t *steps, int64_t *items);
void uhs_batch_destroy(uhs_batch *batch);
/* create + run + destroy */
int uhs_run_batch(const uhs_stencil_desc *descs, const uhs_memref *a, const uhs_memref *b, int32_t n,
                  const uhs_params *params, void *stream);

/* ---- tuner database ------------------------------------------------------ */
/* The planner's first source of launch parameters.  Entries are keyed by the
 * program's shape class (rank, star or box, radius), element type and domain
 * extents.  A uhs_run / uhs_sweep whose params are NULL or all zero apart from
 * flags, without UHS_FLAG_NO_TUNE_DB, takes the entry with its exact key, else
 * the entry of the same class and element type nearest in log2 extents, else
 * the planner's defaults.  An entry's float-pair arithmetic is applied as
 * UHS_ARITH_AUTO, so the range check still guards it.  Filled by the tuner
 * (uxxxxxxxxh_gb300/tuner.py, exhaustive search) or the learned cost model. */
int uhs_tune_put(const uhs_stencil_desc *desc, const uhs_params *best, double gstencil_per_s);
/* The parameters the database would give desc (UHS_EINVAL when it has none
 * for the class); *exact is set to 1 for an exact-key hit. */
int uhs_tune_get(const uhs_stencil_desc *desc, uhs_params *out, int32_t *exact);
void uhs_tune_clear(void);
int64_t uhs_tune_size(void);
/* Persist the database as text (written to path.tmp, then renamed) and merge
 * a saved one back.  uhs_tune_load checks the whole file first: a file that
 * does not parse, or holds a field out of range, returns UHS_EPARSE and
 * changes nothing. */
int uhs_tune_save(const char *path);
int uhs_tune_load(const char *path);

/* ---- learned cost model --------------------------------------------------- */
/* A small MLP (in_dim -> hidden x layers (ReLU) -> 1) trained and evaluated by
 * the library's own GPU kernels; the tuner uses it to rank launch candidates
 * of programs it has not timed (uxxxxxxxxh_gb300/costmodel.py).  Parameters
 * are one flat float array, layer by layer [W (out x in, row-major), b (out)].
 * Training minimises the mean squared error with Adam on minibatches drawn by
 * a seeded permutation of a data set copied to the device once. */
typedef struct uhs_mlp uhs_mlp;
int uhs_mlp_create(int32_t in_dim, int32_t hidden, int32_t layers, uint64_t seed, uhs_mlp **out);
void uhs_mlp_destroy(uhs_mlp *m);
int64_t uhs_mlp_num_params(const uhs_mlp *m);
int uhs_mlp_get_params(const uhs_mlp *m, float *out);
int uhs_mlp_set_params(uhs_mlp *m, const float *in);
/* y[i] = net(x[i]) for n rows of in_dim floats (host arrays). */
int uhs_mlp_forward(uhs_mlp *m, const float *x, int32_t n, float *y);
/* Mean squared error of the n rows against y and its gradient with respect
 * to every parameter (host arrays; grad has uhs_mlp_num_params entries). */
int uhs_mlp_loss_grad(uhs_mlp *m, const float *x, const float *y, int32_t n, float *loss, float *grad);
int uhs_mlp_train(uhs_mlp *m, const float *x, const float *y, int32_t n, int32_t epochs, int32_t batch, float lr,
                  uint64_t seed, float *final_loss);

/* Number of kernels this library launched since load (diagnostics). */
int64_t uhs_launch_count(void);

/* Return the device memory the library's scratch pools keep for reuse (the
 * float-pair copies of pair-resident runs) to the driver, on every device
 * used so far.  Memory of runs still in flight is released when they end. */
int uhs_release_scratch(void);

/* Diagnostics: exercise the failure-reporting path.  Launches one CTA whose
 * mbarrier wait can never complete, bounded at `cycles` SM clocks (1 to 2^31;
 * 2^31 is the sweep kernels' bound, about one second at 2 GHz).  When the
 * bound runs out the kernel records a timeout in the device status word the
 * way the sweep kernels' bounded waits do and returns normally -- nothing
 * faults and the device stays usable.  Returns UHS_ETIMEOUT with the message
 * the sweeps would give, after the stream drained. */
int uhs_probe_wait_timeout(int64_t cycles, void *stream);

/* Diagnostics: the FP64 pipe's rate on the current device, in DFMA per
 * second -- the ceiling of a sweep in native FP64 arithmetic, which issues
 * one DFMA per term and point.  Every SM runs independent DFMA chains for
 * about 20 ms, timed with CUDA events on stream; returns after that. */
int uhs_probe_dfma_rate(double *per_second, void *stream);

/* Diagnostics: fail every library-owned device allocation larger than
 * `bytes` as an out-of-memory would (0 removes the cap), so callers can test
 * their handling of UHS_ENOMEM.  Allocations already made are kept. */
int uhs_set_alloc_cap(int64_t bytes);

#ifdef __cplusplus
}
#endif
#endif /* UHS_H_ */
