// Persistent batched sweep: one launch advances every grid of a batch by one
// timestep, whatever its extents, stencil shape or precision.
//
// The host cuts every grid into work items (tile x z-chunk), lists them
// costliest first, and launches one CTA per resident slot (SMs x occupancy).
// Each CTA takes the next item from a per-launch counter, copies the item's
// grid arguments (pointers,
// strides, domain, coefficients) into shared memory and runs the streaming
// sweep body of that grid's variant (stream_item), chosen from a compile-time
// pack of variants: all 12 shapes in float-pair FP64 and native FP32 in one
// kernel, native FP64 in another.  All variants use 256 threads and the
// cp.async loader, so the pack shares one block shape; shared memory is sized
// for the largest variant.  A batch's T-step loop is captured once into a CUDA
// graph by the runtime and replayed.
#include "stream_launch.cuh"

namespace uhs {
namespace {

// 256-thread variants: rank 3 r1 box and FP32 r1 star 32x32 (VY 4); other
// rank 3 stars 32x16 (VY 2: a VY 4 register queue of float pairs or doubles
// spills at the pack's 80 registers); r2/r3 box 32x16 (VY 2, PD 2); rank 2
// rows of 256.  batch_tile() gives the host the same tile.
template <int SHAPE, int R, int ST>
constexpr bool batch_vy2() {
    return (SHAPE == kBox3 && R >= 2) || (SHAPE == kStar3 && (ST != kStF32 || R >= 2));
}
template <int SHAPE, int R, int ST, int AR>
using BV = std::conditional_t<
    is_rank2_shape(SHAPE), StreamCfg<SHAPE, R, ST, AR, kLdCpAsync, 256, 1, 1, 4>,
    std::conditional_t<(SHAPE == kBox3 && R >= 2), StreamCfg<SHAPE, R, ST, AR, kLdCpAsync, 32, 8, 2, 2>,
                       std::conditional_t<batch_vy2<SHAPE, R, ST>(),
                                          StreamCfg<SHAPE, R, ST, AR, kLdCpAsync, 32, 8, 2, 3>,
                                          StreamCfg<SHAPE, R, ST, AR, kLdCpAsync, 32, 8, 4, 3>>>>;

template <int ST, int AR>
struct Twelve {
    template <int I>
    using At = BV<(I < 3 ? kStar3 : I < 6 ? kBox3 : I < 9 ? kStar2 : kBox2), I % 3 + 1, ST, AR>;
};

template <class... Cs>
struct Pack {
    static constexpr int N = sizeof...(Cs);
    static constexpr int SMEM = std::max({Cs::SMEM...});
    static constexpr int THREADS = 256;
    static_assert(((Cs::THREADS == 256) && ...), "pack variants share the block shape");
};

template <class T>
struct MainPackOf;
template <int... I>
struct MainPackOf<std::integer_sequence<int, I...>> {
    using type = Pack<typename Twelve<kStF64, kArDf32>::template At<I>...,
                      typename Twelve<kStF32, kArNative>::template At<I>...>;
};
template <class T>
struct NativePackOf;
template <int... I>
struct NativePackOf<std::integer_sequence<int, I...>> {
    using type = Pack<typename Twelve<kStF64, kArNative>::template At<I>...>;
};
using MainPack = MainPackOf<std::make_integer_sequence<int, 12>>::type;
using NativePack = NativePackOf<std::make_integer_sequence<int, 12>>::type;

// Each variant is a separate (not inlined) function, so its registers are
// allocated on its own: the kernel needs the largest variant's count rather
// than what one inlined body holding every variant would keep live.
template <class C>
__device__ __noinline__ void item_call(const BatchArgs &a, int bx, int by, int bz, unsigned char *smem) {
    (void)stream_item<C>(a, bx, by, bz, smem);
}

template <class... Cs>
__device__ __forceinline__ void run_kind(Pack<Cs...>, int kind, const BatchArgs &a, int bx, int by, int bz,
                                         unsigned char *smem) {
    int k = 0;
    ((kind == k++ ? item_call<Cs>(a, bx, by, bz, smem) : (void)0), ...);
}

// Items are fetched dynamically (one atomicAdd per item on a per-launch
// counter): the host orders the list by decreasing estimated cost, so the
// long items start first and the launch ends on short ones.
template <class P>
__global__ void __launch_bounds__(256, 3) k_stream_batch(const BatchGrid *__restrict__ grids,
                                                      const int4 *__restrict__ items, int n_items, int dir,
                                                      int *__restrict__ counter) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ BatchArgs sa;
    __shared__ int skind;
    __shared__ int snext;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (;;) {
        if (tid == 0) snext = atomicAdd(counter, 1);
        __syncthreads();
        const int it = snext;
        if (it >= n_items) break;
        const int4 w = items[it];
        const uint4 *src = reinterpret_cast<const uint4 *>(&grids[w.x].dir[dir]);
        uint4 *dst = reinterpret_cast<uint4 *>(&sa);
        for (int i = tid; i < static_cast<int>(sizeof(BatchArgs) / 16); i += 256) dst[i] = src[i];
        if (tid == 0) skind = grids[w.x].kind;
        __syncthreads();
        run_kind(P{}, skind, sa, w.y, w.z, w.w, smem);
    }
}

int shape_index(int shape, int R) {
    const int base = shape == kStar3 ? 0 : shape == kBox3 ? 3 : shape == kStar2 ? 6 : 9;
    return base + R - 1;
}

template <class P>
cudaError_t prepare(BatchPackInfo *info) {
    static bool done = false;
    static cudaError_t err = cudaSuccess;
    static int occ = 0;
    if (!done) {
        err = cudaFuncSetAttribute(k_stream_batch<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, P::SMEM);
        if (err == cudaSuccess)
            err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_stream_batch<P>, P::THREADS, P::SMEM);
        done = true;
    }
    info->smem = P::SMEM;
    info->threads = P::THREADS;
    info->occ = occ;
    return err;
}

}  // namespace

int batch_kind(int pack, int shape, int R, int st, int ar) {
    if (R < 1 || R > 3) return -1;
    const int i = shape_index(shape, R);
    if (pack == kPackMain) {
        if (st == kStF64 && ar == kArDf32) return i;
        if (st == kStF32 && ar == kArNative) return 12 + i;
        return -1;
    }
    if (pack == kPackF64Native && st == kStF64 && ar == kArNative) return i;
    return -1;
}

// 32-plane z-chunks: longer chunks re-read fewer halo planes but give fewer,
// longer items; on GB300 16, 24, 32 and 16(R+1) planes timed within 2 % on
// the 64-grid suite, and 32 was fastest.
void batch_tile(int shape, int R, int st, int *bx, int *by, int *zchunk) {
    if (is_rank2_shape(shape)) {
        *bx = 256;
        *by = 1;
        *zchunk = 128;
    } else {
        const bool vy2 = (shape == kBox3 && R >= 2) || (shape == kStar3 && (st != kStF32 || R >= 2));
        *bx = 32;
        *by = vy2 ? 16 : 32;
        *zchunk = 32;
    }
}

cudaError_t batch_prepare(int pack, BatchPackInfo *info) {
    return pack == kPackMain ? prepare<MainPack>(info) : prepare<NativePack>(info);
}

cudaError_t batch_launch(int pack, const BatchGrid *grids, const int4 *items, int n_items, int dir, int ctas,
                         int *counter, cudaStream_t st) {
    if (n_items <= 0) return cudaSuccess;
    if (pack == kPackMain)
        k_stream_batch<MainPack><<<ctas, dim3(32, 8), MainPack::SMEM, st>>>(grids, items, n_items, dir, counter);
    else
        k_stream_batch<NativePack><<<ctas, dim3(32, 8), NativePack::SMEM, st>>>(grids, items, n_items, dir, counter);
    count_launch();
    return cudaGetLastError();
}

void batch_fill_args(BatchArgs *a, const StreamCall &c, int nt) {
    std::memset(a, 0, sizeof *a);
    a->in = c.in.data;
    a->out = c.out.data;
    a->in_s0 = c.in.s[0];
    a->in_s1 = c.in.s[1];
    a->out_s0 = c.out.s[0];
    a->out_s1 = c.out.s[1];
    a->n0 = c.in.n[0];
    a->n1 = c.in.n[1];
    a->n2 = c.in.n[2];
    a->lb0 = c.lb[0];
    a->lb1 = c.lb[1];
    a->lb2 = c.lb[2];
    a->ub0 = c.ub[0];
    a->ub1 = c.ub[1];
    a->ub2 = c.ub[2];
    a->zchunk = c.zchunk;
    a->shift = 0;
    a->pair_loads = c.pair_loads;
    a->pair_shift = c.pair_shift;
    a->err = c.err;
    fill_coefs(a->cd, a->chl, a->cl_sum, c.coef, nt < kBatchNT ? nt : kBatchNT, c.shape, c.R);
    fill_coef_abs(a->cab, a->chl, nt < kBatchNT ? nt : kBatchNT);
}

}  // namespace uhs
