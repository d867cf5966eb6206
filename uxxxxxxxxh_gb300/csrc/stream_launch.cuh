// Launch side of the streaming kernels: argument packing and the table of
// compiled variants.  Included by the per-storage translation units
// (stream_*.cu), which instantiate the variants in parallel builds.
#pragma once
#include <cstring>

#include "stream_call.h"
#include "stream_kernel.cuh"

namespace uhs {

template <class C>
cudaError_t launch_cfg(const StreamCall &c) {
    StreamArgs<C::NT> a;
    std::memset(&a, 0, sizeof a);
    if (c.tmap) a.tmap = *c.tmap;
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
    a.shift = c.shift;
    a.pair_loads = c.pair_loads;
    a.pair_shift = c.pair_shift;
    a.xoff = C::VX == 2 ? c.xoff : 0;
    a.err = c.err;
    fill_coefs(a.cd, a.chl, a.cl_sum, c.coef, C::NT, c.shape, c.R);
    fill_coef_abs(a.cab, a.chl, C::NT);
    const int64_t nz = c.ub[0] - c.lb[0], ny = c.ub[1] - c.lb[1], nx = c.ub[2] - c.lb[2];
    if (!c.occ_out && (nz <= 0 || ny <= 0 || nx <= 0)) return cudaSuccess;
    void (*kern)(const StreamArgs<C::NT>);
    if constexpr (stream_occ4<C>()) kern = k_stream_occ4<C>;
    else kern = k_stream<C>;
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    if (c.occ_out) {
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(c.occ_out, kern, C::THREADS, C::SMEM);
    }
    dim3 grid(static_cast<unsigned>((nx + a.xoff + C::CX - 1) / C::CX), static_cast<unsigned>((ny + C::BY - 1) / C::BY),
              static_cast<unsigned>((nz + c.zchunk - 1) / c.zchunk));
    kern<<<grid, dim3(C::BX, C::TYT), C::SMEM, c.stream>>>(a);
    count_launch();
    return cudaGetLastError();
}

template <int SHAPE, int R, int ST, int AR, int LD>
cudaError_t dispatch_tile(const StreamCall &c) {
    constexpr bool is2d = ShapeInfo<SHAPE, R>::is2d;
    if constexpr (is2d && ShapeInfo<SHAPE, R>::star && (ST == kStF32 || ST == kStF32x2)) {
        // lane-shuffle variants: the default strips of FP32 (256, cp.async)
        // and float-pair grids (128)
        if (c.xshuffle) {
            if constexpr (ST == kStF32 && LD == kLdCpAsync)
                return c.tile == 2 ? launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 256, 1, 1, 4, 1>>(c)
                                   : cudaErrorInvalidValue;
            else if constexpr (ST == kStF32x2)
                return c.tile == 0 ? launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 128, 1, 1, 4, 1>>(c)
                                   : cudaErrorInvalidValue;
            else
                return cudaErrorInvalidValue;
        }
    }
    if constexpr (is2d) {
        constexpr int PD = 4;
        // two points along x: stars in float arithmetic (FP32, float pairs)
        constexpr bool VX2 = ShapeInfo<SHAPE, R>::star && (ST == kStF32 || AR == kArDf32);
        switch (c.tile) {
            case 3:
                if constexpr (VX2) return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 64, 1, 1, PD, 0, 2>>(c);
                else return cudaErrorInvalidValue;
            case 4:
                if constexpr (VX2 && LD == kLdCpAsync)
                    return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 128, 1, 1, PD, 0, 2>>(c);
                else return cudaErrorInvalidValue;
            case 1: return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 64, 1, 1, PD>>(c);
            case 2:
                if constexpr (LD == kLdCpAsync) return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 256, 1, 1, PD>>(c);
                else return cudaErrorInvalidValue;
            default: return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 128, 1, 1, PD>>(c);
        }
    } else {
        constexpr int PD = 3;
        constexpr bool big_box = (SHAPE == kBox3 && R >= 2);
        if constexpr (big_box) {
            return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 32, 8, 2, 2>>(c);
        } else {
            switch (c.tile) {
                case 4:  // FP32 stars only: 8 points per thread along y
                    if constexpr (ST == kStF32 && SHAPE == kStar3)
                        return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 32, 4, 8, PD>>(c);
                    else
                        return cudaErrorInvalidValue;
                case 1: return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 32, 4, 4, PD>>(c);
                case 2: return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 64, 4, 2, PD>>(c);
                case 3: return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 32, 8, 2, PD>>(c);
                default: return launch_cfg<StreamCfg<SHAPE, R, ST, AR, LD, 32, 8, 4, PD>>(c);
            }
        }
    }
}

template <int SHAPE, int R, int ST, int AR>
cudaError_t dispatch_loader(const StreamCall &c) {
    return c.ld == kLdTma ? dispatch_tile<SHAPE, R, ST, AR, kLdTma>(c) : dispatch_tile<SHAPE, R, ST, AR, kLdCpAsync>(c);
}

template <int ST, int AR, bool IS2D>
cudaError_t dispatch_shape(const StreamCall &c) {
    constexpr int STAR = IS2D ? kStar2 : kStar3, BOX = IS2D ? kBox2 : kBox3, SEP = IS2D ? kSep2 : kSep3;
    const int fam = (c.shape == kStar2 || c.shape == kStar3) ? 0 : (c.shape == kSep2 || c.shape == kSep3) ? 2 : 1;
    switch (c.R * 3 + fam) {
        case 3: return dispatch_loader<STAR, 1, ST, AR>(c);
        case 4: return dispatch_loader<BOX, 1, ST, AR>(c);
        case 5: return dispatch_loader<SEP, 1, ST, AR>(c);
        case 6: return dispatch_loader<STAR, 2, ST, AR>(c);
        case 7: return dispatch_loader<BOX, 2, ST, AR>(c);
        case 8: return dispatch_loader<SEP, 2, ST, AR>(c);
        case 9: return dispatch_loader<STAR, 3, ST, AR>(c);
        case 10: return dispatch_loader<BOX, 3, ST, AR>(c);
        case 11: return dispatch_loader<SEP, 3, ST, AR>(c);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace uhs
