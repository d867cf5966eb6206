"""Parity of the 2.5D streaming kernels (UHS_KERNEL_STREAM) with the oracle.

FP64 grids in FMA or float-pair (df32) arithmetic must stay within a max
error of 1e-12 relative to the field's largest magnitude after T steps, the
halo bit-exact; FP32 grids within a relative L2 error of 1e-6 of the FP64
oracle; float-pair grids (UHS_F32X2) within 1e-12.  Both loaders (TMA tensor
copies and cp.async) and every tile variant are exercised.
"""
import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib
from gpu_util import assert_f64_close, assert_halo_exact, run_gpu, run_oracle
from uxxxxxxxxh_gb300.workloads import random_case

pytestmark = pytest.mark.gpu

ODD_3D = (21, 35, 70)
ODD_2D = (133, 301)
STREAM = uhs.UHS_KERNEL_STREAM


def _case(rank, r, kind, T=4, seed=7, interior=None):
    interior = interior or (ODD_3D if rank == 3 else ODD_2D)
    return random_case(rank, r, kind, interior, T, seed)


@pytest.mark.parametrize("arith", [uhs.UHS_ARITH_FMA, uhs.UHS_ARITH_DF32])
@pytest.mark.parametrize("use_tma", [1, -1])
@pytest.mark.parametrize("rank,r,kind", uhs.SHAPES)
def test_stream_f64(cuda, rank, r, kind, arith, use_tma):
    # TMA needs 16-byte row pitches: an even padded row length for doubles
    interior = None if use_tma < 0 or rank == 3 else (ODD_2D[0], ODD_2D[1] + 1)
    st, a0 = _case(rank, r, kind, interior=interior)
    ra, rb = run_oracle(st, a0)
    p = uhs.RunParams(kernel=STREAM, arith=arith, use_tma=use_tma)
    assert uhs.plan(st, params=p).kernel == STREAM
    ga, gb = run_gpu(st, a0, p)
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)
    assert_halo_exact(st, ra, ga)
    assert_halo_exact(st, rb, gb)


@pytest.mark.parametrize("rank,r,kind", uhs.SHAPES)
def test_stream_f32(cuda, rank, r, kind):
    import torch
    st, a0 = _case(rank, r, kind)
    a32 = a0.astype(np.float32)
    ra, _ = run_oracle(st, a32.astype(np.float64))
    st32 = st.with_(dtype=uhs.UHS_F32)
    ga, _ = run_gpu(st32, a32, uhs.RunParams(kernel=STREAM), dtype=torch.float32)
    e = oracle.error(st, ra, ga)
    assert e["l2_rel"] <= 1e-6, e
    assert oracle.halo_diff(st32, a32, ga) == 0


@pytest.mark.parametrize("r", [1, 2, 3])
def test_stream_f32_star_vy8(cuda, r):
    """The FP32 star tile with 8 points per thread along y (32 x 4 threads),
    ragged in y and x; the planner refuses it for other shapes and types."""
    import torch
    st, a0 = random_case(3, r, "star", (21, 45, 70), 6, 60 + r)
    a32 = a0.astype(np.float32)
    ra, _ = run_oracle(st, a32.astype(np.float64))
    st32 = st.with_(dtype=uhs.UHS_F32)
    p = uhs.RunParams(kernel=STREAM, tile_x=32, tile_y=32, vy=8)
    assert uhs.plan(st32, params=p).vy == 8
    ga, _ = run_gpu(st32, a32, p, dtype=torch.float32)
    e = oracle.error(st, ra, ga)
    assert e["l2_rel"] <= 1e-6, e
    assert oracle.halo_diff(st32, a32, ga) == 0
    with pytest.raises(uhs.UhsError):
        uhs.plan(st, params=p)  # FP64
    stb, _ = random_case(3, 1, "box", (8, 8, 32), 2, 63, dtype=uhs.UHS_F32)
    with pytest.raises(uhs.UhsError):
        uhs.plan(stb, params=p)


def _pairs(a: np.ndarray) -> np.ndarray:
    hi = a.astype(np.float32)
    lo = (a - hi.astype(np.float64)).astype(np.float32)
    return np.stack([hi, lo], axis=-1).reshape(-1).view(np.float64)


def _unpair(p: np.ndarray) -> np.ndarray:
    f = p.view(np.float32).reshape(-1, 2).astype(np.float64)
    return f[:, 0] + f[:, 1]


@pytest.mark.parametrize("rank,r,kind", [(3, 1, "star"), (3, 2, "box"), (2, 3, "star"), (2, 1, "box")])
@pytest.mark.parametrize("use_tma", [1, -1])
def test_stream_f32x2_pairs(cuda, rank, r, kind, use_tma):
    interior = None if use_tma < 0 or rank == 3 else (ODD_2D[0], ODD_2D[1] + 1)
    st, a0 = _case(rank, r, kind, interior=interior)
    pairs = _pairs(a0)
    start = _unpair(pairs)
    ra, _ = run_oracle(st, start)
    stp = st.with_(dtype=uhs.UHS_F32X2)
    ga, _ = run_gpu(stp, pairs, uhs.RunParams(kernel=STREAM, use_tma=use_tma))
    assert_f64_close(st, ra, _unpair(ga))
    assert oracle.halo_diff(stp, pairs, ga) == 0


@pytest.mark.parametrize("tile_x,tile_y,vy", [(32, 32, 4), (32, 16, 4), (64, 8, 2), (32, 16, 2)])
@pytest.mark.parametrize("arith", [uhs.UHS_ARITH_FMA, uhs.UHS_ARITH_DF32])
def test_stream_tile_variants_3d(cuda, tile_x, tile_y, vy, arith):
    st, a0 = _case(3, 2, "star", T=2, interior=(40, 37, 130))
    ra, _ = run_oracle(st, a0)
    for tma in (1, -1):
        p = uhs.RunParams(kernel=STREAM, arith=arith, tile_x=tile_x, tile_y=tile_y, vy=vy, use_tma=tma)
        got = uhs.plan(st, params=p)
        assert (got.tile_x, got.tile_y, got.vy) == (tile_x, tile_y, vy)
        ga, _ = run_gpu(st, a0, p)
        assert_f64_close(st, ra, ga)


@pytest.mark.parametrize("tile_x", [64, 128, 256])
def test_stream_tile_variants_2d(cuda, tile_x):
    st, a0 = _case(2, 1, "box", T=2, interior=(90, 1000))
    ra, _ = run_oracle(st, a0)
    ga, _ = run_gpu(st, a0, uhs.RunParams(kernel=STREAM, tile_x=tile_x))
    assert_f64_close(st, ra, ga)


def test_stream_offset_domain_exercises_tma_shift(cuda):
    """Domain starting one cell past the halo: the TMA box start is rounded
    down to its 16-byte granule and the kernel indexes from the remainder."""
    st, a0 = _case(3, 1, "star", T=2, interior=(12, 20, 50))
    st = st.with_(lb=(1, 1, 2), ub=(st.ub[0], st.ub[1], st.ub[2] - 3))
    ra, _ = run_oracle(st, a0)
    for arith in (uhs.UHS_ARITH_FMA, uhs.UHS_ARITH_DF32):
        ga, _ = run_gpu(st, a0, uhs.RunParams(kernel=STREAM, arith=arith, use_tma=1))
        assert_f64_close(st, ra, ga)
        assert_halo_exact(st, ra, ga)


def test_stream_z_chunks_and_small_grids(cuda):
    for interior, tz in [((1, 1, 1), 0), ((5, 3, 33), 1), ((64, 8, 40), 7), ((30, 30, 30), 1000)]:
        st, a0 = random_case(3, 3, "star", interior, 2, 3)
        ra, _ = run_oracle(st, a0)
        ga, _ = run_gpu(st, a0, uhs.RunParams(kernel=STREAM, arith=uhs.UHS_ARITH_DF32, tile_z=tz))
        assert_f64_close(st, ra, ga)


def test_df32_range_error_is_reported(cuda):
    st, a0 = _case(3, 1, "star", T=2, interior=(8, 8, 40))
    a0[len(a0) // 2] = 1e300
    with pytest.raises(uhs.UhsError) as ei:
        run_gpu(st, a0, uhs.RunParams(kernel=STREAM, arith=uhs.UHS_ARITH_DF32))
    assert ei.value.code == uhs._lib.UHS_ERANGE
    # the device status word is cleared: a following in-range run succeeds
    st2, b0 = _case(3, 1, "star", T=2, interior=(8, 8, 40))
    ra, _ = run_oracle(st2, b0)
    ga, _ = run_gpu(st2, b0, uhs.RunParams(kernel=STREAM, arith=uhs.UHS_ARITH_DF32))
    assert_f64_close(st2, ra, ga)


def test_df32_handles_zeros_tiny_and_negative_values(cuda):
    st, a0 = _case(3, 1, "box", T=2, interior=(10, 10, 40))
    a0[::7] = 0.0
    a0[1::11] = -a0[1::11]
    a0[2::13] *= 1e-30
    ra, _ = run_oracle(st, a0)
    ga, _ = run_gpu(st, a0, uhs.RunParams(kernel=STREAM, arith=uhs.UHS_ARITH_DF32))
    assert_f64_close(st, ra, ga)


def test_forced_tma_on_unaligned_rows_is_refused(cuda):
    st, a0 = _case(2, 1, "star", interior=(20, 301))  # 303 doubles per row
    with pytest.raises(uhs.UhsError) as ei:
        run_gpu(st, a0, uhs.RunParams(kernel=STREAM, use_tma=1))
    assert ei.value.code == uhs._lib.UHS_EUNSUPPORTED


def test_auto_arithmetic_uses_float_pairs_and_falls_back_on_range(cuda):
    st, a0 = _case(3, 1, "star", T=4, interior=(12, 20, 40))
    assert uhs.plan(st).arith == uhs.UHS_ARITH_DF32
    ra, _ = run_oracle(st, a0)
    ga, _ = run_gpu(st, a0)  # UHS_ARITH_AUTO
    assert_f64_close(st, ra, ga)
    # a value near the float-pair limit: AUTO must run native FP64 instead of failing
    a1 = a0.copy()
    a1[len(a1) // 2] = 1e36
    ra1, _ = run_oracle(st, a1)
    ga1, _ = run_gpu(st, a1)
    assert_f64_close(st, ra1, ga1)
    # growth bound: coefficients summing to 2.8 over T = 200 steps exceed 2^128
    st2 = st.with_(terms=[(t[0], t[1], t[2], 0.4) for t in st.terms], iterations=2)
    ra2, _ = run_oracle(st2, a0)
    ga2, _ = run_gpu(st2, a0)
    assert_f64_close(st2, ra2, ga2)


def test_f32_pair_loads_and_single_loads_agree(cuda):
    """Even pitches take the 8-byte cp.async path, odd ones the 4-byte path."""
    import torch
    for interior in [(9, 20, 64), (9, 20, 63)]:
        st, a0 = _case(3, 2, "star", T=2, interior=interior)
        st32 = st.with_(dtype=uhs.UHS_F32)
        a32 = a0.astype(np.float32)
        ra, _ = run_oracle(st, a32.astype(np.float64))
        ga, _ = run_gpu(st32, a32, uhs.RunParams(kernel=STREAM, use_tma=-1), dtype=torch.float32)
        assert oracle.error(st, ra, ga)["l2_rel"] <= 1e-6


@pytest.mark.parametrize("r", [1, 2, 3])
@pytest.mark.parametrize("dtype", ["f32", "f32x2"])
def test_lane_shuffle_rank2_stars(cuda, r, dtype):
    """UHS_FLAG_XSHUFFLE: x-neighbours of rank-2 stars from the adjacent lanes
    by warp shuffles (edge lanes from shared memory).  The same terms in the
    same order as the shared-memory sweep: bit-identical to it, and within
    the element type's bar of the oracle."""
    import numpy as np
    import torch
    st, a0 = random_case(2, r, "star", (157, 700), 4, 90 + r)
    if dtype == "f32":
        st = st.with_(dtype=_lib.UHS_F32)
        data, tdt = a0.astype(np.float32), torch.float32
    else:
        hi = a0.astype(np.float32)
        lo = (a0 - hi.astype(np.float64)).astype(np.float32)
        data, tdt = np.stack([hi, lo], -1).reshape(-1).view(np.float64), torch.float64
        st = st.with_(dtype=_lib.UHS_F32X2)
    flags = _lib.UHS_FLAG_XSHUFFLE
    assert uhs.plan(st, None, uhs.RunParams(flags=flags)).tile_x == (256 if dtype == "f32" else 128)
    outs = []
    for f in (0, flags):
        p = uhs.RunParams(kernel=STREAM, tile_x=256 if dtype == "f32" else 128, vx=1,
                          use_tma=-1 if dtype == "f32" else 0, flags=f | _lib.UHS_FLAG_NO_TUNE_DB)
        outs.append(run_gpu(st, data, p, dtype=tdt))
    for x, y in zip(outs[0], outs[1]):
        assert np.array_equal(x.view(np.uint32 if dtype == "f32" else np.uint64),
                              y.view(np.uint32 if dtype == "f32" else np.uint64))
    ra, _ = run_oracle(st, a0 if dtype == "f32x2" else a0.astype(np.float32).astype(np.float64))
    got = outs[1][0]
    if dtype == "f32x2":
        got = got.view(np.float32).reshape(-1, 2).astype(np.float64).sum(1)
        assert oracle.error(st, ra, got)["max_rel"] <= 1e-12
    else:
        assert oracle.error(st, ra, got.astype(np.float64))["l2_rel"] <= 1e-6


@pytest.mark.parametrize("r", [1, 2, 3])
@pytest.mark.parametrize("dtype", ["f32", "f32x2", "f64"])
@pytest.mark.parametrize("tile_x,use_tma", [(128, 0), (128, -1), (256, -1)])
def test_two_points_along_x_rank2_stars(cuda, r, dtype, tile_x, use_tma):
    """vx = 2: each thread sweeps two adjacent columns of a rank-2 star
    (float pairs: the two points' sums packed).  Per point the same terms in
    the same order and the same roundings as one point per thread: bit-
    identical to it, on odd widths whose rows alternate between 2-point
    vector stores and single stores, and within the element type's bar of
    the oracle."""
    import torch
    # odd rows (cp.async): row starts alternate in alignment; even rows let TMA load
    st, a0 = random_case(2, r, "star", (157, 702 if use_tma == 0 else 701), 4, 120 + r)
    tdt = torch.float64
    if dtype == "f32":
        st = st.with_(dtype=_lib.UHS_F32)
        data, tdt, arith = a0.astype(np.float32), torch.float32, uhs.UHS_ARITH_FMA
    elif dtype == "f32x2":
        hi = a0.astype(np.float32)
        lo = (a0 - hi.astype(np.float64)).astype(np.float32)
        data = np.stack([hi, lo], -1).reshape(-1).view(np.float64)
        st, arith = st.with_(dtype=_lib.UHS_F32X2), uhs.UHS_ARITH_DF32
    else:
        data, arith = a0, uhs.UHS_ARITH_DF32
    base = dict(kernel=STREAM, arith=arith, use_tma=use_tma, flags=_lib.UHS_FLAG_NO_TUNE_DB)
    one = uhs.RunParams(**base, tile_x=128 if tile_x == 128 else 256 if dtype == "f32" else 128)
    two = uhs.RunParams(**base, tile_x=tile_x, vx=2)
    pl = uhs.plan(st, None, two)
    assert (pl.vx, pl.tile_x) == (2, tile_x)
    outs = [run_gpu(st, data, p, dtype=tdt) for p in (one, two)]
    u = np.uint32 if dtype == "f32" else np.uint64
    for x, y in zip(outs[0], outs[1]):
        assert np.array_equal(x.view(u), y.view(u))
    ra, _ = run_oracle(st, a0 if dtype != "f32" else a0.astype(np.float32).astype(np.float64))
    got = outs[1][0]
    if dtype == "f32x2":
        got = got.view(np.float32).reshape(-1, 2).astype(np.float64).sum(1)
        assert oracle.error(st, ra, got)["max_rel"] <= 1e-12
    elif dtype == "f64":
        assert_f64_close(st, ra, got)
        assert_halo_exact(st, ra, got)
    else:
        assert oracle.error(st, ra, got.astype(np.float64))["l2_rel"] <= 1e-6


@pytest.mark.parametrize("r", [1, 3])
def test_two_points_along_x_pair_resident(cuda, r):
    """vx = 2 carried into the float-pair sweeps of a pair-resident FP64 run
    (T = 8): bit-identical to one point per thread."""
    st, a0 = random_case(2, r, "star", (211, 503), 8, 140 + r)
    outs = [run_gpu(st, a0, uhs.RunParams(kernel=STREAM, flags=_lib.UHS_FLAG_NO_TUNE_DB, **kw))
            for kw in ({}, {"vx": 2, "tile_x": 256})]
    for x, y in zip(outs[0], outs[1]):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64))
    ra, _ = run_oracle(st, a0)
    assert_f64_close(st, ra, outs[1][0])
