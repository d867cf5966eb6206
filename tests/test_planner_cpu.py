"""The planner's default launches (no parameters, no tuner database), planned
on the host: the per-class tiles chosen from timing the defaults against
exhaustive tuning on GB300, and that a caller's tile overrides them.  The
z-chunk caps act at launch time; `tile_z` stays 0 (automatic) in the plan."""
import pytest

from uxxxxxxxxh_gb300 import _lib
from uxxxxxxxxh_gb300.runtime import RunParams, memref_raw, plan
from uxxxxxxxxh_gb300.stencil import box_offsets, make_stencil
from uxxxxxxxxh_gb300.workloads import cfg3, random_case

F = _lib
NO_DB = RunParams(flags=F.UHS_FLAG_NO_TUNE_DB)


def planned(st):
    p = plan(st, memref_raw(1 << 20, st.sizes), params=NO_DB)
    return p.tile_x, p.tile_y, p.vy


def separable_box(r, dtype):
    """A rank-1 box (the planner sweeps it as 1D passes)."""
    w = [1.0 + abs(d) for d in range(-r, r + 1)]
    offs = box_offsets(3, r)
    coefs = [w[dz + r] * w[dy + r] * w[dx + r] / sum(w) ** 3 for dz, dy, dx in offs]
    return make_stencil(f"sep{r}", 3, (96, 96, 96), r, offs, coefs, dtype=dtype)


@pytest.mark.parametrize("r,want", [(1, (32, 16, 4)), (2, (32, 16, 4)), (3, (32, 16, 4))])
def test_float_pair_stars(r, want):
    st, _ = random_case(3, r, "star", (64, 64, 64), 2, 1)
    assert planned(st) == want


@pytest.mark.parametrize("r", [1, 2, 3])
def test_float_pair_grid_stars(r):
    """Float-pair grids (the sweeps of pair-resident runs) take 32 x 16 tiles
    of 4 points per thread for every radius."""
    st, _ = random_case(3, r, "star", (64, 64, 64), 2, 1, dtype=F.UHS_F32X2)
    assert planned(st) == (32, 16, 4)


@pytest.mark.parametrize("r,want", [(1, (32, 16, 4)), (2, (32, 16, 4)), (3, (32, 16, 4))])
def test_float_pair_separable_boxes(r, want):
    st = separable_box(r, F.UHS_F64)
    assert plan(st, memref_raw(1 << 20, st.sizes), params=NO_DB).factored == 1
    assert planned(st) == want


def test_float_pair_term_by_term_boxes():
    st, _ = random_case(3, 1, "box", (64, 64, 64), 2, 2)
    assert planned(st) == (32, 16, 4)
    st, _ = random_case(3, 3, "box", (64, 64, 64), 2, 3)
    assert planned(st) == (32, 16, 2)  # radius 2-3 boxes have one tile


@pytest.mark.parametrize("r,rows,want", [(1, 512, (32, 16, 4)), (2, 512, (32, 32, 4)), (2, 294, (32, 16, 4)),
                                         (3, 512, (32, 16, 4))])
def test_fp32_stars(r, rows, want):
    """Radius 2 takes 32-row tiles only when they leave at most 2 % of the
    rows idle (294 rows: 10 tiles of 32 would cover 320)."""
    st, _ = random_case(3, r, "star", (64, rows, 96), 2, 4, dtype=F.UHS_F32)
    assert planned(st) == want


def test_fp32_separable_box_and_2d_strips():
    st, _ = cfg3(n=64)
    st = st.with_(dtype=F.UHS_F32)
    assert planned(st) == (32, 16, 4)
    for r, kind in ((1, "star"), (3, "box")):
        st, _ = random_case(2, r, kind, (300, 700), 2, 5, dtype=F.UHS_F32)
        assert planned(st)[0] == 256
        # FP64 grids in float pairs: boxes 128-wide strips; stars swept in
        # place two points per thread over 256 columns (cp.async)
        st64 = st.with_(dtype=F.UHS_F64)
        p = plan(st64, memref_raw(1 << 20, st64.sizes), params=NO_DB)
        assert (p.tile_x, p.vx) == ((256, 2) if kind == "star" else (128, 1))


def test_float_pair_2d_term_by_term_boxes_load_by_cp_async():
    st, _ = random_case(2, 2, "box", (300, 700), 2, 6)
    p = plan(st, memref_raw(1 << 20, st.sizes), params=NO_DB)
    assert p.use_tma == -1
    # stars on float-pair grids take TMA (128 columns, two points per thread)
    star, _ = random_case(2, 2, "star", (300, 700), 2, 6, dtype=F.UHS_F32X2)
    assert plan(star, memref_raw(1 << 20, star.sizes), params=NO_DB).use_tma == 1


def test_caller_tiles_override_the_defaults():
    st, _ = random_case(3, 1, "star", (64, 64, 64), 2, 7)
    p = plan(st, memref_raw(1 << 20, st.sizes),
             params=RunParams(tile_x=32, tile_y=32, vy=4, tile_z=24, flags=F.UHS_FLAG_NO_TUNE_DB))
    assert (p.tile_x, p.tile_y, p.vy, p.tile_z) == (32, 32, 4, 24)


def test_prefetch_is_the_built_depth():
    """Load-ahead depth is built into each variant: the plan reports it, a
    caller may repeat it, any other value is refused."""
    st, _ = random_case(3, 1, "star", (32, 32, 32), 2, 8)
    assert plan(st, params=NO_DB).prefetch == 3
    assert plan(st, params=RunParams(prefetch=3, flags=F.UHS_FLAG_NO_TUNE_DB)).prefetch == 3
    with pytest.raises(_lib.UhsError) as ei:
        plan(st, params=RunParams(prefetch=2, flags=F.UHS_FLAG_NO_TUNE_DB))
    assert ei.value.code == F.UHS_EUNSUPPORTED
    big_box, _ = random_case(3, 3, "box", (32, 32, 32), 2, 9)
    assert plan(big_box, params=NO_DB).prefetch == 2
    strip, _ = random_case(2, 2, "star", (64, 64), 2, 10)
    assert plan(strip, params=NO_DB).prefetch == 4
    gen = dict(kernel=F.UHS_KERNEL_GENERIC, arith=F.UHS_ARITH_FMA, flags=F.UHS_FLAG_NO_TUNE_DB)
    assert plan(st, params=RunParams(**gen)).use_tma == -1
    assert plan(st, params=RunParams(prefetch=1, **gen)).kernel == F.UHS_KERNEL_GENERIC
    for bad in (dict(prefetch=3), dict(use_tma=1)):
        with pytest.raises(_lib.UhsError) as ei:
            plan(st, params=RunParams(**bad, **gen))
        assert ei.value.code == F.UHS_EUNSUPPORTED


def test_lane_shuffle_flag_is_for_rank2_stars():
    """UHS_FLAG_XSHUFFLE plans the 256-wide FP32 strip (128 for float pairs)
    and is refused for other shapes, element types and strip widths."""
    st, _ = random_case(2, 2, "star", (300, 700), 2, 11, dtype=F.UHS_F32)
    assert plan(st, memref_raw(1 << 20, st.sizes), params=RunParams(flags=F.UHS_FLAG_XSHUFFLE | F.UHS_FLAG_NO_TUNE_DB)).tile_x == 256
    for bad in (random_case(3, 1, "star", (40, 40, 40), 2, 12, dtype=F.UHS_F32)[0],
                random_case(2, 1, "box", (300, 700), 2, 13, dtype=F.UHS_F32)[0],
                random_case(2, 1, "star", (300, 700), 2, 14)[0].with_(dtype=F.UHS_F64)):
        with pytest.raises(F.UhsError):
            plan(bad, memref_raw(1 << 20, bad.sizes), params=RunParams(arith=F.UHS_ARITH_FMA,
                                                                        flags=F.UHS_FLAG_XSHUFFLE | F.UHS_FLAG_NO_TUNE_DB))
    with pytest.raises(F.UhsError):
        plan(st, memref_raw(1 << 20, st.sizes), params=RunParams(tile_x=64, flags=F.UHS_FLAG_XSHUFFLE | F.UHS_FLAG_NO_TUNE_DB))


def test_two_points_along_x_is_for_rank2_stars():
    """vx = 2 plans the 256-column tile (128 threads, cp.async) by default and
    the 128-column one on request, for rank-2 stars on FP32 grids or in float
    pairs; it is refused for rank-3 grids, boxes, native FP64, other widths,
    and with lane shuffles."""
    st, _ = random_case(2, 2, "star", (300, 700), 2, 11, dtype=F.UHS_F32)
    raw = memref_raw(1 << 20, st.sizes)
    p = plan(st, raw, params=RunParams(vx=2, flags=F.UHS_FLAG_NO_TUNE_DB))
    assert (p.vx, p.tile_x, p.use_tma) == (2, 256, -1)
    p = plan(st, raw, params=RunParams(vx=2, tile_x=128, flags=F.UHS_FLAG_NO_TUNE_DB))
    assert (p.vx, p.tile_x) == (2, 128)
    pairs = st.with_(dtype=F.UHS_F32X2)
    assert plan(pairs, raw, params=RunParams(vx=2, flags=F.UHS_FLAG_NO_TUNE_DB)).vx == 2
    # defaults: float pairs take two points (128 columns by TMA, 256 by
    # cp.async where TMA cannot load the rows); FP32 only radius 2 by TMA
    p = plan(pairs, raw, params=NO_DB)
    assert (p.vx, p.tile_x, p.use_tma) == (2, 128, 1)
    odd = random_case(2, 2, "star", (300, 701), 2, 11, dtype=F.UHS_F32X2)[0]
    p = plan(odd, memref_raw(1 << 20, odd.sizes), params=RunParams(use_tma=-1, flags=F.UHS_FLAG_NO_TUNE_DB))
    assert (p.vx, p.tile_x, p.use_tma) == (2, 256, -1)
    p = plan(st, raw, params=NO_DB)
    assert (p.vx, p.tile_x, p.use_tma) == (2, 128, 1)
    for r in (1, 3):
        s = random_case(2, r, "star", (300, 700), 2, 11, dtype=F.UHS_F32)[0]
        assert plan(s, memref_raw(1 << 20, s.sizes), params=NO_DB).vx == 1
    f64 = st.with_(dtype=F.UHS_F64)
    assert plan(f64, raw, params=RunParams(vx=2, arith=F.UHS_ARITH_DF32, flags=F.UHS_FLAG_NO_TUNE_DB)).vx == 2
    bad_cases = [
        (random_case(3, 1, "star", (40, 40, 40), 2, 12, dtype=F.UHS_F32)[0], {}),
        (random_case(2, 1, "box", (300, 700), 2, 13, dtype=F.UHS_F32)[0], {}),
        (f64, dict(arith=F.UHS_ARITH_FMA)),
        (st, dict(tile_x=64)),
        (st, dict(flags=F.UHS_FLAG_XSHUFFLE)),
    ]
    for bad, kw in bad_cases:
        kw = {**kw, "flags": kw.get("flags", 0) | F.UHS_FLAG_NO_TUNE_DB}
        with pytest.raises(F.UhsError):
            plan(bad, memref_raw(1 << 20, bad.sizes), params=RunParams(vx=2, **kw))
    with pytest.raises(F.UhsError):
        plan(st, raw, params=RunParams(vx=3, flags=F.UHS_FLAG_NO_TUNE_DB))


def test_temporal_fusion_planning():
    """k_temporal 2 and 4 plan for every star and box shape of rank 2 and
    radius-1 shapes of rank 3 (depth 2 for radius 2-3 in 3D); fused boxes are
    summed term by term (not factored); float-pair grids and two points per
    thread along x are refused."""
    for rank, r, kind in [(2, 3, "box"), (2, 1, "star"), (3, 1, "box"), (3, 3, "star")]:
        st, _ = random_case(rank, r, kind, (40, 300) if rank == 2 else (20, 20, 40), 4, 3)
        for k in ((2, 4) if rank == 2 or r == 1 else (2,)):
            p = plan(st, memref_raw(1 << 20, st.sizes), params=RunParams(k_temporal=k, flags=F.UHS_FLAG_NO_TUNE_DB))
            assert (p.k_temporal, p.factored, p.prefetch) == (k, 0, 2)
    st, _ = random_case(3, 2, "box", (20, 20, 40), 4, 3)
    with pytest.raises(F.UhsError):
        plan(st, memref_raw(1 << 20, st.sizes), params=RunParams(k_temporal=4, flags=F.UHS_FLAG_NO_TUNE_DB))
    st, _ = random_case(2, 1, "star", (40, 300), 4, 3)
    for bad in (dict(vx=2), dict(k_temporal=3)):
        with pytest.raises(F.UhsError):
            plan(st, memref_raw(1 << 20, st.sizes), params=RunParams(**{"k_temporal": 2, **bad}))
    with pytest.raises(F.UhsError):
        plan(st.with_(dtype=F.UHS_F32X2), memref_raw(1 << 20, st.sizes), params=RunParams(k_temporal=2))
