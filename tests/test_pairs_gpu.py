"""Pair-resident runs: FP64 programs of T >= 8 float-pair sweeps run on
float-pair copies of their grids (split once, T sweeps on pairs, domain joined
back).  Both grids must match the oracle within 1e-12 after T steps, with the
halo bit-exact, on 2D and 3D stars of radius 1-3 and boxes (separable and
term by term), on strided grids whose halos differ between a and b, with the
in-place path (UHS_FLAG_IN_PLACE) and with the fallback when the scratch
cannot be allocated."""
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib
from gpu_util import assert_f64_close, assert_halo_exact, run_gpu, run_oracle
from uxxxxxxxxh_gb300.workloads import random_case

pytestmark = pytest.mark.gpu


def _separable_box(rank, r, interior, T, seed):
    """A rank-1 box (swept as 1D passes) on random_case's data."""
    from uxxxxxxxxh_gb300.stencil import box_offsets, make_stencil
    _, a0 = random_case(rank, r, "box", interior, T, seed)
    w = [1.0 + abs(d) for d in range(-r, r + 1)]
    offs = box_offsets(rank, r)
    if rank == 3:
        coefs = [w[dz + r] * w[dy + r] * w[dx + r] / sum(w) ** 3 for dz, dy, dx in offs]
    else:
        coefs = [w[dy + r] * w[dx + r] / sum(w) ** 2 for dz, dy, dx in offs]
    return make_stencil(f"sep{rank}d{r}", rank, interior, r, offs, coefs, iterations=T), a0


@pytest.mark.parametrize("rank,r,kind,interior,T", [
    (3, 1, "star", (40, 37, 66), 8),
    (3, 2, "star", (24, 30, 50), 10),
    (3, 3, "star", (12, 14, 30), 8),
    (2, 1, "star", (90, 130), 12),
    (2, 2, "star", (70, 61), 8),
    (2, 3, "star", (40, 50), 8),
    (3, 3, "sep", (14, 15, 20), 8),
    (2, 2, "sep", (60, 44), 8),
    (3, 1, "box", (12, 14, 30), 8),
    (3, 2, "box", (12, 14, 30), 8),
    (2, 2, "box", (40, 50), 8),
])
def test_pair_resident_run_matches_oracle(cuda, rank, r, kind, interior, T):
    if kind == "sep":
        st, a0 = _separable_box(rank, r, interior, T, 70 + r)
        assert uhs.plan(st).factored == 1
    else:
        st, a0 = random_case(rank, r, kind, interior, T, 70 + r)
    b0 = 2.0 * uhs.workloads.splitmix_uniform(170 + r, a0.size) - 1.0  # b's halo differs from a's
    ra, rb = run_oracle(st, a0, b0)
    n0 = uhs.launch_count()
    ga, gb = run_gpu(st, a0, uhs.RunParams(arith=_lib.UHS_ARITH_DF32), b0)
    assert uhs.launch_count() - n0 == T + 4  # two conversions in, T sweeps, two out
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)
    assert_halo_exact(st, ra, ga)
    assert_halo_exact(st, rb, gb)
    # the in-place path: same bar, and within 1e-12 of the pair-resident run
    ia, ib = run_gpu(st, a0, uhs.RunParams(flags=_lib.UHS_FLAG_IN_PLACE), b0)
    assert_f64_close(st, ra, ia)
    assert_f64_close(st, rb, ib)
    assert oracle.error(st, ga, ia)["max_rel"] <= 1e-12


def test_short_runs_sweep_in_place(cuda):
    """Below T = 8 the conversions would cost more than they save: the sweeps
    run on the FP64 grids (T launches) and meet the bar."""
    st, a0 = random_case(3, 3, "star", (12, 14, 30), 6, 63)
    ra, rb = run_oracle(st, a0)
    n0 = uhs.launch_count()
    ga, gb = run_gpu(st, a0, uhs.RunParams(arith=_lib.UHS_ARITH_DF32))
    assert uhs.launch_count() - n0 == 6
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)


def test_pair_resident_run_on_strided_grids(cuda):
    """Grids that are views into larger allocations (row and plane strides
    wider than the extents): the conversions follow the memref strides."""
    import torch
    st, a0 = random_case(3, 1, "star", (18, 20, 30), 8, 81)
    sz = st.sizes
    big_a = torch.zeros((sz[0] + 2, sz[1] + 3, sz[2] + 6), dtype=torch.float64, device="cuda")
    big_b = torch.zeros_like(big_a)
    a = big_a[1:1 + sz[0], 2:2 + sz[1], 4:4 + sz[2]]
    b = big_b[1:1 + sz[0], 2:2 + sz[1], 4:4 + sz[2]]
    a.copy_(torch.from_numpy(a0.reshape(sz)))
    b.copy_(a)
    uhs.run(st, a, b)
    torch.cuda.synchronize()
    ra, rb = run_oracle(st, a0)
    assert_f64_close(st, ra, a.cpu().numpy().reshape(-1))
    assert_f64_close(st, rb, b.cpu().numpy().reshape(-1))
    assert_halo_exact(st, ra, a.cpu().numpy().reshape(-1))
    # the cells around the views were not touched
    mask = torch.ones_like(big_a, dtype=torch.bool)
    mask[1:1 + sz[0], 2:2 + sz[1], 4:4 + sz[2]] = False
    assert not big_a[mask].any() and not big_b[mask].any()


def test_scratch_allocation_failure_falls_back_to_in_place(cuda):
    """With every library allocation above 64 bytes failing, the run sweeps
    the FP64 grids in place and still meets the bar."""
    L = _lib.lib()
    st, a0 = random_case(3, 2, "star", (20, 24, 40), 8, 91)
    ra, rb = run_oracle(st, a0)
    run_gpu(st, a0)  # the stream's status word exists before the cap
    assert L.uhs_set_alloc_cap(64) == _lib.UHS_OK
    try:
        ga, gb = run_gpu(st, a0)
    finally:
        assert L.uhs_set_alloc_cap(0) == _lib.UHS_OK
    assert_f64_close(st, ra, ga)
    assert_f64_close(st, rb, gb)


def _grids_on_device(st, a0):
    import torch
    a = torch.from_numpy(a0.reshape(st.sizes)).cuda()
    return a, a.clone()


def test_float_pair_sweeps_are_what_pair_resident_runs_launch(cuda):
    """T >= 8 launches two conversions in, T sweeps and two conversions out;
    T = 6, or UHS_FLAG_IN_PLACE, launches the T sweeps alone (plus the float
    range scan of UHS_ARITH_AUTO)."""
    import torch
    st, a0 = random_case(3, 1, "star", (16, 16, 32), 8, 95)
    a, b = _grids_on_device(st, a0)
    p = uhs.RunParams(arith=_lib.UHS_ARITH_DF32)
    uhs.run(st, a, b, p)
    n0 = uhs.launch_count()
    uhs.run(st, a, b, p)
    assert uhs.launch_count() - n0 == 8 + 4
    n0 = uhs.launch_count()
    uhs.run(st, a, b, uhs.RunParams(arith=_lib.UHS_ARITH_DF32, flags=_lib.UHS_FLAG_IN_PLACE))
    assert uhs.launch_count() - n0 == 8
    st6 = st.with_(iterations=6)
    n0 = uhs.launch_count()
    uhs.run(st6, a, b, p)
    assert uhs.launch_count() - n0 == 6
    torch.cuda.synchronize()
