"""Batches: many programs advanced by one persistent launch per timestep,
the timestep loop replayed from a CUDA graph.  Every grid of the batch must
match its own oracle run (FP64 within 1e-12, FP32 within a relative L2 of
1e-6), whatever mix of shapes, precisions, extents and T shares the batch."""
import numpy as np
import pytest

import oracle
import uxxxxxxxxh_gb300 as uhs
from gpu_util import assert_f64_close, run_oracle, to_dev
from uxxxxxxxxh_gb300.workloads import cfg5_specs, random_case

pytestmark = pytest.mark.gpu


def _grids(specs):
    import torch
    devs_a, devs_b, host = [], [], []
    for st, seed in specs:
        a0 = 2.0 * uhs.workloads.splitmix_uniform(seed, int(np.prod(st.sizes))) - 1.0
        if st.dtype == uhs.UHS_F32:
            a0 = a0.astype(np.float32).astype(np.float64)
            d = to_dev(a0.astype(np.float32), st, torch.float32)
        else:
            d = to_dev(a0, st)
        devs_a.append(d)
        devs_b.append(d.clone())
        host.append(a0)
    return devs_a, devs_b, host


def _check(specs, devs_a, devs_b, host):
    for (st, _), da, db, a0 in zip(specs, devs_a, devs_b, host):
        ra, rb = run_oracle(st, a0)
        ga = da.cpu().numpy().reshape(-1).astype(np.float64)
        gb = db.cpu().numpy().reshape(-1).astype(np.float64)
        if st.dtype == uhs.UHS_F32:
            assert oracle.error(st, ra, ga)["l2_rel"] <= 1e-6, st.name
            if st.iterations > 1:
                assert oracle.error(st, rb, gb)["l2_rel"] <= 1e-6, st.name
        else:
            assert_f64_close(st, ra, ga)
            assert_f64_close(st, rb, gb)


def test_mixed_batch_matches_oracle(cuda):
    specs = cfg5_specs(n_grids=24, T=4, seed=11, side2=(40, 300), side3=(12, 48))
    kinds = {(st.rank, st.radius[2], st.nterms, st.dtype) for st, _ in specs}
    assert len(kinds) >= 10
    a, b, host = _grids(specs)
    batch = uhs.Batch([s for s, _ in specs], a, b)
    stats = batch.stats()
    assert stats["steps"] == 4 and stats["launches"] >= 4
    batch.run()
    _check(specs, a, b, host)
    batch.close()


def test_batch_with_different_iteration_counts_and_replay(cuda):
    specs = cfg5_specs(n_grids=9, T=4, seed=12, side2=(50, 200), side3=(10, 30))
    Ts = [4, 2, 1, 6, 4, 2, 0, 4, 2]
    specs = [(st.with_(iterations=t), sd) for (st, sd), t in zip(specs, Ts)]
    a, b, host = _grids(specs)
    batch = uhs.Batch([s for s, _ in specs], a, b)
    assert batch.stats()["steps"] == 6
    batch.run()
    _check(specs, a, b, host)
    # a second replay continues from the first run's result
    batch.run()
    for (st, _), da, a0 in zip(specs, a, host):
        if st.iterations == 0 or st.dtype == uhs.UHS_F32 or st.iterations == 1:
            continue
        r1, r1b = run_oracle(st, a0)
        r2, _ = run_oracle(st, r1, r1b)
        assert_f64_close(st, r2, da.cpu().numpy().reshape(-1))
    batch.close()


def test_one_launch_per_timestep_for_a_mixed_precision_batch(cuda):
    specs = cfg5_specs(n_grids=12, T=6, seed=13, side2=(64, 128), side3=(16, 24))
    a, b, _ = _grids(specs)
    batch = uhs.Batch([s for s, _ in specs], a, b)
    n0 = uhs.launch_count()
    batch.run()
    assert batch.stats()["launches"] == 6
    assert uhs.launch_count() - n0 == 6


def test_batch_rejects_programs_outside_the_streaming_kernels(cuda):
    st, a0 = random_case(3, 1, "star", (8, 8, 8), 2, 1)
    odd = st.with_(terms=st.terms + [(1, 1, 0, 0.01)])  # not a star, not a full box
    a = to_dev(a0, st)
    with pytest.raises(uhs.UhsError):
        uhs.Batch([st, st.with_(terms=[(0, 0, 0, 1.0)])], [a, a.clone()], [a.clone(), a.clone()])
    del odd


def test_large_grids_run_as_their_own_launches_beside_the_persistent_kernel(cuda):
    """Grids of 2^21 points or more are swept by their standalone plan in
    parallel branches of the batch's graph: a float-pair 7-point star and an
    FP32 2D 49-point box above the threshold (T = 1 and T = 4), with small
    grids of several shapes in the persistent kernel; every grid matches its
    oracle run, and the launch count adds the large grids' sweeps."""
    small = cfg5_specs(n_grids=6, T=4, seed=17, side2=(40, 120), side3=(12, 30))
    big1, _ = random_case(3, 1, "star", (136, 128, 128), 1, 31)
    big2, _ = random_case(2, 3, "box", (1500, 1400), 4, 32, dtype=uhs.UHS_F32)
    assert big1.interior_points >= 1 << 21 and big2.interior_points >= 1 << 21
    specs = small + [(big1, 301), (big2, 302)]
    a, b, host = _grids(specs)
    batch = uhs.Batch([s for s, _ in specs], a, b)
    stats = batch.stats()
    assert stats["steps"] == 4
    assert stats["launches"] == 4 + 1 + 4  # persistent steps + the large grids' sweeps
    n0 = uhs.launch_count()
    batch.run()
    assert uhs.launch_count() - n0 == stats["launches"]
    _check(specs, a, b, host)
    batch.close()


def test_large_float_pair_grid_runs_pair_resident_in_the_batch(cuda):
    """A large FP64 7-point star with T = 8 runs pair-resident inside the
    batch (split, 8 sweeps on pairs, join: 12 launches), beside a large FP64
    19-point star of T = 6 that stays in place (below 8 sweeps the
    conversions would not pay); both match the oracle, halos bit-exact, and a
    second replay continues from the first."""
    small = cfg5_specs(n_grids=4, T=2, seed=19, side2=(40, 100), side3=(12, 24))
    big1, _ = random_case(3, 1, "star", (136, 128, 128), 8, 41)
    big2, _ = random_case(3, 3, "star", (130, 130, 130), 6, 42)
    specs = small + [(big1, 401), (big2, 402)]
    a, b, host = _grids(specs)
    batch = uhs.Batch([s for s, _ in specs], a, b)
    assert batch.stats()["launches"] == 2 + (8 + 4) + 6
    batch.run()
    _check(specs, a, b, host)
    for (st, _), da, db in zip(specs[-2:], a[-2:], b[-2:]):
        assert oracle.halo_diff(st, host[specs.index((st, _))], da.cpu().numpy().reshape(-1)) == 0
    batch.run()
    st, a0 = specs[-2][0], host[-2]
    r1, r1b = run_oracle(st, a0)
    r2, _ = run_oracle(st, r1, r1b)
    assert_f64_close(st, r2, a[-2].cpu().numpy().reshape(-1))
    batch.close()


@pytest.mark.parametrize("rank,r", [(3, 1), (3, 2), (3, 3), (2, 1), (2, 2), (2, 3)])
def test_batched_float_pair_sums_match_the_standalone_sweep_bitwise(cuda, rank, r):
    """The persistent batch kernel sums each point on its own; the standalone
    sweep sums two points per packed instruction (rows in 3D, columns in 2D).
    The float-pair bounded sums do the same operations per point in both, so
    a small FP64 star in a batch and the same grid swept alone (both in
    place, T = 4) end with the same bits.  (Boxes are not compared: the
    batch sweeps them term by term, the standalone plan as separable
    passes.)"""
    import torch
    st, a0 = random_case(rank, r, "star", (18, 22, 40) if rank == 3 else (60, 300), 4, 700 + 10 * rank + r)
    sa = to_dev(a0, st)
    sb = sa.clone()
    uhs.run(st, sa, sb)
    ba = to_dev(a0, st)
    bb = ba.clone()
    batch = uhs.Batch([st], [ba], [bb])
    assert batch.stats()["launches"] == 4  # one persistent launch per step, no solo sweeps
    batch.run()
    torch.cuda.synchronize()
    for x, y in ((sa, ba), (sb, bb)):
        assert np.array_equal(x.cpu().numpy().view(np.uint64), y.cpu().numpy().view(np.uint64))
    batch.close()
