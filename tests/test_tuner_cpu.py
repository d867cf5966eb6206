"""Tuner candidate lists are planned on the host (no GPU needed)."""
from uxxxxxxxxh_gb300 import _lib
from uxxxxxxxxh_gb300.tuner import N_FEATURES, candidates, features
from uxxxxxxxxh_gb300.workloads import random_case


def test_tensor_core_kernel_is_only_tuned_on_request():
    st, _ = random_case(3, 3, "box", (64, 64, 64), 2, 5, dtype=_lib.UHS_F32)
    plain = candidates(st)
    assert all(p.kernel != _lib.UHS_KERNEL_MMA for p in plain)
    with_mma = candidates(st, include_mma=True)
    assert any(p.kernel == _lib.UHS_KERNEL_MMA for p in with_mma)
    assert len(with_mma) > len(plain)


def test_candidates_are_distinct_and_featurised():
    for rank, r, kind, dt in ((3, 1, "star", _lib.UHS_F32), (3, 2, "box", _lib.UHS_F64), (2, 3, "star", _lib.UHS_F64)):
        st, _ = random_case(rank, r, kind, (40, 50, 60) if rank == 3 else (300, 400), 2, 6, dtype=dt)
        cs = candidates(st)
        keys = {tuple(vars(p).values()) for p in cs}
        assert len(keys) == len(cs) > 1
        for p in cs:
            assert len(features(st, p)) == N_FEATURES


def test_vy8_tile_is_a_candidate_for_fp32_stars_only():
    st, _ = random_case(3, 2, "star", (40, 300, 64), 2, 7, dtype=_lib.UHS_F32)
    assert any(p.vy == 8 for p in candidates(st))
    st64 = st.with_(dtype=_lib.UHS_F64)
    assert not any(p.vy == 8 for p in candidates(st64))
