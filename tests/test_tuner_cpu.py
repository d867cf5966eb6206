"""Host-side tuner logic, no GPU needed: candidate lists (planned on the
host), the tuner database file (round trip, corrupted files rejected without
effect) and a candidate that fails to launch."""
import pytest

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


def _push_two():
    from uxxxxxxxxh_gb300.runtime import RunParams
    from uxxxxxxxxh_gb300.tuner import push_params
    a, _ = random_case(3, 1, "star", (64, 64, 64), 2, 8)
    b, _ = random_case(2, 3, "box", (500, 700), 2, 9, dtype=_lib.UHS_F32)
    push_params(a, RunParams(kernel=_lib.UHS_KERNEL_STREAM, arith=_lib.UHS_ARITH_DF32, tile_x=64, tile_y=8, vy=2,
                             tile_z=16, use_tma=1), 123.5)
    push_params(b, RunParams(kernel=_lib.UHS_KERNEL_STREAM, tile_x=256, use_tma=-1), 77.0)
    return a, b


def test_tuner_database_round_trip(tmp_path):
    from uxxxxxxxxh_gb300 import tuner
    tuner.db_clear()
    a, b = _push_two()
    before = {s.name: tuner.db_get(s) for s in (a, b)}
    path = str(tmp_path / "tune.db")
    tuner.db_save(path)
    tuner.db_clear()
    assert _lib.lib().uhs_tune_size() == 0
    tuner.db_load(path)
    assert _lib.lib().uhs_tune_size() == 2
    for s in (a, b):
        assert tuner.db_get(s) == before[s.name]
    tuner.db_clear()


@pytest.mark.parametrize("text", [
    "not a database\n",
    "uhs-tune 1\n3 0 1 0 64 64 64 2 3 64 8 16 1 1 0 2 0\n",             # a field short
    "uhs-tune 1\n3 0 9 0 64 64 64 2 3 64 8 16 1 1 0 2 0 12.5\n",        # radius 9
    "uhs-tune 1\n3 2 1 0 64 64 64 2 3 64 8 16 1 1 0 2 0 12.5\n",        # a 2D shape on a 3D key
    "uhs-tune 1\n3 0 1 0 64 64 64 2 3 64 8 16 1 1 0 2 0 12.5 junk\n",   # trailing field
    "",
])
def test_corrupted_tuner_database_is_rejected_and_changes_nothing(tmp_path, text):
    from uxxxxxxxxh_gb300 import tuner
    tuner.db_clear()
    a, b = _push_two()
    before = {s.name: tuner.db_get(s) for s in (a, b)}
    path = tmp_path / "bad.db"
    path.write_text(text)
    with pytest.raises(_lib.UhsError) as ei:
        tuner.db_load(str(path))
    assert ei.value.code == _lib.UHS_EPARSE
    assert _lib.lib().uhs_tune_size() == 2
    for s in (a, b):
        assert tuner.db_get(s) == before[s.name]
    with pytest.raises(_lib.UhsError) as ei:
        tuner.db_load(str(tmp_path / "missing.db"))
    assert ei.value.code == _lib.UHS_EINVAL
    tuner.db_clear()


def test_tuner_skips_a_candidate_that_fails_to_launch(monkeypatch):
    """A candidate whose launch fails (as a variant needing more shared memory
    than the part has would) is skipped; the tuner keeps the others."""
    from uxxxxxxxxh_gb300 import tuner
    st, _ = random_case(3, 2, "star", (40, 50, 60), 2, 10)
    cands = tuner.candidates(st)
    bad = cands[0]

    def fake_measure(st_, a, b, p, reps=3, stream=None, min_ms=2.0):
        if p == bad:
            raise _lib.UhsError(_lib.UHS_ECUDA, "launch failed: too much shared memory")
        return 1.0 + cands.index(p)

    monkeypatch.setattr(tuner, "measure", fake_measure)
    best, results = tuner.Tuner().tune(st, a=object(), b=object(), push=False)
    assert len(results) == len(cands) - 1
    assert best == cands[1]


def test_tuner_database_keeps_two_points_along_x_and_reads_version_1(tmp_path):
    """Files are written as version 2 with the vx column; an entry with two
    points per thread along x survives a round trip, and a version-1 file
    (no vx column) still loads, its entries with vx 0 (the planner's
    choice)."""
    from uxxxxxxxxh_gb300 import tuner
    from uxxxxxxxxh_gb300.runtime import RunParams
    tuner.db_clear()
    st, _ = random_case(2, 1, "star", (300, 700), 2, 5, dtype=_lib.UHS_F32)
    tuner.push_params(st, RunParams(kernel=_lib.UHS_KERNEL_STREAM, arith=_lib.UHS_ARITH_FMA, tile_x=128, vx=2), 500.0)
    path = tmp_path / "tune.db"
    tuner.db_save(str(path))
    assert path.read_text().startswith("uhs-tune 2\n")
    tuner.db_clear()
    tuner.db_load(str(path))
    got, exact = tuner.db_get(st)
    assert exact and (got.tile_x, got.vx) == (128, 2)
    tuner.db_clear()
    old = tmp_path / "old.db"
    old.write_text("uhs-tune 1\n3 0 1 0 64 64 64 2 3 64 8 16 1 1 0 2 0 12.5\n")
    tuner.db_load(str(old))
    assert _lib.lib().uhs_tune_size() == 1
    st3, _ = random_case(3, 1, "star", (64, 64, 64), 2, 5)
    got, _ = tuner.db_get(st3)
    assert got is not None and got.vx == 0 and got.tile_x == 64
    tuner.db_clear()
