"""The exhaustive tuner and the planner's tuner database on the GPU."""
import pytest

import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import tuner
from gpu_util import assert_f64_close, run_gpu, run_oracle
from uxxxxxxxxh_gb300.workloads import random_case

pytestmark = pytest.mark.gpu


def test_tune_pushes_the_winner_into_the_planner(cuda):
    tuner.db_clear()
    st, a0 = random_case(3, 1, "star", (64, 64, 96), 2, 1)
    t = tuner.Tuner()
    best, results = t.tune(st, reps=2)
    assert len(results) >= 20
    assert min(r[0] for r in results) == pytest.approx(1.0 / t.best[t.key(st)]["gst"])
    got, exact = tuner.db_get(st)
    assert exact and (got.tile_x, got.tile_y, got.vy, got.use_tma) == (best.tile_x, best.tile_y, best.vy,
                                                                         best.use_tma)
    planned = uhs.plan(st)
    assert (planned.tile_x, planned.tile_y) == (best.tile_x, best.tile_y)
    # a near extent uses the same class entry; the run is still correct
    st2, b0 = random_case(3, 1, "star", (60, 70, 90), 2, 2)
    assert tuner.db_get(st2)[1] is False
    ra, _ = run_oracle(st2, b0)
    ga, _ = run_gpu(st2, b0)
    assert_f64_close(st2, ra, ga)
    # opting out of the database
    p = uhs.plan(st, params=uhs.RunParams(flags=uhs._lib.UHS_FLAG_NO_TUNE_DB))
    assert p.kernel == uhs.UHS_KERNEL_STREAM
    tuner.db_clear()
    assert uhs._lib.lib().uhs_tune_size() == 0


def test_every_candidate_runs_and_is_timed(cuda):
    for args in [(2, 2, "box", (300, 257)), (3, 3, "star", (40, 30, 64))]:
        st, _ = random_case(*args, 2, 3)
        a, b = tuner.device_grids(st)
        for p in tuner.candidates(st):
            assert tuner.measure(st, a, b, p, reps=1) > 0.0
