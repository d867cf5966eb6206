"""What the trained cost model gains.  The shipped network
(uxxxxxxxxh_gb300/data/costmodel.json, trained by tuner_study on GB300
timings of programs drawn from seed 101) ranks the launch candidates of
programs drawn from another seed, which it never saw; each program is also
tuned exhaustively (the yardstick).  Compared with the methods without it:

* an uninformed pick (the median candidate): the network's pick is faster;
* exhaustive tuning: on each of the 12 shapes the learned tuner's pick --
  the network's three best-ranked candidates, timed (3 timings instead of
  dozens) -- reaches at least 95 % of the exhaustive best on every program;
  the network's pick alone (no timing) at least 97 % on average and 80 % on
  every program.

Set UHS_COSTMODEL_OUT to write the per-program table."""
import json
import os
import statistics

import pytest

from uxxxxxxxxh_gb300 import _lib
from uxxxxxxxxh_gb300.costmodel import CostModel
from uxxxxxxxxh_gb300.runtime import RunParams, memref_raw, plan
from uxxxxxxxxh_gb300.tuner import Tuner, device_grids, measure
from uxxxxxxxxh_gb300.tuner_study import draw_programs

pytestmark = pytest.mark.gpu


def test_trained_model_gain_on_unseen_programs(cuda):
    cm = CostModel.default()
    rows = []
    for st in draw_programs(24, seed=909, cover=True):
        a, b = device_grids(st)
        _, results = Tuner().tune(st, a, b, reps=3, push=False)
        ns = sorted(r[0] for r in results)
        best_p = min(results, key=lambda r: r[0])[1]
        pick = cm.pick(st)
        pick3 = cm.pick_verified(st, a, b, k=3)
        dflt = plan(st, memref_raw(1 << 20, st.sizes), params=RunParams(flags=_lib.UHS_FLAG_NO_TUNE_DB))
        dflt.flags = _lib.UHS_FLAG_NO_TUNE_DB
        # the exhaustive winner re-timed with the picks, interleaved, over
        # >= 4 ms each (the table's own minimum is biased low by its noise)
        named = (("exhaustive", best_p), ("mlp", pick), ("mlp_top3", pick3), ("default", dflt))
        acc = {k: [] for k, _ in named}
        for _ in range(3):
            for k, p in named:
                acc[k].append(measure(st, a, b, p, reps=3, min_ms=4.0))
        t = {k: min(v) for k, v in acc.items()}
        best = min(t.values())
        rows.append({"program": st.name, "shape": st.name.split("_", 1)[1], "dtype": st.dtype,
                     "candidates": len(ns),
                     "best_ns": best, "median_ns": ns[len(ns) // 2], **{k + "_ns": v for k, v in t.items()}})
        del a, b
    if os.environ.get("UHS_COSTMODEL_OUT"):
        with open(os.environ["UHS_COSTMODEL_OUT"], "w") as f:
            json.dump(rows, f, indent=1)
    # faster than an uninformed pick on (nearly) every program
    beats_median = sum(r["mlp_ns"] <= r["median_ns"] * 1.02 for r in rows)
    assert beats_median >= len(rows) - 1, rows
    gain_vs_median = statistics.mean(r["median_ns"] / r["mlp_ns"] for r in rows)
    assert gain_vs_median > 1.2
    # per shape (12 shapes, an FP64 and an FP32 program each): the learned
    # tuner's verified pick (the network's three best candidates, timed)
    # within 5 % of the exhaustive best on every program; the network's
    # untimed pick within 3 % on average and within 20 % on every program
    # (its misses are single small grids of a few microseconds a sweep,
    # e.g. a 1921 x 1516 2d3r FP32 star at 0.84, where the 128- and
    # 256-column strips of one or two points per thread differ by wave
    # quantisation the network does not resolve)
    worst, worst3 = {}, {}
    for r in rows:
        worst[r["shape"]] = min(worst.get(r["shape"], 1.0), r["best_ns"] / r["mlp_ns"])
        worst3[r["shape"]] = min(worst3.get(r["shape"], 1.0), r["best_ns"] / r["mlp_top3_ns"])
    assert len(worst3) == 12 and min(worst3.values()) >= 0.95, worst3
    assert min(worst.values()) >= 0.80, worst
    assert statistics.mean(r["best_ns"] / r["mlp_ns"] for r in rows) >= 0.97, rows
    # top-3 verified picks keep >= 95% of the exhaustive best on average
    assert statistics.mean(r["best_ns"] / r["mlp_top3_ns"] for r in rows) >= 0.95
    # and never fall far behind the planner's own default
    assert statistics.mean(r["default_ns"] / r["mlp_top3_ns"] for r in rows) >= 0.98
