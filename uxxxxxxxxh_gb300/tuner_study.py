"""Train the learned cost model on the tuner's own GB300 timings and measure its
picks against exhaustive tuning.

    python -m uxxxxxxxxh_gb300.tuner_study [--train N] [--small S] [--test M] [--out result.json]
                                           [--model costmodel.json]

1. N training programs drawn from a seed across the 12 shapes and FP32/FP64,
   extents log-uniform (3D sides 48-384, 2D sides 512-6144, each axis drawn
   separately), and S more on small, irregular grids (3D sides 24-128, 2D
   256-2048), each tuned exhaustively: every timing becomes a record.
2. The network (costmodel.CostModel, the library's MLP kernels) is trained
   on the GPU on those records.
3. M held-out programs from another seed, at least one per shape and element
   type, are tuned exhaustively (the yardstick).  For each: the exhaustive best,
   the model's pick and the planner's default (no tuner database) are
   compared by their measured throughput, and so is the model's top-3
   verified pick (the fastest of its three best-ranked candidates, timed).
The JSON written holds every held-out program's three throughputs, the
per-shape worst ratio of the model's pick to the exhaustive best, and the
mean gain of the model's pick over the default.
"""
from __future__ import annotations

import argparse
import json
import math
import time
from dataclasses import asdict

from . import _lib
from .costmodel import CostModel
from .runtime import RunParams, plan
from .stencil import box_offsets, make_stencil, star_offsets
from .runtime import memref_raw
from .tuner import Tuner, device_grids, measure
from .workloads import normalised, splitmix_uniform

SHAPES12 = [(rank, r, kind) for rank in (2, 3) for kind in ("star", "box") for r in (1, 2, 3)]


def draw_programs(n: int, seed: int, cover: bool = False, small: bool = False) -> list:
    """n programs from the seed: shape and element type drawn (or, with cover,
    cycling through the 12 shapes in FP64 and FP32), extents log-uniform per
    axis; `small` draws the small and irregular grids (3D sides 24-128, 2D
    256-2048) where the launch's wave quantisation decides."""
    u = splitmix_uniform(seed, n * 8)
    out = []
    for g in range(n):
        v = u[8 * g:8 * g + 8]
        if cover:
            rank, r, kind = SHAPES12[(g // 2) % 12]
            f64 = g % 2 == 0
        else:
            rank, r, kind = SHAPES12[min(11, int(v[0] * 12))]
            f64 = v[4] >= 0.5
        lo, hi = (512, 6144) if rank == 2 else (48, 384)
        if small:
            lo, hi = (256, 2048) if rank == 2 else (24, 128)
        if rank == 3 and kind == "box" and r >= 2:
            hi = min(hi, 192)  # keep the slow native-FP64 boxes within seconds of timing
        sides = [int(round(math.exp(math.log(lo) + x * (math.log(hi) - math.log(lo))))) for x in v[1:1 + rank]]
        offs = star_offsets(rank, r) if kind == "star" else box_offsets(rank, r)
        coefs = normalised(splitmix_uniform(seed * 977 + g, len(offs)) + 0.05)
        dtype = _lib.UHS_F64 if f64 else _lib.UHS_F32
        out.append(make_stencil(f"p{g}_{rank}d{r}r_{kind}", rank, sides, r, offs, coefs, iterations=2, dtype=dtype))
    return out


def run(n_train: int, n_test: int, reps: int, epochs: int, out: str | None, model_path: str | None,
        seed: int = 101, n_small: int = 0, net_seed: int | None = None) -> dict:
    t0 = time.time()
    tr = Tuner()
    for st in draw_programs(n_train, seed) + draw_programs(n_small, seed + 50, small=True):
        a, b = device_grids(st)
        tr.tune(st, a, b, reps=reps, push=False)
        del a, b
    t_collect = time.time() - t0
    cm = CostModel(seed=seed if net_seed is None else net_seed)
    t1 = time.time()
    loss = cm.fit(tr.records, epochs=epochs)
    t_train = time.time() - t1
    rows = []
    for st in draw_programs(n_test, seed + 1, cover=True):
        a, b = device_grids(st)
        exhaustive = Tuner()
        _, results = exhaustive.tune(st, a, b, reps=reps, push=False)
        best_p = min(results, key=lambda r: r[0])[1]
        pick = cm.pick(st)
        pick3 = cm.pick_verified(st, a, b, k=3, reps=reps)
        dflt = plan(st, memref_raw(1 << 20, st.sizes), params=RunParams(flags=_lib.UHS_FLAG_NO_TUNE_DB))
        dflt.flags = _lib.UHS_FLAG_NO_TUNE_DB
        # Re-time the three picks interleaved over >= 10 ms each: the
        # exhaustive table's minimum is biased low by its own noise.
        acc = {"best": [], "mlp": [], "mlp_top3": [], "default": []}
        for _ in range(3):
            for name, p in (("best", best_p), ("mlp", pick), ("mlp_top3", pick3), ("default", dflt)):
                acc[name].append(measure(st, a, b, p, reps=reps, min_ms=4.0))
        g = {k: 1.0 / min(v) for k, v in acc.items()}
        rows.append({"program": st.name, "rank": st.rank, "radius": max(st.radius), "dtype": st.dtype,
                     "extents": [u - l for l, u in zip(st.lb, st.ub)],
                     "best_gst": max(g["best"], g["mlp"], g["mlp_top3"]),
                     "mlp_gst": g["mlp"], "mlp_top3_gst": g["mlp_top3"], "default_gst": g["default"],
                     "mlp_pick": asdict(pick), "exhaustive_pick": asdict(best_p), "default": asdict(dflt)})
        del a, b
    by_shape, by_shape3 = {}, {}
    for r in rows:
        k = f"{r['rank']}d{r['radius']}r_{r['program'].rsplit('_', 1)[-1]}_{'f64' if r['dtype'] == 0 else 'f32'}"
        by_shape[k] = min(by_shape.get(k, 1e9), r["mlp_gst"] / r["best_gst"])
        by_shape3[k] = min(by_shape3.get(k, 1e9), r["mlp_top3_gst"] / r["best_gst"])
    gains = [(r["mlp_gst"] or 0.0) / r["default_gst"] for r in rows if r["default_gst"]]
    res = {"train_programs": n_train, "small_train_programs": n_small, "records": len(tr.records),
           "final_train_loss": loss,
           "collect_seconds": t_collect, "train_seconds": t_train, "test_programs": n_test,
           "worst_ratio_by_shape": by_shape, "worst_ratio": min(by_shape.values()),
           "worst_ratio_top3_by_shape": by_shape3, "worst_ratio_top3": min(by_shape3.values()),
           "mean_ratio_top3": sum(r["mlp_top3_gst"] / r["best_gst"] for r in rows) / len(rows),
           "mean_ratio": sum((r["mlp_gst"] or 0.0) / r["best_gst"] for r in rows) / len(rows),
           "mean_gain_over_default": sum(gains) / max(1, len(gains)),
           "mean_default_ratio": sum((r["default_gst"] or 0.0) / r["best_gst"] for r in rows) / len(rows),
           "rows": rows}
    if out:
        with open(out, "w") as f:
            json.dump(res, f, indent=1)
    if model_path:
        cm.save(model_path)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=120)
    ap.add_argument("--small", type=int, default=0, help="extra training programs on small, irregular grids")
    ap.add_argument("--test", type=int, default=24)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--epochs", type=int, default=300)
    ap.add_argument("--out", default=None)
    ap.add_argument("--model", default=None)
    ap.add_argument("--net-seed", type=int, default=None,
                    help="seed of the networks' initial weights and minibatch order (default: the program seed)")
    a = ap.parse_args()
    res = run(a.train, a.test, a.reps, a.epochs, a.out, a.model, n_small=a.small, net_seed=a.net_seed)
    print(json.dumps({k: v for k, v in res.items() if k != "rows"}))


if __name__ == "__main__":
    main()
