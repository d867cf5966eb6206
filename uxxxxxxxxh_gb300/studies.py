"""Measurement studies beyond the headline bench line.

    python -m uxxxxxxxxh_gb300.studies shapes [--out f.json] [--programs f.json]

shapes: the 12 reference cases at the reference GPU harness's own sizes
(UH-GPU/*/*.dsl: 8192^2 interior for rank 2, 512^3 for rank 3, FP64, T = 4,
1-3 cell halos), each in FP64 float pairs, native FP64 and FP32, launched with
the exhaustive tuner's best configuration for that exact program; reported as
GStencil/s beside the reference's published A100 figure for the same case
(scripts/figure_scripts/data.xlsx, sheet GPU, as ns per sweep).  Each row also
times the planner's own choice (no tuner database) against that best.

Coefficients: by default seeded random ones (no two alike, so no box
factors into 1D passes -- the general case); with --programs, the programs
recorded from the reference's own UH-GPU/*.dsl files (their "gpu" entries:
terms, sizes, T), whose boxes are rank-1 and run as separable passes.

The precision study of configuration 4 compares against the FP64 oracle and
therefore lives with the tests (tests/test_precision_gpu.py).
"""
from __future__ import annotations

import argparse
from dataclasses import asdict
import json
import os
import sys

from . import _lib
from .runtime import RunParams, memref_raw, plan
from .stencil import Stencil, box_offsets, make_stencil, star_offsets
from .tuner import Tuner, device_grids, measure
from .workloads import normalised, splitmix_uniform

# Reference A100 ns per sweep (UHStencil, FP64, 8192^2 / 512^3), data.xlsx sheet GPU.
A100_NS = {"2d1r_star": 797988, "2d2r_star": 814611, "2d3r_star": 818823, "2d1r_box": 802797,
           "2d2r_box": 987816, "2d3r_box": 1586535, "3d1r_star": 1676043, "3d2r_star": 2447721,
           "3d3r_star": 2480094, "3d1r_box": 3503287, "3d2r_box": 8349494, "3d3r_box": 21153389}


def program_of(case: str, programs: dict | None) -> Stencil:
    """The case's stencil program: the recorded reference program when
    `programs` holds it, else the seeded random-coefficient one."""
    rank, r, kind = int(case[0]), int(case[2]), case.split("_")[1]
    if programs is not None:
        rec = programs[case]["gpu"]
        return Stencil(name=rec["name"], rank=rec["rank"], sizes=tuple(rec["sizes"]), lb=tuple(rec["lb"]),
                       ub=tuple(rec["ub"]), terms=[tuple(t) for t in rec["terms"]], iterations=rec["iterations"],
                       exact_order=rec["exact_order"])
    interior = (8192, 8192) if rank == 2 else (512, 512, 512)
    offs = star_offsets(rank, r) if kind == "star" else box_offsets(rank, r)
    coefs = normalised(splitmix_uniform(1234 + r, len(offs)) + 0.05)
    return make_stencil(case, rank, interior, r, offs, coefs, iterations=4)


def shapes_study(out: str | None = None, reps: int = 3, programs_path: str | None = None) -> dict:
    programs = None
    if programs_path:
        with open(programs_path) as f:
            programs = json.load(f)
    rows = []
    for case, ns in A100_NS.items():
        base = program_of(case, programs)
        rank = base.rank
        row = {"case": case, "points": len(base.terms), "a100_gst": base.interior_points / (ns * 1e-9) / 1e9,
               "coefficients": "reference" if programs is not None else "random"}
        for label, dtype in (("f64", _lib.UHS_F64), ("f32", _lib.UHS_F32)):
            st = base.with_(dtype=dtype)
            row[f"{label}_factored"] = plan(st, memref_raw(1 << 20, st.sizes),
                                            params=RunParams(flags=_lib.UHS_FLAG_NO_TUNE_DB)).factored
            a, b = device_grids(st)
            t = Tuner()
            best, results = t.tune(st, a, b, reps=reps, push=False)
            row[f"{label}_best"] = {k: v for k, v in asdict(best).items() if v and k != "flags"}
            # the planner's own choice (no tuner database), timed the same way
            dflt = plan(st, memref_raw(1 << 20, st.sizes), params=RunParams(flags=_lib.UHS_FLAG_NO_TUNE_DB))
            dflt.flags = _lib.UHS_FLAG_NO_TUNE_DB
            row[f"{label}_default_gst"] = 1.0 / min(measure(st, a, b, dflt, reps=reps) for _ in range(2))
            row[f"{label}_default"] = {k: v for k, v in asdict(dflt).items() if v and k != "flags"}
            if dtype == _lib.UHS_F64:
                df = [1.0 / ns_ for ns_, p in results if p.arith == _lib.UHS_ARITH_DF32]
                nat = [1.0 / ns_ for ns_, p in results if p.arith != _lib.UHS_ARITH_DF32]
                row["f64_df32_gst"] = max(df) if df else None
                row["f64_native_gst"] = max(nat) if nat else None
            else:
                row["f32_gst"] = max(1.0 / ns_ for ns_, _ in results)
            del a, b
        row["f64_best_vs_a100"] = max(row["f64_df32_gst"] or 0, row["f64_native_gst"] or 0) / row["a100_gst"]
        row["f32_vs_f64"] = row["f32_gst"] / max(row["f64_df32_gst"] or 0, row["f64_native_gst"] or 0)
        row["f64_default_vs_best"] = row["f64_default_gst"] / max(row["f64_df32_gst"] or 0, row["f64_native_gst"] or 0)
        row["f32_default_vs_best"] = row["f32_default_gst"] / row["f32_gst"]
        rows.append(row)
        print(json.dumps(row), flush=True)
    res = {"study": "shapes", "coefficients": "reference" if programs is not None else "random", "rows": rows}
    if out:
        with open(out, "w") as f:
            json.dump(res, f, indent=1)
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["shapes"])
    ap.add_argument("--out", default=None)
    ap.add_argument("--programs", default=None, help="JSON of recorded reference programs")
    a = ap.parse_args()
    shapes_study(a.out, programs_path=a.programs)


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    main()
