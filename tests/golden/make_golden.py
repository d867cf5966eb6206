"""Generate the golden fixtures under tests/golden/ from the reference checkout.

Run here, where the reference checkout and oracle/_ref (oracle/build_ref.py)
exist:   python tests/golden/make_golden.py [REFERENCE_ROOT]

Writes
  reference_stencils.json  every UH-SW and UH-GPU case's stencil program as
                           the library's DSL reader reads the case's .dsl file
                           (grid extents, domain, T, terms in expression order);
  reference_pins.json      per case, the SHA-256 of the grid the reference's
                           own CPU loop leaves after running on its own data
                           (rand() % 50, as the drivers' main() fills it), with
                           a few sample cells.  Each digest is written only
                           after the oracle's result was checked bit-for-bit
                           against the reference's result in this run.
  fusion_pins.json         the spatially fused program laplaceAddInput
                           (test/Examples/StencilDialect/laplaceAddInputIteration:
                           a producer kernel inlined into its consumer) as the
                           DSL reader reads it, and the SHA-256 of the grid its
                           driver's serial loop leaves (run as an executable,
                           grid read from the mpe_result file it writes),
                           written after the oracle reproduced it bit-for-bit.
UH-SW cases run mpe_verify (T = 20 on 4096^2 / 256^3).  UH-SW/3d3r_box's
mpe_verify jumps past its loops (stencil_3d343pt_driver.serial.c:43), so the
343-point box is pinned through UH-GPU/3d3r_box's cpu_verify (T = 4 on 512^3).

  python tests/golden/make_golden.py [REFERENCE_ROOT] [--fusion-only]
"""
from __future__ import annotations

import glob
import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import uxxxxxxxxh_gb300 as uhs  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["2d1r_star", "2d2r_star", "2d3r_star", "2d1r_box", "2d2r_box", "2d3r_box",
         "3d1r_star", "3d2r_star", "3d3r_star", "3d1r_box", "3d2r_box", "3d3r_box"]
# (case, driver kind) pairs whose reference loop is pinned
PINNED = [(c, "sw") for c in CASES if c != "3d3r_box"] + [("3d3r_box", "gpu")]


def stencil_record(st: uhs.Stencil, dsl_rel: str) -> dict:
    return {"dsl": dsl_rel, "name": st.name, "rank": st.rank, "sizes": list(st.sizes), "lb": list(st.lb),
            "ub": list(st.ub), "iterations": st.iterations, "exact_order": st.exact_order,
            "terms": [list(t) for t in st.terms]}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(a.tobytes()).hexdigest()


def samples(a: np.ndarray, st: uhs.Stencil) -> list:
    sz = st.sizes
    pts = [tuple(l for l in st.lb), tuple((l + u) // 2 for l, u in zip(st.lb, st.ub)),
           tuple(u - 1 for u in st.ub)]
    out = []
    for p in pts:
        i = (p[0] * sz[1] + p[1]) * sz[2] + p[2]
        out.append([list(p), float(a[i])])
    return out


def fusion(ref_root: str) -> None:
    import tempfile
    from oracle import build_ref
    st = uhs.parse_dsl_file(os.path.join(ref_root, build_ref.FUSION_DSL))
    n = int(np.prod(st.sizes))
    a, b = np.empty(n), np.empty(n)
    oracle.fill_rand50([a, b])  # the driver fills input and output alike
    oracle.iterate_f64(st, a, b)
    with tempfile.TemporaryDirectory() as d:
        ref = np.array(build_ref.run_fusion_driver(d))
    same = np.array_equal(ref.view(np.uint64), a.view(np.uint64))
    print(f"fusion laplaceAddInput: bit-exact={same}", flush=True)
    if not same:
        raise SystemExit("oracle differs from the reference on the fused program")
    rec = {"program": stencil_record(st, build_ref.FUSION_DSL), "driver": build_ref.FUSION[1], "cells": n,
           "iterations": st.iterations, "sha256": digest(a), "samples": samples(a, st)}
    with open(os.path.join(HERE, "fusion_pins.json"), "w") as f:
        json.dump(rec, f, indent=1)


def main(ref_root: str) -> None:
    stencils = {}
    for kind, sub in (("sw", "UH-SW"), ("gpu", "UH-GPU")):
        for case in CASES:
            f = glob.glob(os.path.join(ref_root, sub, case, "*.dsl"))[0]
            st = uhs.parse_dsl_file(f)
            stencils.setdefault(case, {})[kind] = stencil_record(st, os.path.relpath(f, ref_root))
    with open(os.path.join(HERE, "reference_stencils.json"), "w") as f:
        json.dump(stencils, f, indent=1)

    pins = {}
    for case, kind in PINNED:
        rec = stencils[case][kind]
        st = uhs.Stencil(name=rec["name"], rank=rec["rank"], sizes=tuple(rec["sizes"]), lb=tuple(rec["lb"]),
                         ub=tuple(rec["ub"]), terms=[tuple(t) for t in rec["terms"]], iterations=rec["iterations"])
        n = int(np.prod(st.sizes))
        t0 = time.time()
        ref = oracle.run_ref_sw(case, n) if kind == "sw" else oracle.run_ref_gpu_cpu_verify(case, n)
        t_ref = time.time() - t0
        a = np.empty(n)
        b = np.empty(n) if kind == "sw" else np.zeros(n)
        oracle.fill_rand50([a, b] if kind == "sw" else [a])
        t0 = time.time()
        oracle.iterate_f64(st, a, b)
        t_or = time.time() - t0
        same = np.array_equal(ref.view(np.uint64), a.view(np.uint64))
        print(f"{case:10s} {kind}: bit-exact={same}  reference {t_ref:.1f}s  oracle {t_or:.1f}s", flush=True)
        if not same:
            raise SystemExit(f"oracle differs from the reference on {case} ({kind})")
        pins[case] = {"driver": kind, "dsl": rec["dsl"], "cells": n, "iterations": st.iterations,
                      "sha256": digest(a), "samples": samples(a, st)}
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(pins, f, indent=1)
    fusion(ref_root)


if __name__ == "__main__":
    from oracle.build_ref import reference_root
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    root = args[0] if args else reference_root()
    if not root:
        raise SystemExit("reference checkout not found (pass its path or set UHS_REFERENCE_ROOT)")
    if "--fusion-only" in sys.argv:
        fusion(root)
    else:
        main(root)
