"""Benchmark of the stencil backend on one GB300 (or N independent replicas).

Workload (default): 3d1r_star (7-point) FP64 on a 512^3 interior with a
1-cell zero halo, U[-1,1) data, 7 normalised U[0,1) coefficients, T = 50
sweeps with double-buffer ping-pong -- the configuration the GStencil/s metric
is quoted on.  One "step" is one complete program run (T sweeps of the grid)
through uhs_run() on the workload's input: both grids are reset to it before
every step, outside the timed interval.

Reported (one JSON line, rank 0):
  value      GStencil/s = interior points * T / time, grids resident in HBM
  e2e        the same metric through the C ABI with host buffers: pinned host
             -> device copy of the input grid, the run, device -> host copy of
             the result, all inside the timed region, with two runs in flight
             on two streams (one run's copies overlap the other's sweeps);
             e2e_serial is the same with one run at a time
  roofline   the sweep kernel's algorithmic bytes (16 B per point-update for
             FP64: one read and one write) per launch over its average launch
             time, against the measured HBM copy bandwidth
  cpu_baseline  the oracle's restatement of the reference's serial loops on
             this host's cores, on a bounded sample of the same workload
  fp32       the same workload on FP32 grids, with its L2 error against the
             FP64 oracle and, at full size on the GPU, against this library's
             FP64 sweep of the same rounded input (uhs.error_norms)
  plain_f64  the same workload in native IEEE binary64 arithmetic (DFMA), its
             kernel against the HBM roofline and the FP64 pipe's measured
             DFMA rate; speedup_vs_plain_f64 sets the default FP64 path and
             FP32 beside it, each with its error against the FP64 oracle
Inputs (1.09 GB per grid) are larger than the 129 MB L2, so no flush is
needed between timed iterations.

--impl reference times the reference's CPU implementation of the path (the
oracle port of mpe_verify, all host threads) on the same workload instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", default="cfg2", choices=["cfg1", "cfg2", "cfg3", "cfg4", "cfg5"])
    p.add_argument("--side", type=int, default=0, help="interior side override (smaller case for profiling)")
    p.add_argument("--iters", type=int, default=0, help="T override")
    p.add_argument("--dtype", choices=["f64", "f32"], default="f64", help="grid element type of the main run")
    p.add_argument("--arith", type=int, default=0)
    p.add_argument("--kernel", type=int, default=0)
    p.add_argument("--ktemporal", type=int, default=0, help="temporal fusion depth of the main run (1, 2, 4)")
    p.add_argument("--flags", type=int, default=0, help="UHS_FLAG_* bits added to the main run's parameters")
    p.add_argument("--tile-x", type=int, default=0, help="CTA tile along x of the main run (0: planner)")
    p.add_argument("--vx", type=int, default=0, help="points per thread along x of the main run (rank-2 stars: 2)")
    p.add_argument("--no-cpu", action="store_true", help="skip the oracle (profiling runs)")
    p.add_argument("--no-fp32", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-plain", action="store_true", help="skip the plain (native) FP64 arm")
    p.add_argument("--no-tune", action="store_true", help="cfg5: skip the standalone cost-model / exhaustive comparison")
    return p.parse_args()


# DRAM bytes per point-update of the sweep kernels, from one ncu capture of
# each on GB300 (dram__bytes_read.sum + dram__bytes_write.sum of one launch
# over its interior points; 320^3 interiors for rank 3, 8192^2 for rank 2,
# profiles/ holds the summaries).  A launch's traffic grows with the points it
# sweeps, so the per-launch figure for another size is this times its
# interior points.  Keyed by (shape, grid element type the kernel sweeps,
# arithmetic).
NCU_BYTES_PER_POINT = {
    # FP64 grids swept in place (320^3)
    ("3d1r_star", "f64", "df32"): 15.10, ("3d1r_star", "f64", "fma"): 15.20,
    # the sweeps of pair-resident runs (float-pair grids) and FP32 grids:
    # profiles/traffic_sweeps_small_cases.md
    ("3d1r_star", "f32x2", "df32"): 15.34, ("3d1r_star", "f32", "fma"): 6.78,
    ("3d2r_star", "f32x2", "df32"): 15.97, ("3d2r_star", "f32", "fma"): 6.91,
    ("3d3r_box_sep", "f32x2", "df32"): 16.08, ("3d3r_box_sep", "f32", "fma"): 7.11,
    # rank-2 float-pair stars sweep two points per thread along x:
    # profiles/k_stream_2d5pt_two_points_8192sq.md
    ("2d1r_star", "f32x2", "df32"): 15.74, ("2d1r_star", "f32", "fma"): 7.35,
}


def traffic_key(st, kernel_elem: str, arith: str, factored: bool):
    star = all(sum(1 for v in t[:3] if v) <= 1 for t in st.terms)
    kind = "star" if star else ("box_sep" if factored else "box")
    return (f"{st.rank}d{max(st.radius)}r_{kind}", kernel_elem, arith)


def workload_label(st) -> str:
    """The workload's name as both arms print it in config.workload."""
    return (f"{st.name}: {'x'.join(str(u - l) for l, u in zip(st.lb, st.ub))} interior, "
            f"halo {st.lb[2]}, T={st.iterations}")


ARITH_LABELS = {1: "fma (IEEE binary64 DFMA for FP64 grids, FFMA for FP32)",
                2: "exact (separately rounded IEEE products and sums, expression order)",
                3: "df32 (float pairs on the FP32 pipes: 48-bit significand; under AUTO scaled by a power of two "
                   "chosen per run, so the exponent window is about 2^190 wide anywhere in FP64's range)"}


def arith_names_full(code: int) -> str:
    return ARITH_LABELS.get(code, str(code))


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_bf16_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"])
    return 1900.0


def make_workload(args):
    from uxxxxxxxxh_gb300 import workloads as W
    fn = getattr(W, args.config)
    kw = {}
    if args.side:
        kw["n"] = args.side
    if args.iters:
        kw["T"] = args.iters
    st, a0 = fn(**kw)
    if getattr(args, "dtype", "f64") == "f32":
        from uxxxxxxxxh_gb300._lib import UHS_F32
        st = st.with_(dtype=UHS_F32)
    return st, a0


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            if len(r) >= 9:
                for nm, v in zip(names, r[5:9]):
                    if v.strip() == "Active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_sample(st, a0, budget_s: float = 12.0):
    """Oracle (port of the reference's serial loops) on all host threads:
    whole-grid sweeps, as many as fit the time budget (at most T)."""
    import oracle
    a, b = a0.copy(), a0.copy()
    oracle.set_threads(os.cpu_count() or 1)
    t0 = time.perf_counter()
    oracle.sweep_f64(st, a, b)
    t1 = time.perf_counter() - t0
    sweeps = int(max(1, min(st.iterations, budget_s // max(t1, 1e-6))))
    if sweeps > 1:
        t0 = time.perf_counter()
        for i in range(sweeps):
            if i % 2 == 0:
                oracle.sweep_f64(st, a, b)
            else:
                oracle.sweep_f64(st, b, a)
        t1 = time.perf_counter() - t0
    gst = st.interior_points * sweeps / t1 / 1e9
    cores = oracle.max_threads()
    return {"value": gst, "unit": "GStencil/s", "cores": cores, "kind": "port",
            "how": f"oracle port of the reference's serial loops on {cores} host threads",
            "sample": f"{sweeps} whole-grid sweep(s) of the {st.name} grid {tuple(st.sizes)} "
                      f"({st.interior_points} interior points each)", "seconds": t1}


def cpu_sample_1thread(st, a0):
    """The same port on one thread -- the reference's own CPU path is serial
    (mpe_verify) -- for one whole-grid sweep."""
    import oracle
    a, b = a0.copy(), a0.copy()
    oracle.set_threads(1)
    try:
        t0 = time.perf_counter()
        oracle.sweep_f64(st, a, b)
        t1 = time.perf_counter() - t0
    finally:
        oracle.set_threads(os.cpu_count() or 1)
    return {"value": st.interior_points / t1 / 1e9, "unit": "GStencil/s", "cores": 1, "kind": "port",
            "how": "oracle port of the reference's serial loops on 1 thread, as the reference runs them",
            "sample": f"1 whole-grid sweep of the {st.name} grid {tuple(st.sizes)}", "seconds": t1}


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    import oracle
    st, a0 = make_workload(args)
    oracle.set_threads(os.cpu_count() or 1)
    for _ in range(args.warmup):
        cpu_sample(st, a0, budget_s=1.0)
    vals = []
    samp = None
    for _ in range(args.steps):
        samp = cpu_sample(st, a0, budget_s=8.0)
        vals.append(samp["value"])
    v = statistics.median(vals)
    samp["value"] = v
    line = {"metric": "GStencil/s", "value": v, "unit": "GStencil/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": samp["seconds"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded SplitMix64)",
            "impl": "reference",
            "config": {"workload": workload_label(st), "l2": "inputs larger than L2 (no flush)"},
            "cpu_baseline": samp,
            "e2e": {"value": v, "unit": "GStencil/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def reduce_max_ms(ms: float, dist, device) -> float:
    """Max over ranks of each replica's own timing (a no-op on one rank)."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_gst(points_per_step: int, steps: int, ms: float, world: int) -> float:
    """Whole-job GStencil/s: every rank sweeps its own replica of the
    workload, so the job processes world * points per step in the max time."""
    return world * points_per_step * steps / (ms * 1e-3) / 1e9


def sweep_launch_ms(uhs, st, a, b, plan, stream, n: int, flags: int = 0) -> float:
    """Average duration of the sweep kernel alone: n single-sweep calls with
    the planned launch (alternating direction), CUDA events on the stream the
    kernel is launched on."""
    import torch
    q = uhs.RunParams(**{**plan.__dict__, "flags": uhs._lib.UHS_FLAG_NO_SYNC | uhs._lib.UHS_FLAG_NO_TUNE_DB | flags})
    s1 = st.with_(iterations=1)
    uhs.sweep(s1, a, b, q, stream=stream)
    uhs.sweep(s1, b, a, q, stream=stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(n):
        src, dst = (a, b) if i % 2 == 0 else (b, a)
        uhs.sweep(s1, src, dst, q, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / n


def box_paths(uhs, args, stream):
    """The 343-point Gaussian box (cfg3) on every path the backend has for
    it: FP32 grids on the CUDA cores term by term, as separable 1D passes and
    on the tensor cores (split-tf32 tcgen05), FP64 grids term by term (float
    pairs and native FP64) and separable; GStencil/s of one whole run and the
    error against the FP64 oracle."""
    import torch
    import oracle
    st, a0 = make_workload(args)
    oracle.set_threads(os.cpu_count() or 1)
    ra, rb = a0.copy(), a0.copy()
    oracle.iterate_f64(st, ra, rb)
    F = uhs._lib
    paths = {
        "f32_cuda_cores": (F.UHS_F32, uhs.RunParams(kernel=F.UHS_KERNEL_STREAM, flags=F.UHS_FLAG_NO_FACTOR)),
        "f32_separable": (F.UHS_F32, uhs.RunParams(kernel=F.UHS_KERNEL_STREAM)),
        "f32_tensor_cores": (F.UHS_F32, uhs.RunParams(kernel=F.UHS_KERNEL_MMA)),
        "f64_df32_cuda_cores": (F.UHS_F64, uhs.RunParams(arith=F.UHS_ARITH_DF32, flags=F.UHS_FLAG_NO_FACTOR)),
        "f64_native_cuda_cores": (F.UHS_F64, uhs.RunParams(arith=F.UHS_ARITH_FMA, flags=F.UHS_FLAG_NO_FACTOR)),
        "f64_separable": (F.UHS_F64, uhs.RunParams(arith=F.UHS_ARITH_DF32)),
    }
    out = {}
    for name, (dt, p) in paths.items():
        s = st.with_(dtype=dt)
        tdt = torch.float32 if dt == F.UHS_F32 else torch.float64
        a = torch.from_numpy(a0.reshape(st.sizes)).to(tdt).cuda()
        b = a.clone()
        q = uhs.RunParams(**{**p.__dict__, "flags": p.flags | F.UHS_FLAG_NO_SYNC})
        with torch.cuda.stream(stream):
            ms, _ = timed_runs(uhs, s, a, b, q, max(1, args.steps), max(1, args.warmup), stream)
        a.copy_(torch.from_numpy(a0.reshape(st.sizes)).to(tdt))
        b.copy_(a)
        uhs.run(s, a, b, p)
        e = oracle.error(st, ra, a.double().cpu().numpy().reshape(-1))
        q = uhs.plan(s, a, p)
        gst = st.interior_points * st.iterations * max(1, args.steps) / (ms * 1e-3) / 1e9
        out[name] = {"gstencil_s": gst, "l2_rel": e["l2_rel"], "max_rel": e["max_rel"], "kernel": q.kernel}
        if q.kernel == F.UHS_KERNEL_MMA:
            # Tensor-core rate: each output column takes K = tile_x + 8 window
            # columns per (dz, dy) row shift and three split-tf32 MMAs (hi.hi,
            # lo.hi, hi.lo); useful work is 2P flops per point.  Dense tf32
            # runs at half the bf16 rate, so the peak is half the measured bf16.
            d = 2 * max(st.radius) + 1
            issued = gst * 2 * (q.tile_x + 8) * d * d * 3 / 1e3
            peak = load_bf16_peak() / 2
            out[name]["tensor"] = {"useful_tflops": gst * 2 * len(st.terms) / 1e3, "issued_tflops": issued,
                                   "tf32_peak_tflops": peak, "frac": issued / peak,
                                   "peak_source": "half the measured bf16 dense rate (MEASURED_PEAKS.json)"}
        del a, b
    return out


def timed_runs(uhs, st, a, b, params, steps, warmup, stream, dist=None):
    """Time `steps` runs of the program, each on the workload's own input:
    before every run (outside the timed interval) both grids are reset to the
    input that a held at entry, so every step sweeps the same data rather than
    the previous step's result.  Each run is bracketed by CUDA events on the
    launching stream; returns the summed milliseconds and the kernels launched
    inside the timed intervals."""
    import torch
    a0 = a.clone()

    def reset():
        a.copy_(a0)
        b.copy_(a0)

    for _ in range(warmup):
        reset()
        uhs.run(st, a, b, params, stream=stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    launches = 0
    for e0, e1 in ev:
        reset()
        n0 = uhs.launch_count()
        e0.record(stream)
        uhs.run(st, a, b, params, stream=stream)
        e1.record(stream)
        launches += uhs.launch_count() - n0
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    a.copy_(a0)
    b.copy_(a0)
    torch.cuda.synchronize()
    del a0
    return ms, launches


def bench_batch(args, rank: int, world: int, local: int):
    """cfg5: 64 programs across all 12 shapes, FP32 and FP64, 20 timesteps,
    one persistent launch per timestep replayed from a CUDA graph.  Grid data
    is drawn on the device (seeded) -- the batch timing does not depend on it;
    the parity of batches is covered by tests/test_batch_gpu.py.  Beside it
    (unless --no-tune): the same programs launched one by one with launch
    parameters from the cost model and from exhaustive tuning."""
    import torch
    import uxxxxxxxxh_gb300 as uhs
    from uxxxxxxxxh_gb300.workloads import cfg5_specs
    # --side N: the same suite drawn on smaller grids (3D sides up to N, 2D up
    # to 8N), for profiling runs
    specs = cfg5_specs(n_grids=64, T=args.iters or 20) if not args.side else \
        cfg5_specs(n_grids=64, T=args.iters or 20, side2=(64, 8 * args.side), side3=(16, args.side))
    gen = torch.Generator(device="cuda")
    A, B = [], []
    for st, seed in specs:
        gen.manual_seed(seed)
        dt = torch.float32 if st.dtype == uhs.UHS_F32 else torch.float64
        shape = st.sizes if st.rank == 3 else st.sizes[1:]
        a = torch.rand(shape, generator=gen, device="cuda", dtype=torch.float64).mul_(2).sub_(1).to(dt)
        A.append(a)
        B.append(a.clone())
    host0 = None if args.no_cpu else [a.cpu() for a in A]  # initial grids, for the oracle check
    batch = uhs.Batch([s for s, _ in specs], A, B, uhs.RunParams())
    stream = torch.cuda.Stream()
    for _ in range(args.warmup):
        batch.run(stream)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    n0 = uhs.launch_count()
    e0.record(stream)
    for _ in range(args.steps):
        batch.run(stream, sync=False)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = uhs.launch_count() - n0
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    pts = sum(st.interior_points * st.iterations for st, _ in specs)
    byts = sum(st.interior_points * st.iterations * 2 * st.elem_bytes for st, _ in specs)
    peak, peak_kind = load_peaks()
    value = pts * args.steps / (ms * 1e-3) / 1e9
    achieved = byts * args.steps / (ms * 1e-3) / 1e9
    st_ = batch.stats()
    errors = None if args.no_cpu else batch_errors(uhs, batch, specs, A, B, host0, stream)
    tuning = None if args.no_tune else standalone_tuning(uhs, specs, A, B, stream, pts)
    line = {"metric": "GStencil/s", "value": value, "unit": "GStencil/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded)",
            "config": {"workload": "cfg5 batched mixed suite: 64 grids, 12 shapes, FP32+FP64, "
                                   f"T={specs[0][0].iterations}" + (f", 3D sides <= {args.side}" if args.side else ""),
                       "launches_per_step": st_["launches"], "timesteps": st_["steps"],
                       "work_items_per_timestep": st_["items"], "l2": f"{sum(2 * st.elem_bytes * st.sizes[0] * st.sizes[1] * st.sizes[2] for st, _ in specs) / 1e9:.1f} GB of grids"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None, "peak_source": peak_kind},
            "gpu_launches": launches, "clocks": clk}
    if errors:
        line["error_vs_oracle"] = errors
    if tuning:
        line["standalone"] = tuning
    if rank == 0:
        print(json.dumps(line), flush=True)


def batch_errors(uhs, batch, specs, A, B, host0, stream):
    """One replay of the batch from the initial grids, every grid scored
    against the FP64 oracle (FP32 grids: the oracle on their float values).
    Returns the worst relative L2 and max error per element type."""
    import torch
    import oracle
    oracle.set_threads(os.cpu_count() or 1)
    for a, b, h in zip(A, B, host0):
        a.copy_(h)
        b.copy_(h)
    batch.run(stream)
    torch.cuda.synchronize()
    worst = {}
    t0 = time.perf_counter()
    for (st, _), a, h in zip(specs, A, host0):
        x0 = h.double().numpy().reshape(-1).copy()
        ra, rb = x0.copy(), x0.copy()
        oracle.iterate_f64(st, ra, rb)
        e = oracle.error(st, ra, a.double().cpu().numpy().reshape(-1))
        k = "f32" if st.dtype == uhs.UHS_F32 else "f64"
        w = worst.setdefault(k, {"grids": 0, "l2_rel": 0.0, "max_rel": 0.0})
        w["grids"] += 1
        w["l2_rel"] = max(w["l2_rel"], e["l2_rel"])
        w["max_rel"] = max(w["max_rel"], e["max_rel"])
    worst["oracle_seconds"] = time.perf_counter() - t0
    return worst


def standalone_tuning(uhs, specs, A, B, stream, pts):
    """The same 64 programs launched one by one (T sweeps each), with launch
    parameters from the shipped cost model (no timing), from its three
    best-ranked candidates timed, and from exhaustive tuning of each program
    (the yardstick).  GStencil/s of one pass over all programs."""
    import torch
    from uxxxxxxxxh_gb300.costmodel import CostModel
    from uxxxxxxxxh_gb300.tuner import Tuner
    cm = CostModel.default()
    F = uhs._lib
    picks = {"mlp": [], "mlp_top3": [], "exhaustive": []}
    t0 = time.perf_counter()
    for i, (st, _) in enumerate(specs):
        picks["mlp"].append(cm.pick(st))
        picks["mlp_top3"].append(cm.pick_verified(st, A[i], B[i], k=3))
        picks["exhaustive"].append(Tuner().tune(st, A[i], B[i], push=False)[0])
    tune_s = time.perf_counter() - t0
    out = {"tuning_seconds": tune_s}
    for name, ps in picks.items():
        qs = [uhs.RunParams(**{**p.__dict__, "flags": F.UHS_FLAG_NO_SYNC | F.UHS_FLAG_NO_TUNE_DB}) for p in ps]

        def one_pass():
            for i, (st, _) in enumerate(specs):
                uhs.run(st, A[i], B[i], qs[i], stream=stream)
        one_pass()
        torch.cuda.synchronize()
        best = None
        for _ in range(2):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            one_pass()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = {"gstencil_s": pts / (best * 1e-3) / 1e9, "ms": best}
    out["mlp_vs_exhaustive"] = out["mlp"]["gstencil_s"] / out["exhaustive"]["gstencil_s"]
    out["mlp_top3_vs_exhaustive"] = out["mlp_top3"]["gstencil_s"] / out["exhaustive"]["gstencil_s"]
    # The batch again, with each pick set in the tuner database: the batch's
    # large grids run their database entry (the persistent kernel's small
    # grids keep its fixed tiles).
    from uxxxxxxxxh_gb300.tuner import db_clear, push_params
    out["batch_with_picks"] = {}
    for name, ps in picks.items():
        db_clear()
        for (st, _), p in zip(specs, ps):
            push_params(st, p, 1.0)
        batch = uhs.Batch([s for s, _ in specs], A, B, uhs.RunParams())
        batch.run(stream)
        torch.cuda.synchronize()
        best = None
        for _ in range(2):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            batch.run(stream, sync=False)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        batch.close()
        out["batch_with_picks"][name] = {"gstencil_s": pts / (best * 1e-3) / 1e9, "ms": best}
    db_clear()
    return out


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank, world)

    import torch
    import uxxxxxxxxh_gb300 as uhs
    torch.cuda.set_device(local)
    if args.config == "cfg5":
        return bench_batch(args, rank, world, local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod
        dist_mod.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist = dist_mod

    st, a0 = make_workload(args)
    params = uhs.RunParams(kernel=args.kernel, arith=args.arith, k_temporal=args.ktemporal,
                           flags=uhs._lib.UHS_FLAG_NO_SYNC | args.flags, tile_x=args.tile_x, vx=args.vx)
    stream = torch.cuda.Stream()
    tdt = torch.float32 if st.dtype == uhs.UHS_F32 else torch.float64
    dev_a = torch.from_numpy(a0.reshape(st.sizes)).to(tdt).cuda()
    dev_b = dev_a.clone()
    torch.cuda.synchronize()

    clocks = Clocks(local)
    clocks.start()
    with torch.cuda.stream(stream):
        ms, launches = timed_runs(uhs, st, dev_a, dev_b, params, args.steps, args.warmup, stream, dist)
    clk = clocks.stop()
    ms = reduce_max_ms(ms, dist, "cuda")
    pts = st.interior_points * st.iterations
    value = aggregate_gst(pts, args.steps, ms, world)
    ms_step = ms / args.steps
    plan = uhs.plan(st, dev_a, params)

    # Roofline of the dominant kernel (the sweep): algorithmic bytes per
    # launch (one read and one write of every interior element) over the
    # kernel's own average duration, timed here on its stream.
    eb = st.elem_bytes
    launches_per_step = max(1, launches // max(1, args.steps))
    sweeps = st.iterations * args.steps
    alg_bytes = 2 * eb * st.interior_points
    peak, peak_kind = load_peaks()
    # FP64 programs of T >= 8 float-pair sweeps run pair-resident (uhs_run):
    # their sweeps are the float-pair kernel on float-pair copies of the
    # grids, so that is the kernel timed here (8-byte pairs: the same 16 B
    # per point-update).
    pair_resident = (st.dtype == uhs.UHS_F64 and plan.kernel == uhs.UHS_KERNEL_STREAM and
                     plan.arith == uhs._lib.UHS_ARITH_DF32 and st.iterations >= 8 and plan.k_temporal <= 1)
    with torch.cuda.stream(stream):
        if pair_resident:
            hi = dev_a.float()
            lo = (dev_a - hi.double()).float()
            pa = torch.stack([hi, lo], -1).view(torch.float64).reshape(dev_a.shape).contiguous()
            pb = pa.clone()
            del hi, lo
            st_k = st.with_(dtype=uhs.UHS_F32X2)
            plan_k = uhs.plan(st_k, pa, uhs.RunParams(kernel=args.kernel, arith=uhs._lib.UHS_ARITH_DF32,
                                                      flags=args.flags, tile_x=args.tile_x, vx=args.vx))
            kernel_ms = sweep_launch_ms(uhs, st_k, pa, pb, plan_k, stream, n=max(10, min(2 * st.iterations, 40)),
                                        flags=args.flags)
            del pa, pb
        else:
            kernel_ms = sweep_launch_ms(uhs, st, dev_a, dev_b, plan, stream, n=max(10, min(2 * st.iterations, 40)),
                                        flags=args.flags)
    avg_launch_s = kernel_ms * 1e-3
    achieved = alg_bytes / avg_launch_s / 1e9
    step_sweep_ms = ms / max(1, sweeps)

    # Correctness of this exact run against the oracle (fresh input).
    errs = None
    cpu = None
    if rank == 0 and not args.no_cpu:
        import oracle
        oracle.set_threads(os.cpu_count() or 1)
        cpu = cpu_sample(st, a0)
        # FP32 runs are scored against the oracle on the same (rounded) input
        src = a0 if st.dtype != uhs.UHS_F32 else a0.astype(np.float32).astype(np.float64)
        ra, rb = src.copy(), src.copy()
        oracle.iterate_f64(st, ra, rb)
        dev_a.copy_(torch.from_numpy(a0.reshape(st.sizes)))
        dev_b.copy_(dev_a)
        uhs.run(st, dev_a, dev_b, uhs.RunParams(kernel=args.kernel, arith=args.arith, k_temporal=args.ktemporal,
                                                flags=args.flags, tile_x=args.tile_x, vx=args.vx))
        got = dev_a.double().cpu().numpy().reshape(-1)
        errs = oracle.error(st, ra, got)
        errs["halo_bit_exact"] = oracle.halo_diff(st, ra, got) == 0

    # FP32 grids on the same workload.
    fp32 = None
    if not args.no_fp32 and st.dtype == uhs.UHS_F64:
        st32 = st.with_(dtype=uhs.UHS_F32)
        a32 = torch.from_numpy(a0.astype(np.float32).reshape(st.sizes)).cuda()
        b32 = a32.clone()
        with torch.cuda.stream(stream):
            ms32, _ = timed_runs(uhs, st32, a32, b32, uhs.RunParams(flags=uhs._lib.UHS_FLAG_NO_SYNC),
                                 args.steps, args.warmup, stream, dist)
        fp32 = {"value": pts * args.steps / (ms32 * 1e-3) / 1e9, "unit": "GStencil/s",
                "speedup_vs_f64_auto": ms / ms32}
        if errs is not None:
            a32.copy_(torch.from_numpy(a0.astype(np.float32).reshape(st.sizes)))
            b32.copy_(a32)
            uhs.run(st32, a32, b32)
            e = oracle.error(st, ra, a32.cpu().numpy().reshape(-1))
            fp32["l2_rel_vs_f64_oracle"] = e["l2_rel"]
            fp32["max_rel_vs_f64_oracle"] = e["max_rel"]
        # The same comparison at full size on the GPU (uhs.error_norms): the
        # FP32 result against this library's FP64 sweep of the same rounded
        # input, which itself is within 1e-12 of the oracle.
        rounded = torch.from_numpy(a0.astype(np.float32).reshape(st.sizes))
        dev_a.copy_(rounded)
        dev_b.copy_(dev_a)
        uhs.run(st, dev_a, dev_b, uhs.RunParams(kernel=args.kernel, arith=args.arith, k_temporal=args.ktemporal))
        a32.copy_(rounded)
        b32.copy_(a32)
        uhs.run(st32, a32, b32)
        e = uhs.error_norms(st32, a32, dev_a)
        fp32["l2_rel_vs_f64_gpu"] = e["l2_rel"]
        fp32["max_rel_vs_f64_gpu"] = e["max_rel"]
        del a32, b32

    # Plain FP64: the same program in native IEEE binary64 arithmetic (one
    # DFMA per term and point, the arithmetic of the reference's GPU kernel),
    # timed the same way; its sweep kernel's rate against the HBM roofline and
    # against the FP64 pipe's DFMA rate measured here.
    plain = None
    if st.dtype == uhs.UHS_F64 and args.arith == 0 and not args.no_plain:
        pparams = uhs.RunParams(kernel=args.kernel, arith=uhs._lib.UHS_ARITH_FMA, flags=uhs._lib.UHS_FLAG_NO_SYNC)
        dev_a.copy_(torch.from_numpy(a0.reshape(st.sizes)))
        dev_b.copy_(dev_a)
        with torch.cuda.stream(stream):
            msp, _ = timed_runs(uhs, st, dev_a, dev_b, pparams, max(2, args.steps // 2), args.warmup, stream, dist)
        msp = reduce_max_ms(msp, dist, "cuda") / max(2, args.steps // 2)
        pplan = uhs.plan(st, dev_a, pparams)
        with torch.cuda.stream(stream):
            pk_ms = sweep_launch_ms(uhs, st, dev_a, dev_b, pplan, stream, n=10)
            dfma = uhs.probe_dfma_rate(stream)
        gst_p = pts / (msp * 1e-3) / 1e9
        # DFMA per point of the planned sweep: one per term, or per term of
        # the 1D passes when a separable box is swept as such
        dfma_pt = st.rank * (2 * max(st.radius) + 1) if pplan.factored == 1 else len(st.terms)
        plain = {"value": gst_p, "unit": "GStencil/s", "arith": ARITH_LABELS[1], "ms_per_step": msp,
                 "kernel_ms": pk_ms, "hbm_frac": alg_bytes / (pk_ms * 1e-3) / 1e9 / peak,
                 "dfma_per_s_measured": dfma, "dfma_per_point": dfma_pt,
                 "dfma_frac": st.interior_points * dfma_pt / (pk_ms * 1e-3) / dfma,
                 "bound": "fp64 pipe (one DFMA per term and point)"}
        if errs is not None:
            dev_a.copy_(torch.from_numpy(a0.reshape(st.sizes)))
            dev_b.copy_(dev_a)
            uhs.run(st, dev_a, dev_b, uhs.RunParams(kernel=args.kernel, arith=uhs._lib.UHS_ARITH_FMA))
            ep = oracle.error(st, ra, dev_a.cpu().numpy().reshape(-1))
            plain["l2_rel_vs_oracle"] = ep["l2_rel"]
            plain["max_rel_vs_oracle"] = ep["max_rel"]

    # End to end through the C ABI with host buffers: each step copies its
    # input grid from pinned host memory, runs the program (uhs_run) and reads
    # the result back.  Measured twice: with one run at a time on one stream,
    # and with two runs in flight on two streams (each its own device grids
    # and host result buffer), so that one run's copies overlap the other's
    # sweeps -- how a service streaming independent grids would drive it.
    e2e = e2e_serial = None
    if not args.no_e2e:
        host_in = torch.from_numpy(a0.reshape(st.sizes)).to(tdt).pin_memory()
        nbytes = host_in.numel() * host_in.element_size()

        def e2e_run(nstreams: int) -> float:
            streams = [stream] + [torch.cuda.Stream() for _ in range(nstreams - 1)]
            grids = [(dev_a, dev_b)] + [(torch.empty_like(dev_a), torch.empty_like(dev_a))
                                        for _ in range(nstreams - 1)]
            outs = [torch.empty_like(host_in).pin_memory() for _ in range(nstreams)]
            for it in range(args.warmup + args.steps):
                if it == args.warmup:
                    torch.cuda.synchronize()
                    if dist:
                        dist.barrier()
                    f0 = torch.cuda.Event(enable_timing=True)
                    f1 = torch.cuda.Event(enable_timing=True)
                    f0.record(streams[0])
                    for s in streams[1:]:
                        s.wait_event(f0)
                k = it % nstreams
                s, (ga, gb) = streams[k], grids[k]
                with torch.cuda.stream(s):
                    ga.copy_(host_in, non_blocking=True)
                    gb.copy_(ga, non_blocking=True)
                    uhs.run(st, ga, gb, params, stream=s)
                    outs[k].copy_(ga, non_blocking=True)
            for s in streams[1:]:
                ev = torch.cuda.Event()
                ev.record(s)
                streams[0].wait_event(ev)
            f1.record(streams[0])
            torch.cuda.synchronize()
            return reduce_max_ms(f0.elapsed_time(f1), dist, "cuda")

        for label, nstreams in (("serial", 1), ("overlapped", 2)):
            ems = e2e_run(nstreams)
            rec = {"value": aggregate_gst(pts, args.steps, ems, world), "unit": "GStencil/s",
                   "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes, "ms_per_step": ems / args.steps,
                   "runs_in_flight": nstreams}
            if label == "serial":
                e2e_serial = rec
            else:
                e2e = rec

    if rank != 0:
        return
    if cpu is not None:
        cpu["single_thread"] = cpu_sample_1thread(st, a0)
    # The metric's comparison: FP32 grids and the default FP64 path against
    # plain FP64, each with its error against the FP64 oracle.
    vs_plain = None
    if plain is not None:
        vs_plain = {"plain_f64_gstencil_s": plain["value"],
                    "f64_auto": plain["ms_per_step"] / ms_step,
                    "f64_auto_arith": arith_names_full(plan.arith),
                    "f64_auto_l2_rel": errs["l2_rel"] if errs else None,
                    "f64_auto_max_rel": errs["max_rel"] if errs else None}
        if fp32 is not None:
            fp32["speedup_vs_plain_f64"] = plain["ms_per_step"] / (ms32 / args.steps)
            vs_plain["fp32"] = fp32["speedup_vs_plain_f64"]
            vs_plain["fp32_l2_rel"] = fp32.get("l2_rel_vs_f64_oracle")
    arith_names = {1: "fma", 2: "exact", 3: "df32"}
    name = {0: "f64", 1: "f32"}.get(st.dtype, "f32x2")
    kname = "f32x2" if pair_resident else name
    tkey = traffic_key(st, kname, arith_names.get(plan.arith, ""), plan.factored == 1)
    bpp = NCU_BYTES_PER_POINT.get(tkey)
    traffic = bpp * st.interior_points if bpp else None
    if plan.kernel == uhs.UHS_KERNEL_MMA:
        name = "f32 (split-tf32 tensor cores)"
    line = {
        "metric": "GStencil/s", "value": value, "unit": "GStencil/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": name, "arith": ARITH_LABELS.get(plan.arith, str(plan.arith)),
        "data": "synthetic (seeded SplitMix64)",
        "config": {"workload": workload_label(st),
                   "parallelism": "replicas" if world > 1 else "1 GPU", "l2": "inputs larger than L2 (no flush)",
                   "kernel": plan.kernel, "arith": arith_names.get(plan.arith, plan.arith),
                   "tile": ([plan_k.tile_x, plan_k.tile_y, plan_k.tile_z, plan_k.vy] if pair_resident else
                            [plan.tile_x, plan.tile_y, plan.tile_z, plan.vy]),
                   "vx": plan_k.vx if pair_resident else plan.vx, "k_temporal": plan.k_temporal,
                   "pair_resident": pair_resident},
        "pct_hbm_roofline": achieved / peak,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic,
                     "traffic_source": (f"ncu DRAM bytes per point of one launch of this kernel {tkey} on a "
                                        "smaller grid, times the points" if traffic else
                                        f"no ncu capture recorded for {tkey}"),
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel": ("float-pair sweep on pair-resident copies of the FP64 grids" if pair_resident
                                else "sweep on the grids in place"),
                     "alg_bytes_per_launch": alg_bytes, "avg_launch_ms": avg_launch_s * 1e3,
                     "step_time_per_sweep_ms": step_sweep_ms},
        "gpu_launches": launches,
        "launches_per_step": launches_per_step,
        "sweep_launches": sweeps,
        "clocks": clk,
        "e2e": e2e,
        "e2e_serial": e2e_serial,
        "cpu_baseline": cpu,
        "error_vs_oracle": errs,
        "fp32": fp32,
        "plain_f64": plain,
        "speedup_vs_plain_f64": vs_plain,
    }
    if args.config == "cfg3" and not args.no_cpu:
        line["box_paths"] = box_paths(uhs, args, stream)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
