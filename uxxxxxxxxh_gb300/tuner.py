"""Exhaustive autotuner for the streaming sweep.

UHStencil searches its compile-time tiling space at random
(scripts/evaluation_scripts_GPU/test_driver.py:169-285: grid/block tile
sizes, inner tile, shared-memory flag; 1000 random configurations, each
compiled and timed with nsys) and keeps the fastest per case
(collect.py:384-419).  Here the same knobs are run-time parameters of one
library, so the search is exhaustive and cheap: every candidate is timed with
CUDA events on device-resident grids, and the winner goes into the library's
tuner database (uhs_tune_put), which the planner consults whenever a caller
leaves the parameters on auto.  Every timing is also kept as a training
record for the learned cost model (costmodel.py).

Candidates (rank 3): tile {32x32 VY4, 32x16 VY4, 64x8 VY2, 32x16 VY2, and for
FP32 stars 32x32 VY8} x
loader {TMA, cp.async} x z-chunk {auto, 16, 64} x arithmetic (FP64:
{float pairs, native}); rank 2: rows {64, 128, 256} and, for stars on FP32
grids or in float pairs, two points per thread along x over {128, 256}
columns x loader x row chunk {auto, 64, 128} x arithmetic; plus the generic kernel, and on request
(include_mma) for FP32 3D boxes of radius 2 and 3 the tensor-core kernel (16
or 32 columns).  Candidates that plan to the same launch are timed once.
"""
from __future__ import annotations

import ctypes
import json
import math
import os
from dataclasses import asdict

from . import _lib
from .runtime import RunParams, launch_geometry, memref_of, memref_raw, plan
from .stencil import Stencil

STREAM, GENERIC, MMA = _lib.UHS_KERNEL_STREAM, _lib.UHS_KERNEL_GENERIC, _lib.UHS_KERNEL_MMA
TILES3 = [(32, 32, 4), (32, 16, 4), (64, 8, 2), (32, 16, 2), (32, 32, 8)]
TILES2 = [64, 128, 256]
TILES2X = [128, 256]  # rank-2 stars, two points per thread along x (vx 2)


def class_features(st: Stencil) -> list:
    """Program features: rank, radius, box, FP64, log2 extents, log2 terms,
    and whether the planner sweeps it as separable 1D passes."""
    rz, ry, rx = st.radius
    r = max(rz, ry, rx)
    box = any(sum(1 for v in t[:3] if v != 0) > 1 for t in st.terms)
    ext = [max(1, u - l) for l, u in zip(st.lb, st.ub)]
    try:
        factored = plan(st, memref_raw(1 << 20, st.sizes),
                        params=RunParams(flags=_lib.UHS_FLAG_NO_TUNE_DB)).factored
    except _lib.UhsError:
        factored = 0
    return [1.0 if st.rank == 3 else 0.0, r / 3.0, 1.0 if box else 0.0, 1.0 if st.dtype != _lib.UHS_F32 else 0.0,
            math.log2(ext[0]) / 10.0, math.log2(ext[1]) / 10.0, math.log2(ext[2]) / 13.0,
            math.log2(len(st.terms)) / 9.0, float(factored)]


def wave_features(st: Stencil, p: RunParams) -> list:
    """How a streaming launch fills the GPU (uhs_launch_geometry): log2 of its
    waves (CTAs over SMs x resident CTAs per SM), the occupied fraction of the
    last wave, and the filled fraction of the last z-chunk.  On small and
    irregular grids these decide between z-chunks of similar cost."""
    if p.kernel != STREAM:
        return [0.0, 0.0, 0.0]
    try:
        g = launch_geometry(st, memref_raw(1 << 20, st.sizes), p)
    except _lib.UhsError:
        return [0.0, 0.0, 0.0]
    if g["ctas"] <= 0:
        return [0.0, 0.0, 0.0]
    slots = max(1, g["sms"] * g["ctas_per_sm"])
    waves = g["ctas"] / slots
    tail = waves - math.floor(waves)
    nz = max(1, st.ub[0] - st.lb[0]) if st.rank == 3 else max(1, st.ub[1] - st.lb[1])
    zc = max(1, g["zchunk"])
    last = (nz % zc) / zc if nz % zc else 1.0
    return [math.log2(max(waves, 1.0 / 64)) / 6.0, tail if tail > 0 else 1.0, last]


def config_features(p: RunParams, st: Stencil | None = None) -> list:
    """Launch features of a planned configuration: tile one-hot, loader,
    arithmetic, z-chunk, generic kernel, and (given the program) how the tile
    quantises its domain: log2 CTA tiles and the idle fraction of edge tiles,
    and how the launch's CTAs fill the GPU (wave_features)."""
    tile = [0.0] * (len(TILES3) + len(TILES2) + len(TILES2X))
    if p.kernel == STREAM:
        if p.tile_y > 1:
            key = (p.tile_x, p.tile_y, p.vy)
            if key in TILES3:
                tile[TILES3.index(key)] = 1.0
        elif p.vx == 2 and p.tile_x in TILES2X:
            tile[len(TILES3) + len(TILES2) + TILES2X.index(p.tile_x)] = 1.0
        elif p.tile_x in TILES2:
            tile[len(TILES3) + TILES2.index(p.tile_x)] = 1.0
    quant = [0.0, 0.0, 0.0]
    if st is not None and p.tile_x > 0:
        ext = [max(1, u - l) for l, u in zip(st.lb, st.ub)]
        ty = max(1, p.tile_y)
        tx_n, ty_n = math.ceil(ext[2] / p.tile_x), math.ceil(ext[1] / ty) if st.rank == 3 else 1
        quant = [math.log2(tx_n * ty_n) / 16.0, tx_n * p.tile_x / ext[2] - 1.0,
                 (ty_n * ty / ext[1] - 1.0) if st.rank == 3 else 0.0]
    waves = wave_features(st, p) if st is not None else [0.0, 0.0, 0.0]
    return tile + [1.0 if p.use_tma == 1 else 0.0, 1.0 if p.arith == _lib.UHS_ARITH_DF32 else 0.0,
                   math.log2(p.tile_z) / 10.0 if p.tile_z > 0 else 0.0, 1.0 if p.kernel == GENERIC else 0.0,
                   1.0 if p.kernel == MMA else 0.0] + quant + waves


N_FEATURES = 9 + 21


def features(st: Stencil, p: RunParams, cls: list | None = None) -> list:
    return (cls if cls is not None else class_features(st)) + config_features(p, st)


def candidates(st: Stencil, include_mma: bool = False) -> list:
    """Distinct planned launches to try for st (planned without the tuner
    database so each candidate is what it says).  The tensor-core kernel is
    left out unless include_mma: its error is an order of magnitude above the
    CUDA-core FP32 sweep's, and a tuned entry is what UHS_KERNEL_AUTO runs."""
    out, seen = [], set()
    ariths = [_lib.UHS_ARITH_DF32, _lib.UHS_ARITH_FMA] if st.dtype == _lib.UHS_F64 else \
        ([_lib.UHS_ARITH_DF32] if st.dtype == _lib.UHS_F32X2 else [_lib.UHS_ARITH_FMA])
    tiles = [dict(tile_x=t[0], tile_y=t[1], vy=t[2]) for t in TILES3] if st.rank == 3 else \
        [dict(tile_x=t, vx=1) for t in TILES2] + [dict(tile_x=t, vx=2) for t in TILES2X]
    zs = [0, 16, 64] if st.rank == 3 else [0, 64, 128]
    raw = [RunParams(kernel=STREAM, arith=ar, use_tma=tma, tile_z=tz, flags=_lib.UHS_FLAG_NO_TUNE_DB, **t)
           for ar in ariths for t in tiles for tma in (1, -1) for tz in zs]
    if st.dtype != _lib.UHS_F32X2:
        raw.append(RunParams(kernel=GENERIC, arith=_lib.UHS_ARITH_FMA, flags=_lib.UHS_FLAG_NO_TUNE_DB))
    if include_mma and st.dtype == _lib.UHS_F32 and st.rank == 3:
        raw += [RunParams(kernel=MMA, tile_x=tx, flags=_lib.UHS_FLAG_NO_TUNE_DB) for tx in (16, 32)]
    # plan against the program's contiguous layout (a 256-byte aligned base,
    # as device allocations are) so loader eligibility is the grid's own
    layout = memref_raw(1 << 20, st.sizes)
    for p in raw:
        try:
            q = plan(st, layout, params=p)
        except _lib.UhsError:
            continue
        q.flags = _lib.UHS_FLAG_NO_TUNE_DB
        q.tile_z = p.tile_z
        key = tuple(asdict(q).values())
        if key in seen:
            continue
        seen.add(key)
        out.append(q)
    return out


def measure(st: Stencil, a, b, p: RunParams, reps: int = 3, stream=None, min_ms: float = 2.0) -> float:
    """Nanoseconds per point-update of one sweep with launch p: CUDA events
    around at least `reps` sweeps (alternating direction) and at least min_ms
    of GPU time, after one timed warm-up sweep that sizes the count."""
    import torch
    q = RunParams(**{**asdict(p), "flags": p.flags | _lib.UHS_FLAG_NO_SYNC | _lib.UHS_FLAG_NO_TUNE_DB})
    s1 = st.with_(iterations=1)
    d = s1.to_desc()
    ma, mb = memref_of(a), memref_of(b)
    c = q.to_c()
    L = _lib.lib()
    stream = stream or torch.cuda.current_stream()
    h = stream.cuda_stream

    def timed(k: int) -> float:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(k):
            src, dst = (ma, mb) if i % 2 == 0 else (mb, ma)
            _lib.check(L.uhs_sweep(d.ref(), ctypes.byref(src), ctypes.byref(dst), ctypes.byref(c), h))
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    first = max(timed(1), 1e-3)
    k = int(min(400, max(reps, math.ceil(min_ms / first))))
    return timed(k) * 1e6 / k / max(1, st.interior_points)


def device_grids(st: Stencil, seed: int = 0):
    """Two device grids for st filled with U[-1,1) (timing inputs)."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    shape = st.sizes if st.rank == 3 else st.sizes[1:]
    a = torch.rand(shape, generator=g, device="cuda", dtype=torch.float64).mul_(2).sub_(1)
    if st.dtype == _lib.UHS_F32:
        a = a.float()
    elif st.dtype == _lib.UHS_F32X2:
        hi = a.float()
        lo = (a - hi.double()).float()
        a = torch.stack([hi, lo], -1).view(torch.float64).reshape(shape)
    return a, a.clone()


class Tuner:
    """Exhaustive tuner with a JSON database of winners and timing records."""

    def __init__(self, path: str | None = None):
        self.path = path
        self.best = {}     # key -> {"params": {...}, "gst": x}
        self.records = []  # {"features": [...], "ns_per_point": x, "key": ..., "params": {...}}
        if path and os.path.exists(path):
            self.load(path)

    @staticmethod
    def key(st: Stencil) -> str:
        ext = "x".join(str(u - l) for l, u in zip(st.lb, st.ub))
        f = class_features(st)
        return f"r{st.rank}_R{round(f[1] * 3)}_{'box' if f[2] else 'star'}_{st.dtype}_{ext}"

    def tune(self, st: Stencil, a=None, b=None, reps: int = 3, push: bool = True, include_mma: bool = False) -> tuple:
        if a is None:
            a, b = device_grids(st)
        results = []
        cls = class_features(st)
        for p in candidates(st, include_mma):
            try:
                ns = measure(st, a, b, p, reps)
            except _lib.UhsError:
                continue
            results.append((ns, p))
            self.records.append({"key": self.key(st), "features": features(st, p, cls), "ns_per_point": ns,
                                 "params": asdict(p)})
        if not results:
            raise RuntimeError(f"no candidate ran for {st.name}")
        ns, bestp = min(results, key=lambda r: r[0])
        self.best[self.key(st)] = {"params": asdict(bestp), "gst": 1.0 / ns}
        if push:
            push_params(st, bestp, 1.0 / ns)
        return bestp, results

    def save(self, path: str | None = None) -> None:
        with open(path or self.path, "w") as f:
            json.dump({"best": self.best, "records": self.records}, f)

    def load(self, path: str) -> None:
        with open(path) as f:
            d = json.load(f)
        self.best = d.get("best", {})
        self.records = d.get("records", [])


def push_params(st: Stencil, p: RunParams, gst: float) -> None:
    q = RunParams(**{**asdict(p), "flags": 0})
    _lib.check(_lib.lib().uhs_tune_put(st.to_desc().ref(), ctypes.byref(q.to_c()), gst))


def db_get(st: Stencil):
    out = _lib.Params()
    exact = ctypes.c_int32()
    rc = _lib.lib().uhs_tune_get(st.to_desc().ref(), ctypes.byref(out), ctypes.byref(exact))
    if rc != _lib.UHS_OK:
        return None, False
    return RunParams.from_c(out), bool(exact.value)


def db_clear() -> None:
    _lib.lib().uhs_tune_clear()


def db_save(path: str) -> None:
    """Write the library's tuner database to path (uhs_tune_save)."""
    _lib.check(_lib.lib().uhs_tune_save(os.fsencode(path)))


def db_load(path: str) -> None:
    """Merge a saved tuner database into the library's (uhs_tune_load); a
    malformed file raises UhsError(UHS_EPARSE) and changes nothing."""
    _lib.check(_lib.lib().uhs_tune_load(os.fsencode(path)))
