"""Calling the C ABI on device grids.

Grids are torch CUDA tensors (torch is used for device memory and streams
only) or raw device pointers.  Each call builds the MLIR memref descriptors the
reference's drivers build (UH-GPU/3d1r_star/3d7pt_main.cpp:147-148) and goes
through uhs_run / uhs_sweep.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

from . import _lib
from .stencil import Stencil


@dataclass
class RunParams:
    kernel: int = 0
    arith: int = 0
    tile_x: int = 0
    tile_y: int = 0
    tile_z: int = 0
    k_temporal: int = 0
    use_tma: int = 0
    flags: int = 0
    vy: int = 0
    prefetch: int = 0
    factored: int = 0
    vx: int = 0

    def to_c(self) -> _lib.Params:
        p = _lib.Params(self.kernel, self.arith, self.tile_x, self.tile_y, self.tile_z, self.k_temporal,
                        self.use_tma, self.flags, self.vy, self.prefetch, self.factored, self.vx)
        return p

    @staticmethod
    def from_c(p: _lib.Params) -> "RunParams":
        return RunParams(p.kernel, p.arith, p.tile_x, p.tile_y, p.tile_z, p.k_temporal, p.use_tma, p.flags, p.vy,
                         p.prefetch, p.factored, p.vx)


def memref_of(t, rank: int | None = None) -> _lib.Memref:
    """Memref descriptor of a contiguous-in-x torch tensor of rank 2 or 3."""
    shape = list(t.shape)
    strides = list(t.stride())
    if len(shape) == 2:
        shape = [1] + shape
        strides = [shape[1] * strides[0]] + strides
    if len(shape) != 3:
        raise ValueError("grids are rank-2 or rank-3 tensors")
    m = _lib.Memref()
    m.allocated = t.data_ptr()
    m.aligned = t.data_ptr()
    m.offset = 0
    for i in range(3):
        m.sizes[i] = shape[i]
        m.strides[i] = strides[i]
    return m


def memref_raw(ptr: int, sizes, strides=None) -> _lib.Memref:
    sizes = list(sizes)
    if strides is None:
        strides = [sizes[1] * sizes[2], sizes[2], 1]
    m = _lib.Memref()
    m.allocated = ptr
    m.aligned = ptr
    m.offset = 0
    for i in range(3):
        m.sizes[i] = sizes[i]
        m.strides[i] = strides[i]
    return m


def _stream_handle(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


def run(stencil: Stencil, a, b, params: RunParams | None = None, stream=None) -> None:
    """Run the program (T = stencil.iterations) on device grids a and b."""
    d = stencil.to_desc()
    ma = a if isinstance(a, _lib.Memref) else memref_of(a)
    mb = b if isinstance(b, _lib.Memref) else memref_of(b)
    p = (params or RunParams()).to_c()
    _lib.check(_lib.lib().uhs_run(d.ref(), ctypes.byref(ma), ctypes.byref(mb), ctypes.byref(p),
                                  _stream_handle(stream)))


def sweep(stencil: Stencil, src, dst, params: RunParams | None = None, stream=None) -> None:
    """One sweep src -> dst."""
    d = stencil.to_desc()
    ma = src if isinstance(src, _lib.Memref) else memref_of(src)
    mb = dst if isinstance(dst, _lib.Memref) else memref_of(dst)
    p = (params or RunParams()).to_c()
    _lib.check(_lib.lib().uhs_sweep(d.ref(), ctypes.byref(ma), ctypes.byref(mb), ctypes.byref(p),
                                    _stream_handle(stream)))


def plan(stencil: Stencil, a=None, params: RunParams | None = None) -> RunParams:
    d = stencil.to_desc()
    out = _lib.Params()
    p = (params or RunParams()).to_c()
    ma = (a if isinstance(a, _lib.Memref) else memref_of(a)) if a is not None else None
    _lib.check(_lib.lib().uhs_plan(d.ref(), ctypes.byref(ma) if ma is not None else None, ctypes.byref(p),
                                   ctypes.byref(out)))
    return RunParams.from_c(out)


def launch_geometry(stencil: Stencil, a=None, params: RunParams | None = None) -> dict:
    """The planned streaming launch's z-chunk, CTAs per SM, CTA count and the
    device's SM count (uhs_launch_geometry)."""
    d = stencil.to_desc()
    out = (ctypes.c_int64 * 4)()
    p = (params or RunParams()).to_c()
    ma = (a if isinstance(a, _lib.Memref) else memref_of(a)) if a is not None else None
    _lib.check(_lib.lib().uhs_launch_geometry(d.ref(), ctypes.byref(ma) if ma is not None else None,
                                              ctypes.byref(p), out))
    return {"zchunk": out[0], "ctas_per_sm": out[1], "ctas": out[2], "sms": out[3]}


def validate(stencil: Stencil, a, b) -> None:
    d = stencil.to_desc()
    ma = a if isinstance(a, _lib.Memref) else memref_of(a)
    mb = b if isinstance(b, _lib.Memref) else memref_of(b)
    _lib.check(_lib.lib().uhs_validate(d.ref(), ctypes.byref(ma), ctypes.byref(mb)))


def launch_count() -> int:
    return int(_lib.lib().uhs_launch_count())


def probe_wait_timeout(cycles: int, stream=None) -> int:
    """Run the failure-reporting probe (uhs_probe_wait_timeout): a device wait
    that runs out after `cycles` SM clocks.  Returns the status code (the
    library reports UHS_ETIMEOUT); uhs_last_error() holds the message."""
    return int(_lib.lib().uhs_probe_wait_timeout(int(cycles), _stream_handle(stream)))


def probe_dfma_rate(stream=None) -> float:
    """FP64 pipe rate of the current device, DFMA per second
    (uhs_probe_dfma_rate)."""
    v = ctypes.c_double()
    _lib.check(_lib.lib().uhs_probe_dfma_rate(ctypes.byref(v), _stream_handle(stream)))
    return v.value


def release_scratch() -> None:
    """Return the memory kept by the library's scratch pools (uhs_release_scratch)."""
    _lib.check(_lib.lib().uhs_release_scratch())


def error_norms(stencil: Stencil, x, ref, stream=None) -> dict:
    """FP64 error of device grid x against the FP64 device grid ref over the
    stencil's domain, reduced on the GPU (uhs_error_norms)."""
    d = stencil.to_desc()
    mx = x if isinstance(x, _lib.Memref) else memref_of(x)
    mr = ref if isinstance(ref, _lib.Memref) else memref_of(ref)
    out = (ctypes.c_double * 4)()
    _lib.check(_lib.lib().uhs_error_norms(d.ref(), ctypes.byref(mx), ctypes.byref(mr), out, _stream_handle(stream)))
    return {"l2_rel": out[0], "max_abs": out[1], "max_rel": out[2], "max_ref": out[3]}


class Batch:
    """Many programs advanced together: one persistent launch per timestep,
    the timestep loop replayed from a CUDA graph (uhs_batch_*)."""

    def __init__(self, stencils, grids_a, grids_b, params: RunParams | None = None):
        n = len(stencils)
        self._holders = [s.to_desc() for s in stencils]
        self._descs = (_lib.StencilDesc * n)(*[h.desc for h in self._holders])
        self._a = (_lib.Memref * n)(*[g if isinstance(g, _lib.Memref) else memref_of(g) for g in grids_a])
        self._b = (_lib.Memref * n)(*[g if isinstance(g, _lib.Memref) else memref_of(g) for g in grids_b])
        self._keep = (grids_a, grids_b)
        p = (params or RunParams()).to_c()
        self._h = ctypes.c_void_p()
        _lib.check(_lib.lib().uhs_batch_create(self._descs, self._a, self._b, n, ctypes.byref(p),
                                               ctypes.byref(self._h)))

    def run(self, stream=None, sync: bool = True) -> None:
        _lib.check(_lib.lib().uhs_batch_run(self._h, _stream_handle(stream), 0 if sync else _lib.UHS_FLAG_NO_SYNC))

    def stats(self) -> dict:
        l, s, i = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        _lib.check(_lib.lib().uhs_batch_stats(self._h, ctypes.byref(l), ctypes.byref(s), ctypes.byref(i)))
        return {"launches": l.value, "steps": s.value, "items": i.value}

    def close(self) -> None:
        if self._h:
            _lib.lib().uhs_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
