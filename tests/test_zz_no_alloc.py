"""The allocation-free error reduction, uhs_error_norms_noalloc.

Some callers of this library cannot allocate device memory: a plugin inside
an application that owns every device allocation, a service that must not
grow its footprint after start-up, a loop that cannot afford the device-wide
synchronisation cudaMalloc may cause.  uhs_error_norms_noalloc serves them
with a fixed scratch array in the library's device memory instead of the
runtime-owned buffer uhs_error_norms allocates.  These tests call it through
the C ABI, twice in a row on different grids (the shared array keeps the
previous call's contents, which must not leak into the next result), and
check each result against uhs_error_norms on the same grids.  The file is
named so pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib
from gpu_util import to_dev
from uxxxxxxxxh_gb300.workloads import random_case

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _noalloc(st, x, ref):
    d = st.to_desc()
    mx, mr = uhs.memref_of(x), uhs.memref_of(ref)
    out = (ctypes.c_double * 4)()
    rc = _lib.lib().uhs_error_norms_noalloc(d.ref(), ctypes.byref(mx), ctypes.byref(mr), out, None)
    return rc, {"l2_rel": out[0], "max_abs": out[1], "max_rel": out[2], "max_ref": out[3]}


def test_noalloc_matches_allocating_reduction_on_two_calls_in_a_row(cuda):
    import torch
    cases = [(3, (33, 41, 70), 1e-9, np.float64), (2, (257, 300), 3e-7, np.float32)]
    for i, (rank, interior, eps, dt) in enumerate(cases):
        st, ref = random_case(rank, 1, "box", interior, 2, 40 + i)
        x = ref + eps * np.random.default_rng(i).standard_normal(ref.size)
        if dt == np.float32:
            st = st.with_(dtype=uhs.UHS_F32)
            dx = to_dev(x.astype(np.float32), st, torch.float32)
        else:
            dx = to_dev(x, st)
        dref = to_dev(ref, st)
        rc, got = _noalloc(st, dx, dref)
        assert rc == _lib.UHS_OK, _lib.last_error()
        want = uhs.error_norms(st, dx, dref)
        for k in want:
            assert got[k] == pytest.approx(want[k], rel=TOL, abs=0.0), (i, k, got, want)
        assert got["l2_rel"] > 0.0


def test_noalloc_takes_a_domain_of_any_size(cuda):
    """The reduction uses at most 608 partial slots, whatever the domain:
    524289 rows (more than 8192 slots of 64 rows would hold) and one
    4-million-wide row both fit and match the allocating reduction."""
    import torch
    for interior in ((_lib.UHS_NOALLOC_MAX_PARTIALS * 64 + 1, 2), (1, 1 << 22)):
        st, ref = random_case(2, 1, "star", interior, 2, 3)
        r = to_dev(ref, st)
        x = r + 1e-9 * torch.randn_like(r)
        rc, got = _noalloc(st, x, r)
        assert rc == _lib.UHS_OK, _lib.last_error()
        want = uhs.error_norms(st, x, r)
        assert got == want and got["l2_rel"] > 0.0


def test_noalloc_leaves_device_memory_untouched(cuda):
    """The entry point's promise: no device allocation.  After one warm-up
    call (which loads the library's device code on first use), the device's
    free memory is the same before and after further calls on a fresh
    stream."""
    import torch
    st, ref = random_case(3, 1, "star", (40, 44, 72), 2, 77)
    r = to_dev(ref, st)
    x = r + 1e-9 * torch.randn_like(r)
    stream = torch.cuda.Stream()
    d = st.to_desc()
    mx, mr = uhs.memref_of(x), uhs.memref_of(r)
    out = (ctypes.c_double * 4)()
    lib = _lib.lib()
    assert lib.uhs_error_norms_noalloc(d.ref(), ctypes.byref(mx), ctypes.byref(mr), out, None) == _lib.UHS_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        rc = lib.uhs_error_norms_noalloc(d.ref(), ctypes.byref(mx), ctypes.byref(mr), out, stream.cuda_stream)
        assert rc == _lib.UHS_OK, _lib.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert out[0] > 0.0
