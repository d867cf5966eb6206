"""The C-ABI library loads, exports every entry point include/*.h declares,
and rejects malformed calls with the documented status codes -- all without
a GPU (validation never touches the device)."""
import ctypes
import os
import re

import pytest

import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\(", text, flags=re.M):
            name = m.group(1)
            if name not in ("if", "for", "while", "return", "sizeof") and not text[m.start():].startswith("#"):
                names.add(name)
    return sorted(n for n in names if n.startswith(("uhs_", "_mlir_ciface_")))


def test_library_exports_every_declared_symbol():
    lib = uhs.lib()
    declared = _declared_functions()
    assert "uhs_run" in declared and "uhs_dsl_parse" in declared
    for name in declared:
        assert hasattr(lib, name), f"libuhs.so does not export {name}"
        assert name in _lib.SIGNATURES, f"{name} has no ctypes signature in _lib.SIGNATURES"


def test_abi_version():
    assert uhs.lib().uhs_abi_version() == 1


def _grid(st, ptr=0x10000):
    return uhs.memref_raw(ptr, st.sizes)


def _st(**kw):
    st = uhs.make_stencil("t", 3, (8, 8, 8), 1, uhs.star_offsets(3, 1), [1 / 7] * 7, iterations=2)
    return st.with_(**kw)


def _validate(st, a, b):
    d = st.to_desc()
    return uhs.lib().uhs_validate(d.ref(), ctypes.byref(a), ctypes.byref(b))


def test_validate_accepts_a_good_program():
    st = _st()
    assert _validate(st, _grid(st, 0x10000), _grid(st, 0x20000)) == _lib.UHS_OK


@pytest.mark.parametrize("mutate,code", [
    (dict(iterations=3), _lib.UHS_EINVAL),          # odd T > 1 (MLIRGen.cpp:317)
    (dict(rank=4), _lib.UHS_EINVAL),
    (dict(dtype=9), _lib.UHS_EINVAL),
    (dict(lb=(0, 1, 1)), _lib.UHS_EINVAL),          # z-1 reaches below the grid
    (dict(ub=(10, 9, 9)), _lib.UHS_EINVAL),         # z+1 reaches past the grid
    (dict(terms=[(5, 0, 0, 1.0)]), _lib.UHS_EUNSUPPORTED),
    (dict(terms=[]), _lib.UHS_EUNSUPPORTED),
])
def test_validate_rejects(mutate, code):
    st = _st(**mutate)
    assert _validate(st, _grid(st, 0x10000), _grid(st, 0x20000)) == code
    assert uhs.lib().uhs_last_error()


def test_validate_rejects_bad_memrefs():
    st = _st()
    a, b = _grid(st, 0x10000), _grid(st, 0x20000)
    assert _validate(st, a, _grid(st, 0x10000)) == _lib.UHS_EINVAL          # same grid twice
    b.strides[2] = 2
    assert _validate(st, a, b) == _lib.UHS_EUNSUPPORTED                     # non-unit x stride
    b = _grid(st, 0x20000)
    b.sizes[1] = 9
    assert _validate(st, a, b) == _lib.UHS_EINVAL                           # shapes differ
    b = _grid(st, 0x20004)
    assert _validate(st, a, b) == _lib.UHS_EINVAL                           # misaligned doubles
    assert _validate(st, a, uhs.memref_raw(0, st.sizes)) == _lib.UHS_EINVAL  # NULL
    span = 8 * st.sizes[0] * st.sizes[1] * st.sizes[2]
    assert _validate(st, a, _grid(st, 0x10000 + span)) == _lib.UHS_OK        # adjacent: fine
    assert _validate(st, a, _grid(st, 0x10000 + span - 8)) == _lib.UHS_EINVAL  # last cell shared
    assert "overlap" in _lib.last_error()
    assert _validate(st, _grid(st, 0x10000 + span - 8), a) == _lib.UHS_EINVAL


def test_errors_raise_in_python():
    st = _st(iterations=5)
    with pytest.raises(uhs.UhsError) as ei:
        uhs.validate(st, _grid(st, 0x10000), _grid(st, 0x20000))
    assert "multiple of 2" in str(ei.value)


def test_wait_probe_rejects_bad_bounds_without_a_gpu():
    """The failure probe validates its bound on the host, before any CUDA call."""
    for cycles in (0, -5, (1 << 31) + 1):
        assert uhs.probe_wait_timeout(cycles) == _lib.UHS_EINVAL
        assert "cycles" in _lib.last_error()


def test_short_or_one_sided_reach_runs_on_the_generic_kernel():
    """The templated star/box kernels read every cell within R on every axis;
    a program reaching less (no z offsets, or only one side) must be planned
    on the generic kernel, which reads only what the program reads."""
    from uxxxxxxxxh_gb300.stencil import Stencil
    # 3D, in-plane 5-point star, no z halo at all
    st = Stencil(name="inplane", rank=3, sizes=(4, 10, 12), lb=(0, 1, 1), ub=(4, 9, 11),
                 terms=[(0, -1, 0, 0.2), (0, 0, -1, 0.2), (0, 0, 0, 0.2), (0, 0, 1, 0.2), (0, 1, 0, 0.2)],
                 iterations=2)
    assert uhs.plan(st).kernel == uhs.UHS_KERNEL_GENERIC
    with pytest.raises(uhs.UhsError):
        uhs.plan(st, params=uhs.RunParams(kernel=uhs.UHS_KERNEL_STREAM))
    # one-sided z reach (dz in {-1, 0}), halo only below
    st2 = Stencil(name="upwind", rank=3, sizes=(6, 10, 12), lb=(1, 1, 1), ub=(6, 9, 11),
                  terms=[(-1, 0, 0, 0.25), (0, -1, 0, 0.125), (0, 0, -1, 0.125), (0, 0, 0, 0.25), (0, 0, 1, 0.125),
                         (0, 1, 0, 0.125)], iterations=2)
    assert uhs.plan(st2).kernel == uhs.UHS_KERNEL_GENERIC
    # a full star still plans on the streaming kernel
    st3 = st2.with_(terms=st2.terms + [(1, 0, 0, 0.0)], ub=(5, 9, 11))
    assert uhs.plan(st3).kernel == uhs.UHS_KERNEL_STREAM


def _header_constants():
    """Every UHS_* enumerator and numeric #define of include/uhs.h with its
    value (enumerators without an initialiser count up from the previous)."""
    text = open(os.path.join(ROOT, "include", "uhs.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    out = {}
    for body in re.findall(r"enum\s*(?:\w+\s*)?(?::\s*\w+\s*)?\{(.*?)\}", text, flags=re.S):
        value = -1
        for item in body.split(","):
            item = item.strip()
            if not item:
                continue
            m = re.fullmatch(r"(UHS_\w+)\s*(?:=\s*(-?\w+))?", item)
            assert m, item
            value = int(m.group(2), 0) if m.group(2) is not None else value + 1
            out[m.group(1)] = value
    for name, val in re.findall(r"^#define\s+(UHS_\w+)\s+(-?\d+)\s*$", text, flags=re.M):
        out[name] = int(val)
    return out


def test_python_constants_mirror_the_header():
    consts = _header_constants()
    assert {"UHS_OK", "UHS_F32X2", "UHS_ARITH_DF32", "UHS_KERNEL_MMA", "UHS_FLAG_IN_PLACE"} <= set(consts)
    for name, value in consts.items():
        if name == "UHS_ABI_VERSION":
            continue
        assert hasattr(_lib, name), f"_lib has no {name}"
        assert getattr(_lib, name) == value, (name, getattr(_lib, name), value)
