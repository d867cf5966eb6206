"""Stencil programs on the host side: the Python mirror of uhs_stencil_desc.

A Stencil is what one UHStencil .dsl program describes for the backend: the
padded grid extents, the domain [lb, ub) written by each sweep, the linear
expression sum_k c_k * in[p + o_k] in the order the DSL writes it, the element
type and the iteration count T (UHStencil/include/Parser/AST.h:160-244 holds
the same facts as an AST).
"""
from __future__ import annotations

import ctypes
import itertools
from dataclasses import dataclass, field, replace
from typing import Sequence

from . import _lib
from ._lib import UHS_F32, UHS_F32X2, UHS_F64

DTYPE_NAMES = {UHS_F64: "f64", UHS_F32: "f32", UHS_F32X2: "f32x2"}
DTYPE_CODES = {v: k for k, v in DTYPE_NAMES.items()}


@dataclass
class Stencil:
    name: str
    rank: int
    sizes: tuple  # padded extents, rank 3 (sizes[0] == 1 for rank 2)
    lb: tuple
    ub: tuple
    terms: list  # [(dz, dy, dx, coef), ...] in expression order
    iterations: int = 1
    dtype: int = UHS_F64
    params: list = field(default_factory=list)
    param_terms: dict = field(default_factory=dict)  # term index -> parameter index
    exact_order: bool = True  # linear form rounds like the DSL expression

    # -- derived facts ------------------------------------------------------
    @property
    def nterms(self) -> int:
        return len(self.terms)

    @property
    def radius(self) -> tuple:
        rz = max(abs(t[0]) for t in self.terms)
        ry = max(abs(t[1]) for t in self.terms)
        rx = max(abs(t[2]) for t in self.terms)
        return rz, ry, rx

    @property
    def interior_points(self) -> int:
        n = 1
        for a, b in zip(self.lb, self.ub):
            n *= max(0, b - a)
        return n

    @property
    def shape(self) -> tuple:
        return tuple(self.sizes[3 - self.rank:])

    @property
    def elem_bytes(self) -> int:
        return 8 if self.dtype == UHS_F64 else 4

    def with_(self, **kw) -> "Stencil":
        return replace(self, **kw)

    def coefficients(self) -> list:
        out = []
        for i, t in enumerate(self.terms):
            out.append(self.params[self.param_terms[i]] if i in self.param_terms else t[3])
        return out

    # -- C ABI ---------------------------------------------------------------
    def to_desc(self) -> "DescHolder":
        return DescHolder(self)


class DescHolder:
    """A uhs_stencil_desc plus the arrays it points into (kept alive here)."""

    def __init__(self, s: Stencil):
        n = s.nterms
        self.terms = (_lib.Term * n)()
        for i, (dz, dy, dx, c) in enumerate(s.terms):
            self.terms[i] = _lib.Term(dz, dy, dx, s.param_terms.get(i, -1), float(c))
        self.params = (ctypes.c_double * max(1, len(s.params)))(*s.params) if s.params else None
        self.desc = _lib.StencilDesc()
        self.desc.rank = s.rank
        self.desc.dtype = s.dtype
        for i in range(3):
            self.desc.lb[i] = s.lb[i]
            self.desc.ub[i] = s.ub[i]
        self.desc.nterms = n
        self.desc.terms = ctypes.cast(self.terms, ctypes.POINTER(_lib.Term))
        self.desc.iterations = s.iterations
        if self.params is not None:
            self.desc.params = ctypes.cast(self.params, ctypes.POINTER(ctypes.c_double))
            self.desc.nparams = len(s.params)

    def ref(self):
        return ctypes.byref(self.desc)


# ---------------------------------------------------------------------------
# Shape generators: the 12 cases {2d,3d} x {r1,r2,r3} x {star,box}
# ---------------------------------------------------------------------------
def star_offsets(rank: int, r: int) -> list:
    """Star of radius r: per axis (slowest first) -1, +1, -2, +2, ..., then the
    centre -- the order the reference's 3d7pt program writes its terms
    (UH-GPU/3d1r_star/stencil_3d7pt_star.dsl)."""
    offs = []
    axes = [0, 1, 2] if rank == 3 else [1, 2]
    for ax in axes:
        for d in range(1, r + 1):
            for s in (-d, d):
                o = [0, 0, 0]
                o[ax] = s
                offs.append(tuple(o))
    offs.append((0, 0, 0))
    return offs


def box_offsets(rank: int, r: int) -> list:
    """Box of radius r in lexicographic (dz, dy, dx) order."""
    zr = range(-r, r + 1) if rank == 3 else [0]
    return [(dz, dy, dx) for dz, dy, dx in itertools.product(zr, range(-r, r + 1), range(-r, r + 1))]


def make_stencil(name: str, rank: int, interior: Sequence[int], radius: int, offsets: list, coefs: Sequence[float],
                 iterations: int = 2, dtype: int = UHS_F64) -> Stencil:
    """Grid of the given interior extents (slowest first) with a `radius`-cell
    halo on every side; the domain is the interior."""
    if len(interior) != rank:
        raise ValueError("interior must have `rank` extents")
    inner = [1] * (3 - rank) + list(interior)
    halo = [0] * (3 - rank) + [radius] * rank
    sizes = tuple(n + 2 * h for n, h in zip(inner, halo))
    lb = tuple(halo)
    ub = tuple(h + n for n, h in zip(inner, halo))
    terms = [(o[0], o[1], o[2], float(c)) for o, c in zip(offsets, coefs)]
    return Stencil(name=name, rank=rank, sizes=sizes, lb=lb, ub=ub, terms=terms, iterations=iterations, dtype=dtype)


def shape_name(rank: int, r: int, kind: str) -> str:
    return f"{rank}d{r}r_{kind}"


SHAPES = [(rank, r, kind) for rank in (2, 3) for kind in ("star", "box") for r in (1, 2, 3)]


def offsets_for(rank: int, r: int, kind: str) -> list:
    return star_offsets(rank, r) if kind == "star" else box_offsets(rank, r)


# ---------------------------------------------------------------------------
# DSL
# ---------------------------------------------------------------------------
def parse_dsl(text: str, filename: str = "<dsl>") -> Stencil:
    """Parse UHStencil DSL text with the library's reader (include/uhs_dsl.h)."""
    L = _lib.lib()
    prog = ctypes.c_void_p()
    _lib.check(L.uhs_dsl_parse(text.encode(), filename.encode(), ctypes.byref(prog)))
    try:
        d = _lib.StencilDesc()
        sizes = (ctypes.c_int64 * 3)()
        _lib.check(L.uhs_program_desc(prog, ctypes.byref(d), sizes))
        terms, param_terms = [], {}
        for i in range(d.nterms):
            t = d.terms[i]
            terms.append((t.dz, t.dy, t.dx, t.coef))
            if t.param >= 0:
                param_terms[i] = t.param
        params = [d.params[i] for i in range(d.nparams)] if d.nparams else []
        return Stencil(name=L.uhs_program_name(prog).decode(), rank=d.rank, sizes=tuple(sizes), lb=tuple(d.lb),
                       ub=tuple(d.ub), terms=terms, iterations=d.iterations, dtype=d.dtype, params=params,
                       param_terms=param_terms, exact_order=bool(L.uhs_program_exact_order(prog)))
    finally:
        L.uhs_program_free(prog)


def parse_dsl_file(path: str) -> Stencil:
    with open(path) as f:
        return parse_dsl(f.read(), path)
