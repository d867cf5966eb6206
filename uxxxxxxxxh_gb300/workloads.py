"""Seeded synthetic workloads: the benchmark configurations of the stencil backend.

All data is generated on the host from one documented generator, SplitMix64
(Steele, Lea & Flood, "Fast splittable pseudorandom number generators",
OOPSLA 2014) used counter-style: draw i of stream `seed` is
mix(seed + (i + 1) * 0x9E3779B97F4A7C15), and a double in [0, 1) is its top 53
bits times 2^-53.  The same host arrays are copied to the GPU and handed to the
CPU oracle, so both see identical inputs.

Configurations (grid = interior plus halo on every side):
  cfg1  2d1r_star f64, 4096^2, 1-cell constant halo, T = 100
  cfg2  3d1r_star f64, 512^3, 1-cell zero halo, T = 50
  cfg3  3d3r_box f64/f32, 256^3, 3-cell zero halo, Gaussian (sigma 1.5) coefficients, T = 10
  cfg4  3d2r_star, 512^3, 2-cell halo, sin(x)cos(y)sin(z) + 1e-3 noise, T = 200
"""
from __future__ import annotations

import math

import numpy as np

from .stencil import Stencil, box_offsets, make_stencil, star_offsets
from ._lib import UHS_F64

GOLDEN = np.uint64(0x9E3779B97F4A7C15)
M1 = np.uint64(0xBF58476D1CE4E5B9)
M2 = np.uint64(0x94D049BB133111EB)


def splitmix_uniform(seed: int, n: int, start: int = 0, chunk: int = 1 << 24) -> np.ndarray:
    """n doubles in [0, 1): draws start .. start+n-1 of stream `seed`."""
    out = np.empty(n, np.float64)
    s = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        for lo in range(0, n, chunk):
            hi = min(n, lo + chunk)
            z = np.arange(start + lo + 1, start + hi + 1, dtype=np.uint64)
            z *= GOLDEN
            z += s
            z ^= z >> np.uint64(30)
            z *= M1
            z ^= z >> np.uint64(27)
            z *= M2
            z ^= z >> np.uint64(31)
            z >>= np.uint64(11)
            out[lo:hi] = z.astype(np.float64) * (2.0 ** -53)
    return out


def normalised(v) -> list:
    s = float(sum(v))
    return [float(x) / s for x in v]


def interior_view(a: np.ndarray, st: Stencil) -> np.ndarray:
    g = a.reshape(st.sizes)
    return g[st.lb[0]:st.ub[0], st.lb[1]:st.ub[1], st.lb[2]:st.ub[2]]


def cfg1(n: int = 4096, T: int = 100, seed: int = 1):
    """2d1r_star: centre 0.2, neighbours U[0.1, 0.3], normalised; interior
    U[0,1); constant halo drawn from the seed (stream seed+1, draw 0)."""
    u = splitmix_uniform(seed + 7, 4)
    coefs = normalised([0.1 + 0.2 * x for x in u] + [0.2])  # y-1, y+1, x-1, x+1, centre
    st = make_stencil("cfg1_2d1r_star", 2, (n, n), 1, star_offsets(2, 1), coefs, iterations=T)
    halo = float(splitmix_uniform(seed + 1, 1)[0])
    a = np.full(int(np.prod(st.sizes)), halo)
    interior_view(a, st)[...] = splitmix_uniform(seed, n * n).reshape(1, n, n)
    return st, a


def cfg2(n: int = 512, T: int = 50, seed: int = 2):
    """3d1r_star: 7 coefficients U[0,1) normalised; interior U[-1,1); zero halo."""
    coefs = normalised(splitmix_uniform(seed + 7, 7))
    st = make_stencil("cfg2_3d1r_star", 3, (n, n, n), 1, star_offsets(3, 1), coefs, iterations=T)
    a = np.zeros(int(np.prod(st.sizes)))
    interior_view(a, st)[...] = (2.0 * splitmix_uniform(seed, n ** 3) - 1.0).reshape(n, n, n)
    return st, a


def cfg3(n: int = 256, T: int = 10, seed: int = 3):
    """3d3r_box: coefficients exp(-d^2 / (2 * 1.5^2)) normalised; interior
    U[0,1); zero halo."""
    offs = box_offsets(3, 3)
    w = [math.exp(-(dz * dz + dy * dy + dx * dx) / (2 * 1.5 ** 2)) for dz, dy, dx in offs]
    st = make_stencil("cfg3_3d3r_box", 3, (n, n, n), 3, offs, normalised(w), iterations=T)
    a = np.zeros(int(np.prod(st.sizes)))
    interior_view(a, st)[...] = splitmix_uniform(seed, n ** 3).reshape(n, n, n)
    return st, a


def cfg4(n: int = 512, T: int = 200, seed: int = 4):
    """3d2r_star: coefficients U[0,1) normalised; field sin(x)cos(y)sin(z) on
    the unit cube's grid (x = 2*pi*i/n) plus 1e-3 * U[0,1) noise; the halo
    holds the smooth field's values (no noise)."""
    coefs = normalised(splitmix_uniform(seed + 7, 13))
    st = make_stencil("cfg4_3d2r_star", 3, (n, n, n), 2, star_offsets(3, 2), coefs, iterations=T)
    sz = st.sizes
    h = 2
    z = 2 * np.pi * (np.arange(sz[0]) - h) / n
    y = 2 * np.pi * (np.arange(sz[1]) - h) / n
    x = 2 * np.pi * (np.arange(sz[2]) - h) / n
    g = (np.sin(z)[:, None, None] * np.cos(y)[None, :, None]) * np.sin(x)[None, None, :]
    a = g.reshape(-1).copy()
    interior_view(a, st)[...] += 1e-3 * splitmix_uniform(seed, n ** 3).reshape(n, n, n)
    return st, a


def random_case(rank: int, r: int, kind: str, interior, T: int, seed: int, dtype: int = UHS_F64):
    """A normalised random-coefficient case of one of the 12 shapes, U[-1,1)
    data including the halo."""
    offs = star_offsets(rank, r) if kind == "star" else box_offsets(rank, r)
    coefs = normalised(splitmix_uniform(seed + 11, len(offs)) + 0.05)
    st = make_stencil(f"{rank}d{r}r_{kind}", rank, interior, r, offs, coefs, iterations=T, dtype=dtype)
    a = 2.0 * splitmix_uniform(seed, int(np.prod(st.sizes))) - 1.0
    return st, a


def cfg5_specs(n_grids: int = 64, T: int = 20, seed: int = 5, side2=(256, 8192), side3=(64, 512)):
    """The batched mixed suite: n_grids programs drawn from the seed, each one
    of the 12 shapes ({2d,3d} x {r1,r2,r3} x {star,box}) in FP32 or FP64,
    2D sides log-uniform in side2, 3D sides log-uniform in side3 (each axis
    drawn separately, so grids are not cubic), normalised U[0,1) coefficients.
    Returns [(Stencil, data seed)]; data is U[-1,1) from that seed."""
    from ._lib import UHS_F32
    u = splitmix_uniform(seed, n_grids * 8)
    out = []
    for g in range(n_grids):
        v = u[8 * g: 8 * g + 8]
        shape = min(11, int(v[0] * 12))
        rank = 2 if shape < 6 else 3
        kind = "star" if shape % 2 == 0 else "box"
        r = 1 + (shape // 2) % 3
        lo, hi = side2 if rank == 2 else side3
        sides = [int(round(math.exp(math.log(lo) + x * (math.log(hi) - math.log(lo))))) for x in v[1:1 + rank]]
        dtype = UHS_F32 if v[4] < 0.5 else UHS_F64
        offs = star_offsets(rank, r) if kind == "star" else box_offsets(rank, r)
        coefs = normalised(splitmix_uniform(seed * 1000 + g, len(offs)) + 0.05)
        st = make_stencil(f"g{g}_{rank}d{r}r_{kind}", rank, sides, r, offs, coefs, iterations=T, dtype=dtype)
        out.append((st, seed * 7919 + g))
    return out
