"""Size-independent properties at the full sizes of the benchmark
configurations (512^3, 4096^2 and 256^3 interiors), where the oracle would
take minutes: fields and coefficients are chosen so that every path must
reproduce them exactly.

* Constant field, coefficients summing to 1 exactly (dyadic values): every
  sweep maps the constant to itself with no rounding, so after T steps the
  grid is bit-identical to its start, on every kernel, arithmetic and
  element type.
* Linear field along x under a symmetric star with dyadic coefficients: the
  field is a fixed point (the halo carries it too), and the values are
  multiples of 2^-10 below 5, so FP32, float pairs and FP64 keep it exactly.
* Cross-method agreement at full size: separable passes against the term by
  term sweep, float pairs against native FP64."""
import pytest

import uxxxxxxxxh_gb300 as uhs
from uxxxxxxxxh_gb300 import _lib
from uxxxxxxxxh_gb300.stencil import box_offsets, make_stencil, star_offsets

pytestmark = pytest.mark.gpu

F = _lib


def dyadic_star(rank, r):
    """Symmetric star coefficients, sum exactly 1: neighbours 2^-6 each,
    centre the rest."""
    offs = star_offsets(rank, r)
    nb = 1.0 / 64
    coefs = [nb if any(o) else 0.0 for o in offs]
    coefs[[i for i, o in enumerate(offs) if not any(o)][0]] = 1.0 - nb * (len(offs) - 1)
    return offs, coefs


def dyadic_box(rank, r):
    offs = box_offsets(rank, r)
    nb = 1.0 / 1024
    coefs = [nb if any(o) else 0.0 for o in offs]
    coefs[[i for i, o in enumerate(offs) if not any(o)][0]] = 1.0 - nb * (len(offs) - 1)
    return offs, coefs


def grids(st, dtype, fill):
    import torch
    shape = st.sizes if st.rank == 3 else st.sizes[1:]
    tdt = torch.float32 if dtype == F.UHS_F32 else torch.float64
    a = fill(shape, tdt)
    if dtype == F.UHS_F32X2:
        hi = a.float()
        a = torch.stack([hi, torch.zeros_like(hi)], -1).view(torch.float64).reshape(shape)
    return a, a.clone()


def const(shape, tdt):
    import torch
    return torch.full(shape, 0.5, dtype=tdt, device="cuda")


def linear_x(shape, tdt):
    import torch
    x = torch.arange(shape[-1], dtype=torch.float64, device="cuda") * 2.0 ** -10 + 0.25
    return x.expand(*shape).contiguous().to(tdt)


CASES = [  # (name, rank, interior, r, kind, T)
    ("cfg2_3d7pt_512", 3, (512, 512, 512), 1, "star", 50),
    ("cfg1_2d5pt_4096", 2, (4096, 4096), 1, "star", 100),
    ("cfg4_3d13pt_512", 3, (512, 512, 512), 2, "star", 20),
    ("cfg3_3d343pt_256", 3, (256, 256, 256), 3, "box", 10),
]
PATHS = [  # (label, element type, params)
    ("f64_auto", F.UHS_F64, uhs.RunParams()),
    ("f64_native", F.UHS_F64, uhs.RunParams(arith=F.UHS_ARITH_FMA)),
    ("f32", F.UHS_F32, uhs.RunParams()),
    ("f32x2", F.UHS_F32X2, uhs.RunParams()),
]


@pytest.mark.parametrize("name,rank,interior,r,kind,T", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("label,dtype,params", PATHS, ids=[p[0] for p in PATHS])
def test_constant_field_is_kept_exactly(cuda, name, rank, interior, r, kind, T, label, dtype, params):
    import torch
    offs, coefs = dyadic_star(rank, r) if kind == "star" else dyadic_box(rank, r)
    st = make_stencil(name, rank, interior, r, offs, coefs, iterations=T, dtype=dtype)
    a, b = grids(st, dtype, const)
    a0 = a.clone()
    uhs.run(st, a, b, params)
    torch.cuda.synchronize()
    assert torch.equal(a, a0)
    del a, b, a0


def test_constant_field_tensor_cores_and_separable_and_batch(cuda):
    """The 343-point box at 256^3: the tensor-core path, the separable path
    (the dyadic box is not rank 1, so a rank-1 dyadic box is used for it) and
    a batch of two full-size grids keep the constant exactly."""
    import torch
    offs, coefs = dyadic_box(3, 3)
    st = make_stencil("box", 3, (256, 256, 256), 3, offs, coefs, iterations=10, dtype=F.UHS_F32)
    a, b = grids(st, F.UHS_F32, const)
    a0 = a.clone()
    uhs.run(st, a, b, uhs.RunParams(kernel=F.UHS_KERNEL_MMA))
    assert torch.equal(a, a0)
    # rank-1 dyadic box: (1/4, 1/2, 1/4) per axis at radius 1, padded to radius 3
    w = [0.0, 0.0, 0.25, 0.5, 0.25, 0.0, 0.0]
    sep = [w[dz + 3] * w[dy + 3] * w[dx + 3] for dz, dy, dx in offs]
    st2 = make_stencil("sep", 3, (256, 256, 256), 3, offs, sep, iterations=10)
    c, d = grids(st2, F.UHS_F64, const)
    c0 = c.clone()
    assert uhs.plan(st2, c).factored == 1
    uhs.run(st2, c, d)
    assert torch.equal(c, c0)
    batch = uhs.Batch([st, st2], [a, c], [b, d], uhs.RunParams())
    batch.run()
    assert torch.equal(a, a0) and torch.equal(c, c0)


@pytest.mark.parametrize("name,rank,interior,r,kind,T", CASES[:3], ids=[c[0] for c in CASES[:3]])
@pytest.mark.parametrize("label,dtype,params", PATHS, ids=[p[0] for p in PATHS])
def test_linear_field_is_a_fixed_point(cuda, name, rank, interior, r, kind, T, label, dtype, params):
    import torch
    offs, coefs = dyadic_star(rank, r)
    st = make_stencil(name, rank, interior, r, offs, coefs, iterations=T, dtype=dtype)
    a, b = grids(st, dtype, linear_x)
    a0 = a.clone()
    uhs.run(st, a, b, params)
    torch.cuda.synchronize()
    assert torch.equal(a, a0)
    del a, b, a0


def test_methods_agree_at_full_size(cuda):
    """cfg3's Gaussian box at 256^3, T = 10 (a rank-1 coefficient tensor):
    separable passes against the term-by-term sweep in float pairs; and cfg2
    at 512^3, T = 50: float pairs against native FP64."""
    import torch
    from uxxxxxxxxh_gb300.workloads import cfg2, cfg3
    st, a0 = cfg3()
    x = torch.from_numpy(a0.reshape(st.sizes)).cuda()
    a, b = x.clone(), x.clone()
    uhs.run(st, a, b, uhs.RunParams(arith=F.UHS_ARITH_DF32))
    c, d = x.clone(), x.clone()
    uhs.run(st, c, d, uhs.RunParams(arith=F.UHS_ARITH_DF32, flags=F.UHS_FLAG_NO_FACTOR))
    assert uhs.plan(st, a).factored == 1
    assert float((a - c).abs().max()) <= 1e-12 * float(c.abs().max())
    del a, b, c, d, x
    st, a0 = cfg2()
    x = torch.from_numpy(a0.reshape(st.sizes)).cuda()
    a, b = x.clone(), x.clone()
    uhs.run(st, a, b, uhs.RunParams(arith=F.UHS_ARITH_DF32))
    c, d = x.clone(), x.clone()
    uhs.run(st, c, d, uhs.RunParams(arith=F.UHS_ARITH_FMA))
    assert float((a - c).abs().max()) <= 1e-12 * float(c.abs().max())
