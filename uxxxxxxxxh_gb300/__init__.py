"""uxxxxxxxxh_gb300 -- GB300-native stencil backend for UHStencil.

The product is libuhs.so (C ABI in include/uhs.h): hand-written sm_103a sweep
kernels and the host runtime that replaces UHStencil's generated
<name>_iteration entry.  This package is the Python mirror of that interface
(descriptors, DSL reader, run/sweep calls); it holds no compute of its own.
"""
from ._lib import (UHS_ARITH_AUTO, UHS_ARITH_DF32, UHS_ARITH_EXACT, UHS_ARITH_FMA, UHS_F32, UHS_F32X2, UHS_F64,
                   UHS_FLAG_IN_PLACE, UHS_FLAG_MMA_TMEM_A, UHS_FLAG_NO_FACTOR, UHS_FLAG_NO_SYNC, UHS_FLAG_NO_TUNE_DB,
                   UHS_FLAG_XSHUFFLE,
                   UHS_KERNEL_AUTO, UHS_KERNEL_GENERIC, UHS_KERNEL_MMA, UHS_KERNEL_STREAM, UhsError, lib)
from .runtime import (Batch, RunParams, error_norms, launch_count, launch_geometry, memref_of, memref_raw, plan,
                      probe_dfma_rate,
                      probe_wait_timeout, release_scratch, run, sweep, validate)
from .stencil import (SHAPES, Stencil, box_offsets, make_stencil, offsets_for, parse_dsl, parse_dsl_file,
                      shape_name, star_offsets)

__all__ = [
    "UHS_ARITH_AUTO", "UHS_ARITH_DF32", "UHS_ARITH_EXACT", "UHS_ARITH_FMA", "UHS_F32", "UHS_F32X2", "UHS_F64",
    "UHS_FLAG_IN_PLACE", "UHS_FLAG_MMA_TMEM_A", "UHS_FLAG_NO_FACTOR", "UHS_FLAG_NO_SYNC", "UHS_FLAG_NO_TUNE_DB",
    "UHS_FLAG_XSHUFFLE",
    "UHS_KERNEL_AUTO", "UHS_KERNEL_GENERIC", "UHS_KERNEL_MMA", "UHS_KERNEL_STREAM", "UhsError", "lib",
    "Batch", "RunParams", "error_norms", "launch_count", "launch_geometry", "memref_of", "memref_raw", "plan",
    "probe_dfma_rate",
    "probe_wait_timeout", "release_scratch", "run", "sweep", "validate", "SHAPES",
    "Stencil", "box_offsets", "make_stencil", "offsets_for", "parse_dsl", "parse_dsl_file", "shape_name",
    "star_offsets",
]
