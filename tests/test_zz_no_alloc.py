"""The allocation-free timestep estimate, called through the C ABI.

phx_estimate_timestep_static exists for callers that may not allocate device
memory (they cannot create a phx_ctx): its only scratch is a fixed
__device__ array inside the library.  This file checks, on the GPU, that two
calls in a row give the same result as the context-based
phx_estimate_timestep (the reduction is a min, so the results are equal bit
for bit) for 1D, 2D and 3D blocks, with the default and with a padded
variable stride, with cell speeds alone and with face speeds; that a smaller
second call is not disturbed by what the first left in the shared scratch;
that both entry points refuse a variable stride smaller than the block; and
that a block above the stated maximum is refused before anything is
launched.  It sits in a file of its own that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

from phoebus_gb300 import abi
from phoebus_gb300.block import _ptr

pytestmark = pytest.mark.gpu

SHAPES = {1: (40, 1, 1), 2: (24, 20, 1), 3: (24, 16, 12)}


def _speeds_block(ndim, nx, pad, seed, dev="cuda"):
    """A phx_block whose cell and face signal speeds are seeded random values
    (a few NaNs included) laid out with var_stride = N + pad; prim/cons point
    at a small tensor (the timestep reads neither).  Returns (struct, keep)."""
    import torch

    ng = 4
    n1t = nx[0] + 2 * ng
    n2t = nx[1] + 2 * ng if ndim >= 2 else 1
    n3t = nx[2] + 2 * ng if ndim >= 3 else 1
    N = n1t * n2t * n3t
    vs = N + pad
    rng = np.random.default_rng(seed)
    cs = rng.uniform(0.05, 1.0, (3, vs))
    fs = rng.uniform(0.05, 1.0, (3, vs))
    cs[0, rng.integers(0, N, 3)] = np.nan
    cell = torch.from_numpy(cs).to(dev)
    face = torch.from_numpy(fs).to(dev)
    dummy = torch.zeros(16, dtype=torch.float64, device=dev)
    s = abi.BlockS()
    s.nx1, s.nx2, s.nx3 = nx
    s.ng, s.ndim = ng, ndim
    s.var_stride = vs if pad else 0
    s.dx1, s.dx2, s.dx3 = 1.0 / nx[0], 1.3 / nx[1], 0.7 / nx[2]
    s.prim = s.cons = _ptr(dummy)
    s.cell_sig, s.face_sig = _ptr(cell), _ptr(face)
    s.geom = None
    return s, (cell, face, dummy)


def _static(lib, p, s, use_face):
    import torch

    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    st = lib.phx_estimate_timestep_static(C.byref(p), C.byref(s), int(use_face), out.data_ptr(),
                                          torch.cuda.current_stream().cuda_stream)
    assert st == 0, f"status {st}: {lib.phx_last_error().decode()}"
    torch.cuda.synchronize()
    return out.item()


def _context(ctx, p, s, use_face):
    import torch

    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    st = ctx.lib.phx_estimate_timestep(ctx.h, C.byref(p), C.byref(s), int(use_face), out.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream)
    assert st == 0, f"status {st}: {ctx.lib.phx_last_error().decode()}"
    torch.cuda.synchronize()
    return out.item()


@pytest.mark.parametrize("use_face", [0, 1])
@pytest.mark.parametrize("pad", [0, 1000])
@pytest.mark.parametrize("ndim", [1, 2, 3])
def test_static_timestep_matches_context_version(built, ndim, pad, use_face):
    """Two calls in a row: a larger block, then a smaller one (stale partial
    minima of the first call must not reach the second); each equals the
    context version bit for bit."""
    from phoebus_gb300.fluid import FluidContext

    ctx = FluidContext(0, exact=False)
    p = abi.default_params(cfl=0.3)
    big = tuple(2 * x if d < ndim else 1 for d, x in enumerate(SHAPES[ndim]))
    s1, keep1 = _speeds_block(ndim, big, pad, 100 + ndim)
    s2, keep2 = _speeds_block(ndim, SHAPES[ndim], pad, 200 + ndim)
    got1 = _static(ctx.lib, p, s1, use_face)
    ref1 = _context(ctx, p, s1, use_face)
    assert got1 == ref1 and np.isfinite(got1) and got1 > 0
    got2 = _static(ctx.lib, p, s2, use_face)
    ref2 = _context(ctx, p, s2, use_face)
    assert got2 == ref2
    assert got1 != got2
    ctx.check()
    ctx.close()


def test_static_timestep_rejects_short_var_stride(built):
    """var_stride below the block's size: both entry points refuse it with
    PHX_ERR_INVALID_ARG and say why in phx_last_error."""
    from phoebus_gb300.fluid import FluidContext

    ctx = FluidContext(0, exact=False)
    p = abi.default_params()
    s, keep = _speeds_block(3, SHAPES[3], 0, 7)
    s.var_stride = 100  # far below N
    import torch

    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")  # nothing may be written
    st = ctx.lib.phx_estimate_timestep_static(C.byref(p), C.byref(s), 1, out.data_ptr(), None)
    assert st == abi.PHX_ERR_INVALID_ARG
    assert b"var_stride" in ctx.lib.phx_last_error()
    st = ctx.lib.phx_estimate_timestep(ctx.h, C.byref(p), C.byref(s), 1, out.data_ptr(), None)
    assert st == abi.PHX_ERR_INVALID_ARG
    torch.cuda.synchronize()
    assert out.item() == -1.0
    ctx.close()


def test_static_timestep_rejects_oversized_block(built):
    import torch

    lib = abi.load(False)
    p = abi.default_params()
    tiny = torch.zeros(16, dtype=torch.float64, device="cuda")  # real address, never read
    s = abi.BlockS()
    s.nx1, s.nx2, s.nx3, s.ng, s.ndim = 257, 256, 256, 4, 3  # 16,842,752 > PHX_DT_STATIC_MAX_ZONES
    s.dx1 = s.dx2 = s.dx3 = 1.0
    s.cell_sig = s.face_sig = _ptr(tiny)
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = lib.phx_estimate_timestep_static(C.byref(p), C.byref(s), 1, out.data_ptr(), None)
    assert st == abi.PHX_ERR_CAPACITY
    assert b"PHX_DT_STATIC_MAX_ZONES" in lib.phx_last_error()
    torch.cuda.synchronize()
    assert out.item() == 0.0
