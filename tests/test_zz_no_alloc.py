"""The allocation-free timestep estimate, called through the C ABI.

phx_estimate_timestep_static exists for callers that may not allocate device
memory (they cannot create a phx_ctx): its only scratch is a fixed
__device__ array inside the library.  This file checks, on the GPU, that two
calls in a row give the same result as the context-based
phx_estimate_timestep (the reduction is a min, so the results are equal bit
for bit), that a smaller second call is not disturbed by what the first left
in the shared scratch, and that a block above the stated maximum is refused
before anything is launched.  It sits in a file of its own that pytest
collects last.
"""
import ctypes as C

import numpy as np
import pytest

from phoebus_gb300 import abi, states
from phoebus_gb300.block import _ptr

pytestmark = pytest.mark.gpu


def _prepared_block(n, seed, p, ctx):
    hb = states.random_block(n, seed)
    db = hb.to_device()
    ctx.Initialize(p, db)
    ctx.CalculateFluxes(p, db)  # face signal speeds for use_face_speeds = 1
    return db


def _static_dt(lib, p, db, use_face):
    import torch

    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    s = db.struct()
    st = lib.phx_estimate_timestep_static(C.byref(p), C.byref(s), int(use_face), out.data_ptr(),
                                          torch.cuda.current_stream().cuda_stream)
    assert st == 0, f"status {st}"
    torch.cuda.synchronize()
    return out.item()


def test_static_timestep_matches_context_version(built):
    import torch

    from phoebus_gb300.fluid import FluidContext

    ctx = FluidContext(0, exact=False)
    lib = ctx.lib
    p = abi.default_params(Gamma=4.0 / 3.0, c2p_tol=1e-10, c2p_max_iter=100, cfl=0.3)
    big = _prepared_block(24, 101, p, ctx)
    small = _prepared_block(12, 202, p, ctx)
    # first call: the larger block (more partial minima written to the scratch)
    ref1 = ctx.EstimateTimestepBlock(p, big, False).item()
    got1 = _static_dt(lib, p, big, False)
    assert got1 == ref1
    # second call in a row: a smaller block; stale partials must not leak in
    ref2 = ctx.EstimateTimestepBlock(p, small, True).item()
    got2 = _static_dt(lib, p, small, True)
    assert got2 == ref2
    assert got1 != got2
    ctx.check()
    ctx.close()
    torch.cuda.synchronize()


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
    assert st == 7  # PHX_ERR_CAPACITY
    torch.cuda.synchronize()
    assert out.item() == 0.0
