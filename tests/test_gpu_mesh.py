"""Tiled meshes (phx_stage_mesh, phx_mesh_exchange): the primitive ghost
exchange with physical boundaries, its agreement with a single periodic
block, batched against block-by-block launches, and the magnetised torus
state on an FMKS mesh."""
import math

import numpy as np
import pytest

from phoebus_gb300 import abi, states, torus
from phoebus_gb300.mesh import TiledMesh
from tests.util import assert_bitwise, host

pytestmark = pytest.mark.gpu


def mink_params():
    return abi.default_params(Gamma=4.0 / 3.0, recon="linear", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)


def tiled_from_block(b, segs):
    """A periodic TiledMesh covering block b's interior, its blocks holding
    the corresponding interior primitives."""
    n = b.nx
    mesh = TiledMesh(n, segs, b.xmin, tuple(b.xmin[d] + n[d] * b.dx[d] for d in range(3)),
                     (abi.BC_PERIODIC,) * 3, (abi.BC_PERIODIC,) * 3, ng=b.ng)
    blocks = mesh.make_blocks("cuda")
    ng = b.ng
    for (s1, s2, s3), blk in zip(mesh.segments(), blocks):
        i0, j0, k0 = mesh.starts[0][s1], mesh.starts[1][s2], mesh.starts[2][s3]
        n1, n2, n3 = blk.nx
        blk["prim"][:, ng:ng + n3, ng:ng + n2, ng:ng + n1] = b["prim"][:, ng + k0:ng + k0 + n3, ng + j0:ng + j0 + n2,
                                                                      ng + i0:ng + i0 + n1]
    return mesh, blocks


def init_mesh(ctx, p, mesh, blocks):
    for blk in blocks:
        ctx.PrimitiveToConserved(p, blk, *blk.interior())
    ctx.MeshExchange(p, mesh, blocks)
    for blk in blocks:
        ctx.ConservedToPrimitive(p, blk)


def rk2_mesh(ctx, p, mesh, blocks, seconds, dt, batched=True, learned=False):
    bases = [b["cons"] for b in blocks]
    ctx.StageMesh(p, mesh, blocks, bases, seconds, 1.0, dt, learned=learned, batched=batched)
    stage2 = []
    for b, s in zip(blocks, seconds):
        c = states.Block(b.nx, b.ng, b.ndim, b.xmin, b.dx, backend="torch", device="cuda", arrays=dict(b.arrays),
                         geom=b.geom)
        c.arrays["cons"] = s
        stage2.append(c)
    ctx.StageMesh(p, mesh, stage2, bases, bases, 0.5, dt, learned=learned, batched=batched)


def test_periodic_mesh_matches_single_block(ctx_exact):
    """A periodic 16^3 state split into 2 x 2 x 2 uneven blocks evolves like
    the single periodic block; the exchange moves primitives instead of
    conserved variables, so ghost zones agree to the con2prim tolerance."""
    import torch

    from phoebus_gb300.fluid import rk2_step

    p = mink_params()
    hb = states.random_block(16, states.SEED + 71)
    single = hb.to_device("cuda")
    mesh, blocks = tiled_from_block(single, [[6, 10], [8, 8], [10, 6]])
    ctx_exact.Initialize(p, single)
    init_mesh(ctx_exact, p, mesh, blocks)
    dt = 0.3 * ctx_exact.EstimateTimestepBlock(p, single, False).item()
    rk2_step(ctx_exact, p, single, torch.zeros_like(single["cons"]), dt)
    rk2_mesh(ctx_exact, p, mesh, blocks, [torch.zeros_like(b["cons"]) for b in blocks], dt)
    ctx_exact.check()
    ng = single.ng
    ref = host(single["prim"])
    worst = 0.0
    for (s1, s2, s3), blk in zip(mesh.segments(), blocks):
        i0, j0, k0 = mesh.starts[0][s1], mesh.starts[1][s2], mesh.starts[2][s3]
        n1, n2, n3 = blk.nx
        got = host(blk["prim"])[:abi.PMU, ng:ng + n3, ng:ng + n2, ng:ng + n1]
        want = ref[:abi.PMU, ng + k0:ng + k0 + n3, ng + j0:ng + j0 + n2, ng + i0:ng + i0 + n1]
        scale = np.abs(ref[:abi.PMU]).reshape(abi.PMU, -1).max(axis=1)[:, None, None, None] + 1e-300
        worst = max(worst, float((np.abs(got - want) / scale).max()))
    assert worst < 1e-8, worst


def small_torus(ctx, n=48):
    p = torus.torus_params()
    mesh = torus.torus_mesh(n=n, lo=16, hi=32)
    blocks = mesh.make_blocks("cuda", torus.torus_geometry())
    info = torus.fill_torus(ctx, p, mesh, blocks)
    ctx.check()
    return p, mesh, blocks, info


def test_torus_state(ctx_fast):
    p, mesh, blocks, info = small_torus(ctx_fast)
    gam = p.gm1 + 1.0
    rmax, pmax, bsqmax = 0.0, 0.0, 0.0
    for b in blocks:
        pr = b["prim"]
        ks, js, is_ = b.isl()
        assert bool(torch_isfinite(pr[:, ks, js, is_]))
        rmax = max(rmax, float(pr[abi.PRHO, ks, js, is_].max()))
        pmax = max(pmax, float(pr[abi.PPRS, ks, js, is_].max()))
        bsqmax = max(bsqmax, float(torus._bsq(pr, b.geom.arrays["cent"])[ks, js, is_].max()))
    assert 0.5 < rmax <= 1.0 + 1e-9, rmax  # rho = 1 at the pressure maximum r = 12
    # HARM-style normalisation: max P / max (b^2 / 2) = 100 (con2prim and the
    # floors move it by a tolerance-sized amount)
    assert abs(pmax / (0.5 * bsqmax) / 100.0 - 1.0) < 0.05, pmax / (0.5 * bsqmax)
    assert info["field_factor"] > 0.0
    del gam


def torch_isfinite(t):
    import torch

    return torch.isfinite(t).all()


def test_outflow_and_periodic_ghosts(ctx_fast):
    """Right after an exchange, ghost primitives are exact copies of their
    source cells (normal velocity pointing in through an outflow face set to
    0)."""
    p, mesh, blocks, _ = small_torus(ctx_fast)
    ctx_fast.MeshExchange(p, mesh, blocks)
    ctx_fast.check()
    ng = blocks[0].ng
    b0 = blocks[mesh.block_index(0, 0, 0)]
    pr = host(b0["prim"])
    n1, n2, n3 = b0.nx
    ks, js = slice(ng, ng + n3), slice(ng, ng + n2)
    # X1 inner outflow: every ghost layer copies the first interior cell, v^1 > 0 zeroed
    edge = pr[:, ks, js, ng].copy()
    edge[abi.PVEL] = np.minimum(edge[abi.PVEL], 0.0)
    for g in range(ng):
        assert_bitwise(pr[:abi.PMU + 1, ks, js, g], edge[:abi.PMU + 1], f"X1 ghost {g}")
    # X3 periodic: the lower ghosts of the first k-block are the last k-block's top interior layers
    top = blocks[mesh.block_index(0, 0, mesh.nseg[2] - 1)]
    tp = host(top["prim"])
    m3 = top.nx[2]
    i_s = slice(ng, ng + n1)
    assert_bitwise(pr[:, 0:ng, js, i_s], tp[:, m3:m3 + ng, js, i_s], "X3 periodic ghosts")


def test_torus_batched_equals_per_block(ctx_exact):
    """Exact build: one RK2 step of the torus mesh through the captured
    batched graph equals the block-by-block launches bit for bit."""
    import torch

    p, mesh, blocks, _ = small_torus(ctx_exact)
    copies = []
    for b in blocks:
        c = states.Block(b.nx, b.ng, b.ndim, b.xmin, b.dx, backend="torch", device="cuda",
                         arrays={k: v.clone() for k, v in b.arrays.items()}, geom=b.geom)
        copies.append(c)
    dt = 0.3 * min(ctx_exact.EstimateTimestepBlock(p, b, False).item() for b in blocks)
    rk2_mesh(ctx_exact, p, mesh, blocks, [torch.zeros_like(b["cons"]) for b in blocks], dt, batched=True)
    rk2_mesh(ctx_exact, p, mesh, copies, [torch.zeros_like(b["cons"]) for b in copies], dt, batched=False)
    ctx_exact.check()
    for x, y in zip(blocks, copies):
        for name in ("prim", "cons", "fail"):
            assert_bitwise(x[name], y[name], name)
        ks, js, is_ = x.isl()
        assert bool(torch.isfinite(x["prim"][:, ks, js, is_]).all())
