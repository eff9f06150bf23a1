"""Batched uneven meshblocks (phx_stage_batched): one persistent launch per
phase over all blocks, the stage replayed as a CUDA graph.  The exact build
equals the single-block stage (itself bitwise equal to the oracle) bit for
bit on every block, over several RK2 steps that reuse the captured graph."""
import numpy as np
import pytest

from phoebus_gb300 import abi, states
from phoebus_gb300.abi import PhxError
from tests.util import assert_bitwise, assert_close, host

pytestmark = pytest.mark.gpu
SIZES = [8, 12, 8, 16, 12, 10]


def params(floors=False):
    p = abi.default_params(Gamma=4.0 / 3.0, recon="mp5", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)
    if floors:  # fixup.cpp defaults: ConstantRhoSie floors, c2p fixup, ceilings
        p.enable_floors, p.enable_c2p_fixup, p.enable_ceilings = 1, 1, 1
        p.rho0_floor, p.sie0_floor = 1e-8, 1e-8
    return p


def make_blocks(ctx, p):
    blocks = []
    for b, n in enumerate(SIZES):
        db = states.random_block(n, states.SEED + 3000 + b).to_device("cuda")
        ctx.Initialize(p, db)
        blocks.append(db)
    ctx.check()
    return blocks


def copy_blocks(blocks):
    out = []
    for b in blocks:
        c = states.Block(b.nx, b.ng, b.ndim, b.xmin, b.dx, backend="torch", device="cuda",
                         arrays={k: v.clone() for k, v in b.arrays.items()})
        out.append(c)
    return out


def rk2_single(ctx, p, blocks, seconds, dt):
    from phoebus_gb300.fluid import rk2_step

    for b, s in zip(blocks, seconds):
        rk2_step(ctx, p, b, s, dt)


def rk2_batched(ctx, p, blocks, seconds, dt):
    import torch  # noqa: F401

    bases = [b["cons"] for b in blocks]
    ctx.StageBatched(p, blocks, bases, seconds, 1.0, dt)
    stage2 = []
    for b, s in zip(blocks, seconds):
        c = states.Block(b.nx, b.ng, b.ndim, b.xmin, b.dx, backend="torch", device="cuda",
                         arrays=dict(b.arrays))
        c.arrays["cons"] = s
        stage2.append(c)
    ctx.StageBatched(p, stage2, bases, bases, 0.5, dt)


@pytest.mark.parametrize("exact,floors", [(True, False), (False, False), (True, True)])
def test_batched_equals_single_block(request, exact, floors):
    import torch

    ctx = request.getfixturevalue("ctx_exact" if exact else "ctx_fast")
    p = params(floors)
    a = make_blocks(ctx, p)
    b = copy_blocks(a)
    sa = [torch.zeros_like(x["cons"]) for x in a]
    sb = [torch.zeros_like(x["cons"]) for x in b]
    dt = 0.2 * min(ctx.EstimateTimestepBlock(p, x, False).item() for x in a)
    for step in range(3):  # the second and third steps replay the captured graphs
        rk2_single(ctx, p, a, sa, dt)
        rk2_batched(ctx, p, b, sb, dt)
        ctx.check()
    info = ctx.batch_info()
    assert info["graph_nodes"] >= 9 and info["x1_cells"] > 0 and info["sweep_seg"] > 0
    for x, y in zip(a, b):
        for name in ("prim", "cons", "fail"):
            if exact:
                assert_bitwise(y[name], x[name], name)
            else:
                g, r = host(y[name]), host(x[name])
                g, r = (g, r) if g.ndim == 4 else (g[None], r[None])
                for v in range(g.shape[0]):
                    # zones whose inversion failed (NaN) must fail in both
                    assert np.array_equal(np.isnan(g[v]), np.isnan(r[v])), name
                    ok = ~np.isnan(r[v])
                    if ok.any():
                        assert_close(g[v][ok], r[v][ok], 1e-12, f"{name}[{v}]")


def test_batched_learned_equals_single_block(ctx_exact):
    """The learned start in the batched stage (bracket launch + root-find
    launch over all blocks) equals the single-block learned stage bit for
    bit (exact build), with the same learned-accepted count."""
    import torch

    from phoebus_gb300 import learned

    theta = learned.init_weights(5)
    theta[-2:] = [-0.3, -1.0]  # brackets [0.25 m, m e^1.1]: a mix of accepted and rejected starts
    ctx_exact.mlp_set_weights(theta)
    p = params()
    a = make_blocks(ctx_exact, p)
    for x in a:  # cold zones: no previous mu, so the first inversions use the learned start
        x["prim"][abi.PMU] = 0.0
    b = copy_blocks(a)
    sa = [torch.zeros_like(x["cons"]) for x in a]
    sb = [torch.zeros_like(x["cons"]) for x in b]
    dt = 0.2 * min(ctx_exact.EstimateTimestepBlock(p, x, False).item() for x in a)
    from phoebus_gb300.fluid import rk2_step

    acc = []
    for run in ("single", "batched"):
        ctx_exact.c2p_stats(reset=True)
        for step in range(2):
            if run == "single":
                for x, s in zip(a, sa):
                    rk2_step(ctx_exact, p, x, s, dt, learned=True)
            else:
                bases = [x["cons"] for x in b]
                ctx_exact.StageBatched(p, b, bases, sb, 1.0, dt, learned=True)
                st2 = []
                for x, s in zip(b, sb):
                    c = states.Block(x.nx, x.ng, x.ndim, x.xmin, x.dx, backend="torch", device="cuda",
                                     arrays=dict(x.arrays))
                    c.arrays["cons"] = s
                    st2.append(c)
                ctx_exact.StageBatched(p, st2, bases, bases, 0.5, dt, learned=True)
        ctx_exact.check()
        acc.append(ctx_exact.c2p_stats(reset=True))
    for x, y in zip(a, b):
        for name in ("prim", "cons", "fail"):
            assert_bitwise(y[name], x[name], name)
    assert acc[0]["learned_accepted"] == acc[1]["learned_accepted"] > 0
    assert acc[0]["iterations"] == acc[1]["iterations"]


def test_batched_refuses_mixed_blocks(ctx_fast):
    import torch

    p = params()
    blocks = make_blocks(ctx_fast, p)[:1]
    mixed = blocks + [states.Block((8, 8, 1), 4, 2, (0, 0, 0), (0.1, 0.1, 1.0), backend="torch",
                                   device="cuda").alloc()]
    with pytest.raises(PhxError) as e:
        ctx_fast.StageBatched(p, mixed, [b["cons"] for b in mixed], [torch.zeros_like(b["cons"]) for b in mixed],
                              1.0, 1e-3)
    assert e.value.status == 1 and "share ndim" in str(e.value)
