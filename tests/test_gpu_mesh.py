"""Tiled meshes (phx_stage_mesh, phx_mesh_exchange, phx_fix_fluxes): the
boundary exchange with physical boundaries and FixFluxes against the
oracle's restatement, agreement with a single periodic block, batched
against block-by-block launches, and the magnetised torus state on an FMKS
mesh."""
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


def rad_mesh_stage(rx, rp, p, mesh, blocks, bases, outs, beta, dt):
    """One moment stage with the fluid static over a tiled mesh, from the
    per-block tasks in PhoebusDriver::RungeKuttaStage's order: opacities,
    fluxes, update, FillDerived (MomentCon2Prim), the radiation c2p fixup,
    floors, MomentFluidSource, floors; the exchange; FillDerived, fixup and
    floors again."""
    for b, base, out in zip(blocks, bases, outs):
        rx.MomentCalculateOpacities(rp, p, b)
        rx.CalculateFluxes(rp, p, b)
        rx.Update(rp, b, base, out, beta, dt)
        b.arrays["rcons"] = out
        rx.MomentCon2Prim(rp, p, b)
        rx.RadConservedToPrimitiveFixup(rp, p, b)
        rx.ApplyFloors(rp, p, b)
        rx.MomentFluidSource(rp, p, b, beta * dt)
        rx.ApplyFloors(rp, p, b)
    rx.MeshExchange(rp, p, mesh, blocks)
    for b in blocks:
        rx.MomentCon2Prim(rp, p, b)
        rx.RadConservedToPrimitiveFixup(rp, p, b)
        rx.ApplyFloors(rp, p, b)


@pytest.mark.parametrize("method", ["moment_m1", "moment_eddington"])
def test_rad_periodic_mesh_matches_single_block(ctx_exact, method):
    """Radiation on a tiled mesh: a periodic 12 x 10 x 8 moment state over a
    static fluid, split into 2 x 2 x 2 blocks (uneven in X1, X2) and stepped
    with the per-block moment tasks and phx_rad_mesh_exchange, evolves bit for bit like
    the single periodic block's phx_rad_stage over two RK2 steps."""
    import torch

    from phoebus_gb300.radiation import RadiationContext, alloc_rad
    from tests.util import random_rad_block

    rx = RadiationContext(ctx_exact)
    rp = abi.default_rad_params(method=method, recon="linear", cfl=0.5, kappa_s=30.0, kappa_a=2.0, jbb_coeff=0.5)
    p = abi.default_params(Cv=1.0)
    hb = random_rad_block((12, 10, 8), 3, seed=29, vmax=0.3)
    ng, n = hb.ng, hb.nx
    wrap = [((np.arange(n[d] + 2 * ng) - ng) % n[d]) + ng for d in range(3)]
    hb["prim"][...] = hb["prim"][:, wrap[2]][:, :, wrap[1]][:, :, :, wrap[0]]  # a periodic fluid
    single = hb.to_device()
    rx.MomentPrim2Con(rp, p, single)
    rx.Initialize(rp, p, single)
    mesh = TiledMesh(n, [[5, 7], [4, 6], [4, 4]], single.xmin,
                     tuple(single.xmin[d] + n[d] * single.dx[d] for d in range(3)), (abi.BC_PERIODIC,) * 3,
                     (abi.BC_PERIODIC,) * 3, ng=ng, bc_vars=abi.BC_VARS_PRIMITIVE)
    blocks = mesh.make_blocks("cuda")
    for (s1, s2, s3), blk in zip(mesh.segments(), blocks):
        alloc_rad(blk)
        org = (mesh.starts[0][s1], mesh.starts[1][s2], mesh.starts[2][s3])
        idx = [torch.as_tensor(((org[d] + np.arange(blk.nx[d] + 2 * ng) - ng) % n[d]) + ng, device="cuda")
               for d in range(3)]
        for name, a in single.arrays.items():
            if name in blk.arrays and a.dim() == 4 and tuple(a.shape[1:]) == tuple(single.shape):
                blk[name].copy_(a[:, idx[2]][:, :, idx[1]][:, :, :, idx[0]])
    buf = torch.zeros_like(single["rcons"])
    bufs = [torch.zeros_like(b["rcons"]) for b in blocks]
    for step in range(2):
        dt = rx.EstimateTimestepBlock(rp, p, single)
        rx.rk2_step(rp, p, single, buf, dt)
        bases = [b["rcons"] for b in blocks]
        rad_mesh_stage(rx, rp, p, mesh, blocks, bases, bufs, 1.0, dt)
        rad_mesh_stage(rx, rp, p, mesh, blocks, bases, bases, 0.5, dt)
        for b, base in zip(blocks, bases):
            b.arrays["rcons"] = base
    rx.check()
    for (s1, s2, s3), blk in zip(mesh.segments(), blocks):
        i0, j0, k0 = mesh.starts[0][s1], mesh.starts[1][s2], mesh.starts[2][s3]
        n1, n2, n3 = blk.nx
        for name, nv in (("rcons", abi.RNCONS), ("rprim", abi.RFAIL + 1)):
            got = host(blk[name])[:nv, ng:ng + n3, ng:ng + n2, ng:ng + n1]
            want = host(single[name])[:nv, ng + k0:ng + k0 + n3, ng + j0:ng + j0 + n2, ng + i0:ng + i0 + n1]
            assert_bitwise(got, want, f"block {(s1, s2, s3)} {name}")


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


def random_interior(ctx, p, mesh, blocks, seed):
    """Random primitives in every block's interior (velocities and fields of
    both signs, so mirrors and the inflow check have work), conserved
    variables by prim2con."""
    import torch

    rng = np.random.default_rng(seed)
    gam = p.gm1 + 1.0
    for b in blocks:
        ks, js, is_ = b.isl()
        shp = b["prim"][0][ks, js, is_].shape
        rho = 10.0 ** rng.uniform(-3.0, 0.0, shp)
        u = rho * 10.0 ** rng.uniform(-2.0, 0.0, shp)
        pr = np.zeros((abi.NPRIM,) + shp)
        pr[abi.PRHO], pr[abi.PENG], pr[abi.PPRS] = rho, u, p.gm1 * u
        pr[abi.PVEL:abi.PVEL + 3] = rng.uniform(-0.5, 0.5, (3,) + shp)
        pr[abi.PB:abi.PB + 3] = rng.uniform(-0.2, 0.2, (3,) + shp)
        if b.geom is not None:  # components of proper size: divide by sqrt(gamma_dd)
            cent = host(b.geom.arrays["cent"])[:, js, is_]
            for d in range(3):
                scale = 1.0 / np.sqrt(cent[abi.G_GCOV + (d + 1) * (d + 2) // 2 + d + 1])
                pr[abi.PVEL + d] *= scale
                pr[abi.PB + d] *= scale
        pr[abi.PGM1], pr[abi.PTMP], pr[abi.PMU] = gam, u / rho, rng.uniform(0.1, 0.9, shp)
        b["prim"][:, ks, js, is_] = torch.from_numpy(pr).to(b["prim"].device)
        ctx.PrimitiveToConserved(p, b, *b.interior())
    ctx.check()


# (bc_lo, bc_hi) per axis; the first is the torus deck's
MESH_BCS = {
    "deck": ((abi.BC_OUTFLOW, abi.BC_OUTFLOW, abi.BC_PERIODIC), (abi.BC_OUTFLOW, abi.BC_OUTFLOW, abi.BC_PERIODIC)),
    "reflect_polar": ((abi.BC_REFLECT, abi.BC_POLAR, abi.BC_PERIODIC), (abi.BC_OUTFLOW, abi.BC_POLAR, abi.BC_PERIODIC)),
    "reflect_x2_x3": ((abi.BC_OUTFLOW, abi.BC_REFLECT, abi.BC_REFLECT), (abi.BC_REFLECT, abi.BC_OUTFLOW, abi.BC_OUTFLOW)),
}


def small_fmks_mesh(bcs, n=26, lo=6, hi=12, bc_vars=abi.BC_VARS_PRIMITIVE, ndim=3):
    from phoebus_gb300.mesh import TiledMesh, split_axis

    segs = [split_axis(n, lo, hi, torus.TORUS_SEED, 40 + d) if d < ndim else [1] for d in range(3)]
    return TiledMesh(tuple(n if d < ndim else 1 for d in range(3)), segs, (math.log(1.2), 0.0, 0.0),
                     (math.log(250.0), 1.0, 2.0 * math.pi), *bcs, bc_vars=bc_vars, ndim=ndim)


@pytest.mark.parametrize("ndim", [3, 2])
@pytest.mark.parametrize("bc_vars", [abi.BC_VARS_PRIMITIVE, abi.BC_VARS_CONSERVED])
@pytest.mark.parametrize("name", list(MESH_BCS))
@pytest.mark.parametrize("geometry", ["fmks", "minkowski"])
def test_mesh_exchange_matches_oracle(ctx_exact, name, geometry, bc_vars, ndim):
    """Exact build: the exchange (neighbour copies, physical boundaries; with
    bc_vars = primitive the outer-X1 inflow check and prim2con in the boundary
    slabs, with bc_vars = conserved the DetGamma-scaled copies and, on FMKS,
    con2prim + the inflow check + prim2con in the outer-X1 slab) equals the
    oracle's literal face-by-face restatement bit for bit -- prims, cons, fail
    flags and cell signal speeds in every ghost zone."""
    from oracle.mesh_oracle import mesh_exchange
    from oracle.oracle import Oracle

    bcs = MESH_BCS[name]
    if bc_vars == abi.BC_VARS_CONSERVED and abi.BC_POLAR in bcs[0] + bcs[1]:
        pytest.skip("polar boundaries need bc_vars = primitive")
    p = torus.torus_params()
    mesh = small_fmks_mesh(bcs, bc_vars=bc_vars, ndim=ndim)
    geom = torus.torus_geometry() if geometry == "fmks" else None
    blocks = mesh.make_blocks("cuda", geom)
    for b in blocks:
        if geom is not None:
            ctx_exact.GeometryFillFMKS(b)
    random_interior(ctx_exact, p, mesh, blocks, seed=100 + 4 * list(MESH_BCS).index(name) + 2 * bc_vars +
                    (geom is not None))
    before = [b.to_host() for b in blocks]
    ctx_exact.MeshExchange(p, mesh, blocks)
    ctx_exact.check()
    mesh_exchange(Oracle(), p, mesh, before)
    for n, (g, r) in enumerate(zip(blocks, before)):
        assert not np.isnan(r["cons"]).any(), f"block {n}: a ghost no rule filled"
        assert_bitwise(g["prim"], r["prim"], f"block {n} prim")
        assert_bitwise(g["cons"], r["cons"], f"block {n} cons")
        assert_bitwise(g["cell_sig"], r["cell_sig"], f"block {n} cell_sig")
        assert_bitwise(g["fail"], r["fail"], f"block {n} fail")


def random_rad_interior(blocks, seed):
    """Radiation fields on every block (ghosts NaN, so a ghost no rule fills
    shows up): random J, H_i / J of both signs with |H| / J up to 1.2 (some
    zones above the inflow check's 0.99 cap), xi, phi, c2pfail, and random
    conserved moments."""
    import torch

    from phoebus_gb300.radiation import alloc_rad

    rng = np.random.default_rng(seed)
    for b in blocks:
        alloc_rad(b, fill=float("nan"))
        ks, js, is_ = b.isl()
        shp = b["rprim"][0][ks, js, is_].shape
        R = np.zeros((abi.RNPRIM,) + shp)
        R[abi.RJ] = 10.0 ** rng.uniform(-3.0, 0.0, shp)
        h = rng.uniform(-1.0, 1.0, (3,) + shp)
        h *= 1.2 * rng.uniform(0.0, 1.0, shp) ** 0.25 / np.maximum(np.sqrt((h * h).sum(0)), 1e-12)
        if b.geom is not None:  # covariant components of proper size: times sqrt(gamma_dd)
            cent = host(b.geom.arrays["cent"])[:, js, is_]
            for d in range(3):
                h[d] *= np.sqrt(cent[abi.G_GCOV + (d + 1) * (d + 2) // 2 + d + 1])
        R[abi.RH:abi.RH + 3] = h
        R[abi.RXI] = rng.uniform(0.0, 1.0, shp)
        R[abi.RPHI] = rng.uniform(0.0, 2.0 * np.pi, shp)
        R[abi.RFAIL] = rng.integers(0, 2, shp).astype(np.float64)
        U = rng.uniform(-1.0, 1.0, (abi.RNCONS,) + shp)
        U[abi.RE] = 10.0 ** rng.uniform(-3.0, 0.0, shp)
        b["rprim"][:, ks, js, is_] = torch.from_numpy(R).to(b["rprim"].device)
        b["rcons"][:, ks, js, is_] = torch.from_numpy(U).to(b["rcons"].device)


def rad_exchange_case(ctx, name, geometry, bc_vars, ndim, method, seed):
    """A small tiled mesh with fluid and radiation interiors, the fluid
    exchanged; returns (p, rp, mesh, blocks, host copies before the radiation
    exchange)."""
    bcs = MESH_BCS[name]
    if bc_vars == abi.BC_VARS_CONSERVED and abi.BC_POLAR in bcs[0] + bcs[1]:
        pytest.skip("polar boundaries need bc_vars = primitive")
    p = torus.torus_params()
    rp = abi.default_rad_params(method=method)
    mesh = small_fmks_mesh(bcs, bc_vars=bc_vars, ndim=ndim)
    geom = torus.torus_geometry() if geometry == "fmks" else None
    blocks = mesh.make_blocks("cuda", geom)
    for b in blocks:
        if geom is not None:
            ctx.GeometryFillFMKS(b)
    random_interior(ctx, p, mesh, blocks, seed=seed)
    ctx.MeshExchange(p, mesh, blocks)
    random_rad_interior(blocks, seed + 1)
    return p, rp, mesh, blocks, [b.to_host() for b in blocks]


@pytest.mark.parametrize("method", ["moment_m1", "moment_eddington"])
@pytest.mark.parametrize("ndim", [3, 2])
@pytest.mark.parametrize("bc_vars", [abi.BC_VARS_PRIMITIVE, abi.BC_VARS_CONSERVED])
@pytest.mark.parametrize("name", list(MESH_BCS))
@pytest.mark.parametrize("geometry", ["fmks", "minkowski"])
def test_rad_mesh_exchange_matches_oracle(ctx_exact, name, geometry, bc_vars, ndim, method):
    """Exact build: the radiation fields' exchange (neighbour copies; the
    boundary functions on every FillGhost radiation field, DetGamma-scaled
    under bc_vars = conserved, F_d and H_d flipped across reflect faces; on
    FMKS the outer-X1 cut of incoming radiation flux; with bc_vars = primitive
    MomentPrim2Con in the physical slabs) equals the oracle's face-by-face
    restatement bit for bit in every ghost zone."""
    from oracle.mesh_oracle import RFILL, rad_mesh_exchange
    from oracle.oracle import RadOracle
    from phoebus_gb300.radiation import RadiationContext

    seed = 300 + 8 * list(MESH_BCS).index(name) + 4 * bc_vars + 2 * (geometry == "fmks") + (ndim == 2)
    p, rp, mesh, blocks, before = rad_exchange_case(ctx_exact, name, geometry, bc_vars, ndim, method, seed)
    rx = RadiationContext(ctx_exact)
    rx.MeshExchange(rp, p, mesh, blocks)
    rx.check()
    rad_mesh_exchange(RadOracle(), rp, p, mesh, before)
    for n, (g, r) in enumerate(zip(blocks, before)):
        assert not np.isnan(r["rcons"]).any(), f"block {n}: a ghost no rule filled"
        assert not np.isnan(r["rprim"][:RFILL]).any(), f"block {n}: a ghost no rule filled"
        assert_bitwise(g["rcons"], r["rcons"], f"block {n} rcons")
        assert_bitwise(g["rprim"][:RFILL], r["rprim"][:RFILL], f"block {n} rprim")


def test_rad_mesh_exchange_inflow_cut(ctx_exact):
    """The outer-X1 cut acts: on the torus deck's FMKS mesh, outer-X1 ghosts
    whose mapped H^1 points into the domain leave the exchange with H^1 = 0
    (within rounding of gamma^1j H_j) and |H| <= 0.99; the others keep the
    copied values."""
    from phoebus_gb300.radiation import RadiationContext

    p, rp, mesh, blocks, _ = rad_exchange_case(ctx_exact, "deck", "fmks", abi.BC_VARS_PRIMITIVE, 3, "moment_m1", 77)
    rx = RadiationContext(ctx_exact)
    rx.MeshExchange(rp, p, mesh, blocks)
    rx.check()
    cut = kept = 0
    for (s1, s2, s3), b in zip(mesh.segments(), blocks):
        if s1 != mesh.nseg[0] - 1:
            continue
        ng, n1 = b.ng, b.nx[0]
        ks, js, _ = b.isl()
        R = host(b["rprim"])
        cent = host(b.geom.arrays["cent"])
        for i in range(ng + n1, 2 * ng + n1):
            H = R[abi.RH:abi.RH + 3, ks, js, i]
            src = R[abi.RH:abi.RH + 3, ks, js, ng + n1 - 1]
            t = cent[:, js, i][:, None, :]

            def flat(a, c):
                return max(a, c) * (max(a, c) + 1) // 2 + min(a, c)

            gcon = [[t[abi.G_GAMCON + flat(a, c)] for c in range(3)] for a in range(3)]
            gcov = [[t[abi.G_GCOV + flat(a + 1, c + 1)] for c in range(3)] for a in range(3)]
            hsrc1 = sum(gcon[0][c] * src[c] for c in range(3))
            into = hsrc1 < 0
            h1 = sum(gcon[0][c] * H[c] for c in range(3))
            hcon = [sum(gcon[a][c] * H[c] for c in range(3)) for a in range(3)]
            xi = np.sqrt(sum(gcov[a][c] * hcon[a] * hcon[c] for a in range(3) for c in range(3)))
            assert np.all(np.abs(h1[into]) <= 1e-12 * (1.0 + np.abs(H).max()))
            assert np.all(xi[into] <= 0.99 * (1 + 1e-12))
            assert_bitwise(H[:, ~into], src[:, ~into], "outer-X1 ghosts with outgoing H")
            cut += int(into.sum())
            kept += int((~into).sum())
    assert cut > 0 and kept > 0


@pytest.mark.parametrize("fixup", [1, 0])
@pytest.mark.parametrize("ndim", [3, 2])
@pytest.mark.parametrize("name", list(MESH_BCS))
def test_rad_fix_fluxes_matches_oracle(ctx_fast, name, ndim, fixup):
    """FixFluxes' radiation part equals the oracle's restatement bit for bit
    on random radiation fluxes (every face of every block compared; a no-op
    with enable_flux_fixup off)."""
    import torch

    from oracle.mesh_oracle import rad_fix_fluxes
    from phoebus_gb300.radiation import RadiationContext, alloc_rad

    p = torus.torus_params()
    p.enable_flux_fixup = fixup
    rp = abi.default_rad_params()
    mesh = small_fmks_mesh(MESH_BCS[name], ndim=ndim)
    blocks = mesh.make_blocks("cuda", None)
    rng = np.random.default_rng(500 + ndim + 4 * fixup + 8 * list(MESH_BCS).index(name))
    for b in blocks:
        alloc_rad(b)
        b["rflux"].copy_(torch.from_numpy(rng.standard_normal(tuple(b["rflux"].shape))))
    before = [b.to_host() for b in blocks]
    rx = RadiationContext(ctx_fast)
    rx.FixFluxes(rp, p, mesh, blocks)
    rx.check()
    rad_fix_fluxes(p, mesh, before)
    changed = 0
    for n, (g, r) in enumerate(zip(blocks, before)):
        assert_bitwise(g["rflux"], r["rflux"], f"block {n} rflux")
        changed += int((host(g["rflux"]) == 0.0).sum())
    assert (changed > 0) == (fixup == 1 and name != "deck")


def test_conserved_exchange_inflow_fixes_ghosts(ctx_exact):
    """bc_vars = conserved on an FMKS mesh with X1 outflow: interior zones
    next to the outer X1 face given an inward velocity (u^1 < 0) leave
    u^1 >= 0 in the outer-X1 ghosts once the slab has gone through
    con2prim, the inflow check and prim2con; without the check the ghosts
    keep the copied inflow.  The cons of the fixed ghosts are prim2con of
    their prims (a con2prim of the ghost gives the prims back)."""
    import torch

    bcs = MESH_BCS["deck"]
    p = torus.torus_params()
    mesh = small_fmks_mesh(bcs, bc_vars=abi.BC_VARS_CONSERVED, ndim=2)
    blocks = mesh.make_blocks("cuda", torus.torus_geometry())
    for b in blocks:
        ctx_exact.GeometryFillFMKS(b)
    random_interior(ctx_exact, p, mesh, blocks, seed=77)
    outer = [b for b, seg in zip(blocks, mesh.segments()) if seg[0] == mesh.nseg[0] - 1]
    for b in outer:  # inward radial velocity in the last interior column
        ks, js, is_ = b.isl()
        last = is_.stop - 1
        g11 = b.geom.arrays["cent"][abi.G_GCOV + 2][js, last]
        v1 = b["prim"][abi.PVEL, ks, js, last]
        b["prim"][abi.PVEL, ks, js, last] = -v1.abs() - 0.1 / torch.sqrt(g11)
        ctx_exact.PrimitiveToConserved(p, b, *b.interior())
    saved = [{k: v.clone() for k, v in b.arrays.items()} for b in blocks]

    def ucon1(b):
        cent = b.geom.arrays["cent"]
        pr = b["prim"]
        g = lambda m, n: cent[abi.G_GCOV + (max(m, n) * (max(m, n) + 1)) // 2 + min(m, n)][None]  # noqa: E731
        W = torch.sqrt(1 + sum(g(m + 1, n + 1) * pr[abi.PVEL + m] * pr[abi.PVEL + n]
                               for m in range(3) for n in range(3)))
        return pr[abi.PVEL] - W * cent[abi.G_BETA][None] / cent[abi.G_ALPHA][None]

    def ghosts(b, a):  # the outer-X1 ghosts beside the interior rows
        return a[..., b.ng:b.ng + b.nx[1], b.n1t - b.ng:]

    p.enable_ox1_fmks_inflow_check = 0
    ctx_exact.MeshExchange(p, mesh, blocks)
    for b in outer:
        ctx_exact.ConservedToPrimitive(p, b)
    ctx_exact.check()
    assert any(bool((ghosts(b, ucon1(b)) < 0).any()) for b in outer), "no inflow to fix"
    for b, a in zip(blocks, saved):
        for k, v in a.items():
            b.arrays[k].copy_(v)
    p.enable_ox1_fmks_inflow_check = 1
    ctx_exact.MeshExchange(p, mesh, blocks)
    ctx_exact.check()
    for b in outer:
        u1 = ghosts(b, ucon1(b))
        scale = ghosts(b, (b.geom.arrays["cent"][abi.G_BETA] / b.geom.arrays["cent"][abi.G_ALPHA])[None]).abs()
        assert bool((u1 >= -1e-12 * scale).all()), float(u1.min())
        cons = b["cons"].clone()
        ctx_exact.PrimitiveToConserved(p, b, *b.entire())
        assert_bitwise(ghosts(b, b["cons"]), ghosts(b, cons), "ghost cons = prim2con(prims)")


@pytest.mark.parametrize("name", list(MESH_BCS))
def test_fix_fluxes_matches_oracle(ctx_fast, name):
    """FixFluxes on random fluxes of both signs, through the mesh entry point
    and the per-block task, against the oracle bit for bit; without
    enable_flux_fixup nothing changes."""
    import torch

    from oracle.mesh_oracle import block_faces, fix_fluxes, fix_fluxes_block

    p = torus.torus_params()
    mesh = small_fmks_mesh(MESH_BCS[name])
    blocks = mesh.make_blocks("cuda", None)
    g = torch.Generator(device="cuda").manual_seed(7)
    for b in blocks:
        b["flux"].copy_(torch.randn(b["flux"].shape, generator=g, device="cuda", dtype=torch.float64))
    start = [b["flux"].clone() for b in blocks]
    p.enable_flux_fixup = 0
    ctx_fast.FixFluxes(p, mesh, blocks)
    ctx_fast.check()
    for b, f0 in zip(blocks, start):
        assert_bitwise(b["flux"], f0, "flux fixup off")
    p.enable_flux_fixup = 1
    ref = [b.to_host() for b in blocks]
    fix_fluxes(p, mesh, ref)
    ctx_fast.FixFluxes(p, mesh, blocks)
    ctx_fast.check()
    for n, (b, r) in enumerate(zip(blocks, ref)):
        assert_bitwise(b["flux"], r["flux"], f"block {n} flux (mesh)")
    # per-block task on the untouched fluxes
    for b, f0, seg in zip(blocks, start, mesh.segments()):
        b["flux"].copy_(f0)
        lo, hi = block_faces(mesh, seg, b)
        ctx_fast.FixFluxesBlock(p, b, lo, hi)
        r = b.to_host()
        r["flux"][...] = host(f0)
        fix_fluxes_block(p, r, lo, hi)
        ctx_fast.check()
        assert_bitwise(b["flux"], r["flux"], "flux (block task)")


def test_mesh_rejects_bad_boundaries(ctx_fast):
    p = torus.torus_params()
    deck = MESH_BCS["deck"]
    bad = [(((abi.BC_POLAR, abi.BC_OUTFLOW, abi.BC_PERIODIC), deck[1]), abi.BC_VARS_PRIMITIVE, "X2 faces"),
           ((deck[0], (abi.BC_OUTFLOW, abi.BC_OUTFLOW, abi.BC_OUTFLOW)), abi.BC_VARS_PRIMITIVE, "periodic"),
           (((abi.BC_OUTFLOW, 7, abi.BC_PERIODIC), deck[1]), abi.BC_VARS_PRIMITIVE, "unknown boundary"),
           (MESH_BCS["reflect_polar"], abi.BC_VARS_CONSERVED, "Polar X2"),
           (deck, 5, "bc_vars")]
    for bcs, bc_vars, msg in bad:
        mesh = small_fmks_mesh(bcs, bc_vars=bc_vars)
        blocks = mesh.make_blocks("cuda", None)
        with pytest.raises(RuntimeError, match=msg):
            ctx_fast.MeshExchange(p, mesh, blocks)


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


@pytest.mark.parametrize("floors,bc_vars", [("ConstantRhoSie", abi.BC_VARS_PRIMITIVE),
                                            ("ExpX1RhoSie", abi.BC_VARS_PRIMITIVE),
                                            ("ExpX1RhoSie", abi.BC_VARS_CONSERVED)])
def test_torus_rk2_matches_oracle(oracle, ctx_exact, floors, bc_vars):
    """Config 5 end to end on a small mesh: one batched RK2 step of the
    magnetised torus (FMKS, WENO5-Z + HLL, gr_outflow with bc_vars =
    primitive as in the deck, or conserved with the slab's con2prim before
    the inflow check, the outer-X1 inflow check, FixFluxes, floors,
    ceilings, c2p fixup) against the oracle's mesh stage from the same
    tables and state.  Bit for bit with both floor models: the ExpX1RhoSie
    floors' exp is the library's written-out one
    (phoebus_gb300/csrc/phx_math.h), which the oracle evaluates too."""
    from oracle.mesh_oracle import mesh_rk2_step
    from phoebus_gb300.fluid import MeshRK2
    p = torus.torus_params()
    if floors == "ConstantRhoSie":
        p.floor_type = abi.FLOOR["ConstantRhoSie"]
        p.rho0_floor, p.sie0_floor = 1e-6, 1e-3
    mesh = torus.torus_mesh(n=48, lo=16, hi=32)
    mesh.bc_vars = bc_vars
    blocks = mesh.make_blocks("cuda", torus.torus_geometry())
    torus.fill_torus(ctx_exact, p, mesh, blocks)
    ctx_exact.check()
    hosts = [b.to_host() for b in blocks]
    rk = MeshRK2(ctx_exact, p, mesh, blocks)
    dt = 0.3 * rk.estimate_dt(False)
    rk.step(dt)
    ctx_exact.check()
    mesh_rk2_step(oracle, p, mesh, hosts, [np.zeros_like(h["cons"]) for h in hosts], dt)
    for n, (g, h) in enumerate(zip(blocks, hosts)):
        for name in ("prim", "cons", "fail"):
            assert_bitwise(g[name], h[name], f"block {n} {name}")
