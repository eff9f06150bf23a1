"""The mesh oracle's literal face-by-face boundary application (neighbour
exchange, then the physical faces X1, X2, X3 in turn, each over the entire
range of the other axes) against the closed form the CUDA exchange
implements: every axis maps the ghost's global cell on its own (periodic
wrap, clamp, mirror), the signs of the mirrored vector components multiply,
and with bc_vars = conserved the DetGamma ratios of the cells each face sets
multiply in face order.  Host only."""
import numpy as np
import pytest

from oracle import mesh_oracle as mo
from phoebus_gb300 import abi
from phoebus_gb300.block import Block
from phoebus_gb300.mesh import TiledMesh

CASES = {
    "deck": ((abi.BC_OUTFLOW, abi.BC_OUTFLOW, abi.BC_PERIODIC), (abi.BC_OUTFLOW, abi.BC_OUTFLOW, abi.BC_PERIODIC)),
    "reflect_polar": ((abi.BC_REFLECT, abi.BC_POLAR, abi.BC_PERIODIC), (abi.BC_OUTFLOW, abi.BC_POLAR, abi.BC_PERIODIC)),
    "all_mirror": ((abi.BC_REFLECT, abi.BC_REFLECT, abi.BC_REFLECT), (abi.BC_REFLECT, abi.BC_POLAR, abi.BC_OUTFLOW)),
}


def host_mesh(bcs, seed, bc_vars, ndim=3):
    n = [(14, 12, 10), (14, 12, 1), (14, 1, 1)][3 - ndim]
    segs = [[[6, 8], [4, 8], [5, 5]][d] if d < ndim else [1] for d in range(3)]
    mesh = TiledMesh(n, segs, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), *bcs, bc_vars=bc_vars, ndim=ndim)
    rng = np.random.default_rng(seed)
    blocks = mesh.make_blocks(geometry=abi.default_geometry(abi.GEOM_FMKS), backend="numpy")
    for b in blocks:
        b["prim"][...] = rng.standard_normal(b["prim"].shape)
        b["cons"][...] = rng.standard_normal(b["cons"].shape)
        b.geom.arrays["cent"][abi.G_DETGAM] = rng.uniform(0.5, 2.0, b.geom.arrays["cent"][0].shape)
    return mesh, blocks


def closed_form(mesh, blocks, mhd=True):
    """Per ghost: the source cell of all axes' maps, signs multiplied, the
    DetGamma ratios (bc_vars = conserved) multiplied in face order."""
    out = [(b["prim"].copy(), b["cons"].copy()) for b in blocks]
    conserved = mesh.bc_vars == abi.BC_VARS_CONSERVED
    for (P, U), b, seg in zip(out, blocks, mesh.segments()):
        org = [int(mesh.starts[d][seg[d]]) for d in range(3)]
        detg = b.geom.arrays["cent"][abi.G_DETGAM]
        for k in range(b.n3t):
            for j in range(b.n2t):
                for i in range(b.n1t):
                    loc = [i, j, k]
                    mloc = list(loc)
                    g, ghost, phys = [], False, [False] * 3
                    sp, su = [np.ones(abi.NPRIM) for _ in range(3)], [np.ones(abi.NCONS) for _ in range(3)]
                    for d in range(3):
                        if d >= b.ndim:
                            g.append(0)
                            continue
                        if not b.ng <= loc[d] < b.ng + b.nx[d]:
                            ghost = True
                        gg = org[d] + loc[d] - b.ng
                        if gg < 0 or gg >= mesh.n[d]:
                            lo = gg < 0
                            bc = mesh.bc_lo[d] if lo else mesh.bc_hi[d]
                            ref = b.ng if lo else b.ng + b.nx[d] - 1
                            if bc == abi.BC_PERIODIC:
                                gg += mesh.n[d] if lo else -mesh.n[d]
                            elif bc == abi.BC_OUTFLOW:
                                phys[d] = True
                                gg = 0 if lo else mesh.n[d] - 1
                                mloc[d] = ref
                            else:
                                phys[d] = True
                                gg = -1 - gg if lo else 2 * mesh.n[d] - 1 - gg
                                mloc[d] = 2 * ref + (-1 if lo else 1) - loc[d]
                                c = 1 if bc == abi.BC_POLAR else d
                                sp[d][abi.PVEL + c] = sp[d][abi.PB + c] = -1.0
                                if bc == abi.BC_REFLECT:
                                    su[d][mo.CMOM + d] = su[d][mo.CB + d] = -1.0
                        g.append(gg)
                    if not ghost:
                        continue
                    o, (li, lj, lk) = mo._owner_cell(mesh, g)
                    src = blocks[o]
                    sl = tuple(x + b.ng if d < b.ndim else 0 for d, x in enumerate((li, lj, lk)))
                    q_p = src["prim"][:, sl[2], sl[1], sl[0]].copy()
                    q_u = src["cons"][:, sl[2], sl[1], sl[0]].copy()
                    for d in range(3):
                        if not phys[d]:
                            continue
                        cc = [loc[e] if e <= d else mloc[e] for e in range(3)]
                        rr = [mloc[e] if e == d else cc[e] for e in range(3)]
                        gr = mo._ratio(detg[cc[1], cc[0]], detg[rr[1], rr[0]]) if conserved else 1.0
                        q_u = su[d] * gr * q_u if conserved else su[d] * q_u
                        q_p = sp[d] * q_p
                    if not conserved:
                        P[:, k, j, i] = q_p
                    U[:, k, j, i] = q_u
    return out


@pytest.mark.parametrize("ndim", [3, 2, 1])
@pytest.mark.parametrize("bc_vars", [abi.BC_VARS_PRIMITIVE, abi.BC_VARS_CONSERVED])
@pytest.mark.parametrize("name", list(CASES))
def test_face_by_face_equals_composed_maps(name, bc_vars, ndim):
    bcs = CASES[name]
    if bc_vars == abi.BC_VARS_CONSERVED and abi.BC_POLAR in bcs[0] + bcs[1]:
        pytest.skip("polar boundaries need bc_vars = primitive")
    mesh, blocks = host_mesh(bcs, 11 + list(CASES).index(name), bc_vars, ndim)
    want = closed_form(mesh, blocks)
    mo._exchange_neighbours(mesh, blocks, True)
    for b, seg in zip(blocks, mesh.segments()):
        for d, outer, bc in mo._physical_faces(mesh, b, seg):
            mo._apply_face(b, d, outer, bc, True, bc_vars)
    for n, (b, (P, U)) in enumerate(zip(blocks, want)):
        assert not np.isnan(b["cons"]).any(), f"block {n}: a ghost no rule filled"
        np.testing.assert_array_equal(b["prim"], P, err_msg=f"block {n} prim")
        np.testing.assert_array_equal(b["cons"], U, err_msg=f"block {n} cons")


def test_split_axis_covers_the_axis_in_range():
    """Segment draws cover n exactly with lengths in [lo, hi] whenever such a
    split exists (a draw that would leave an unsplittable remainder is
    replaced)."""
    from phoebus_gb300.mesh import split_axis

    for lo, hi in [(6, 12), (8, 12), (16, 32), (32, 96)]:
        for n in range(lo, 6 * hi + 2, 2):
            possible = -(-n // hi) <= n // lo
            for stream in range(4):
                if possible:
                    lens = split_axis(n, lo, hi, 1234, stream)
                    assert sum(lens) == n and all(lo <= x <= hi and x % 2 == 0 for x in lens), (n, lo, hi, lens)
                else:
                    with pytest.raises((AssertionError, ValueError)):
                        split_axis(n, lo, hi, 1234, stream)


def test_conserved_exchange_inflow_check(built):
    """bc_vars = conserved with the outer-X1 inflow check on an FMKS mesh
    (ConvertBoundaryConditions, phoebus_boundaries.cpp:333-340, 366-397):
    the outer-X1 ghosts of the blocks on the outer X1 face leave the
    exchange with u^1 >= 0 although their interior neighbours flow inward,
    with primitives that con2prim of the copied conserved variables gives
    where u^1 was already >= 0, and with conserved variables that are
    prim2con of their primitives."""
    import math

    from oracle.oracle import Oracle
    from phoebus_gb300 import torus

    orc = Oracle()
    p = torus.torus_params()
    bcs = CASES["deck"]
    mesh = TiledMesh((12, 10, 1), [[6, 6], [4, 6], [1]], (math.log(1.2), 0.0, 0.0), (math.log(250.0), 1.0, 1.0),
                     *bcs, bc_vars=abi.BC_VARS_CONSERVED, ndim=2)
    blocks = mesh.make_blocks(geometry=torus.torus_geometry(), backend="numpy")
    rng = np.random.default_rng(5)
    for b, seg in zip(blocks, mesh.segments()):
        orc.GeometryFillFMKS(b)
        ks, js, is_ = b.isl()
        shp = b["prim"][0][ks, js, is_].shape
        cent = b.geom.arrays["cent"][:, js, is_][:, None]
        pr = b["prim"]
        rho = 10.0 ** rng.uniform(-3.0, 0.0, shp)
        u = rho * 10.0 ** rng.uniform(-2.0, 0.0, shp)
        pr[abi.PRHO][ks, js, is_], pr[abi.PENG][ks, js, is_], pr[abi.PPRS][ks, js, is_] = rho, u, p.gm1 * u
        for d in range(3):
            g_dd = cent[abi.G_GCOV + (d + 1) * (d + 2) // 2 + d + 1]
            pr[abi.PVEL + d][ks, js, is_] = rng.uniform(-0.5, 0.5, shp) / np.sqrt(g_dd)
            pr[abi.PB + d][ks, js, is_] = rng.uniform(-0.2, 0.2, shp) / np.sqrt(g_dd)
            if d == 0 and seg[0] == mesh.nseg[0] - 1:  # inflow at the outer X1 face
                last = pr[abi.PVEL][ks, js, is_.stop - 1]
                pr[abi.PVEL][ks, js, is_.stop - 1] = -np.abs(last) - 0.1 / np.sqrt(g_dd[..., -1])
        pr[abi.PGM1][ks, js, is_], pr[abi.PTMP][ks, js, is_] = p.gm1 + 1.0, u / rho
        pr[abi.PMU][ks, js, is_] = rng.uniform(0.1, 0.9, shp)
        orc.PrimitiveToConserved(p, b, *b.interior())
    plain = [b.to_host() for b in blocks]
    p_off = torus.torus_params()
    p_off.enable_ox1_fmks_inflow_check = 0
    mo.mesh_exchange(orc, p_off, mesh, plain)
    mo.mesh_exchange(orc, p, mesh, blocks)
    for b, q, seg in zip(blocks, plain, mesh.segments()):
        if seg[0] != mesh.nseg[0] - 1:
            continue
        ib, jb, kb = mo._slab(b, 0, True)
        sl = (slice(kb[0], kb[1] + 1), slice(jb[0], jb[1] + 1), slice(ib[0], ib[1] + 1))
        orc.ConservedToPrimitive(p, q, ib, jb, kb)  # the copied state, inverted
        cent = b.geom.arrays["cent"][:, sl[1], sl[2]][:, None]

        def gam(a, c):  # gamma_{a+1, c+1} from the packed symmetric 4-metric
            hi, lo = max(a, c) + 1, min(a, c) + 1
            return cent[abi.G_GCOV + hi * (hi + 1) // 2 + lo]

        def ucon1(P):
            v = [P[abi.PVEL + a][sl] for a in range(3)]
            vsq = sum(gam(a, c) * v[a] * v[c] for a in range(3) for c in range(3))
            return v[0] - np.sqrt(1.0 + vsq) * cent[abi.G_BETA] / cent[abi.G_ALPHA]

        before, after = ucon1(q["prim"]), ucon1(b["prim"])
        assert (before < 0).sum() > 0, "no inflow to fix"
        scale = np.abs(cent[abi.G_BETA] / cent[abi.G_ALPHA])
        assert np.all(after >= -1e-12 * scale), after.min()
        keep = before >= 0
        for v in range(abi.NPRIM):
            np.testing.assert_array_equal(b["prim"][v][sl][keep], q["prim"][v][sl][keep])
        cons = b["cons"].copy()
        orc.PrimitiveToConserved(p, b, ib, jb, kb)
        np.testing.assert_array_equal(b["cons"][(slice(None),) + sl], cons[(slice(None),) + sl])


def rad_closed_form(mesh, blocks):
    """The radiation fields' composed map per ghost: every FillGhost field
    from the source cell of all axes' maps, F_d and H_d negated per reflect
    axis (polar negates none), and under bc_vars = conserved every field
    times the DetGamma ratios in face order."""
    out = [(b["rcons"].copy(), b["rprim"].copy()) for b in blocks]
    conserved = mesh.bc_vars == abi.BC_VARS_CONSERVED
    for (U, P), b, seg in zip(out, blocks, mesh.segments()):
        org = [int(mesh.starts[d][seg[d]]) for d in range(3)]
        detg = b.geom.arrays["cent"][abi.G_DETGAM]
        for k in range(b.n3t):
            for j in range(b.n2t):
                for i in range(b.n1t):
                    loc = [i, j, k]
                    mloc, g, ghost, phys, refl = list(loc), [], False, [False] * 3, [False] * 3
                    for d in range(3):
                        if d >= b.ndim:
                            g.append(0)
                            continue
                        ghost |= not b.ng <= loc[d] < b.ng + b.nx[d]
                        gg = org[d] + loc[d] - b.ng
                        if gg < 0 or gg >= mesh.n[d]:
                            lo = gg < 0
                            bc = mesh.bc_lo[d] if lo else mesh.bc_hi[d]
                            ref = b.ng if lo else b.ng + b.nx[d] - 1
                            if bc == abi.BC_PERIODIC:
                                gg += mesh.n[d] if lo else -mesh.n[d]
                            elif bc == abi.BC_OUTFLOW:
                                phys[d], gg, mloc[d] = True, 0 if lo else mesh.n[d] - 1, ref
                            else:
                                phys[d] = True
                                gg = -1 - gg if lo else 2 * mesh.n[d] - 1 - gg
                                mloc[d] = 2 * ref + (-1 if lo else 1) - loc[d]
                                refl[d] = bc == abi.BC_REFLECT
                        g.append(gg)
                    if not ghost:
                        continue
                    o, (li, lj, lk) = mo._owner_cell(mesh, g)
                    sl = tuple(x + b.ng if d < b.ndim else 0 for d, x in enumerate((li, lj, lk)))
                    q_u = blocks[o]["rcons"][:, sl[2], sl[1], sl[0]].copy()
                    q_p = blocks[o]["rprim"][:mo.RFILL, sl[2], sl[1], sl[0]].copy()
                    for d in range(3):
                        if not phys[d]:
                            continue
                        su, sp = np.ones(abi.RNCONS), np.ones(mo.RFILL)
                        if refl[d]:
                            su[abi.RF + d] = sp[abi.RH + d] = -1.0
                        cc = [loc[e] if e <= d else mloc[e] for e in range(3)]
                        rr = [mloc[e] if e == d else cc[e] for e in range(3)]
                        gr = mo._ratio(detg[cc[1], cc[0]], detg[rr[1], rr[0]]) if conserved else 1.0
                        q_u = su * gr * q_u if conserved else su * q_u
                        q_p = sp * gr * q_p if conserved else sp * q_p
                    U[:, k, j, i] = q_u
                    P[:mo.RFILL, k, j, i] = q_p
    return out


@pytest.mark.parametrize("ndim", [3, 2])
@pytest.mark.parametrize("bc_vars", [abi.BC_VARS_PRIMITIVE, abi.BC_VARS_CONSERVED])
@pytest.mark.parametrize("name", list(CASES))
def test_rad_face_by_face_equals_composed_maps(name, bc_vars, ndim):
    """The radiation fields through the oracle's neighbour copy and
    face-by-face boundary functions equal the composed map the CUDA exchange
    implements (before ConvertBoundaryConditions' radiation steps)."""
    from phoebus_gb300.radiation import alloc_rad

    bcs = CASES[name]
    if bc_vars == abi.BC_VARS_CONSERVED and abi.BC_POLAR in bcs[0] + bcs[1]:
        pytest.skip("polar boundaries need bc_vars = primitive")
    mesh, blocks = host_mesh(bcs, 21 + list(CASES).index(name), bc_vars, ndim)
    rng = np.random.default_rng(5)
    for b in blocks:
        alloc_rad(b)
        b["rcons"][...] = rng.standard_normal(b["rcons"].shape)
        b["rprim"][...] = rng.standard_normal(b["rprim"].shape)
    want = rad_closed_form(mesh, blocks)
    mo._copy_neighbours(mesh, blocks, [("rcons", range(abi.RNCONS)), ("rprim", range(mo.RFILL))])
    for b, seg in zip(blocks, mesh.segments()):
        for d, outer, bc in mo._physical_faces(mesh, b, seg):
            mo._rad_apply_face(b, d, outer, bc, bc_vars)
    for n, (b, (U, P)) in enumerate(zip(blocks, want)):
        assert not np.isnan(b["rcons"]).any(), f"block {n}: a ghost no rule filled"
        np.testing.assert_array_equal(b["rcons"], U, err_msg=f"block {n} rcons")
        np.testing.assert_array_equal(b["rprim"][:mo.RFILL], P[:mo.RFILL], err_msg=f"block {n} rprim")
