"""The mesh oracle's literal face-by-face boundary application (neighbour
exchange, then the physical faces X1, X2, X3 in turn, each over the entire
range of the other axes) against the closed form the CUDA exchange
implements: every axis maps the ghost's global cell on its own (periodic
wrap, clamp, mirror) and the signs of the mirrored vector components
multiply.  Host only."""
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


def host_mesh(bcs, seed):
    mesh = TiledMesh((14, 12, 10), [[6, 8], [4, 8], [5, 5]], (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), *bcs)
    rng = np.random.default_rng(seed)
    blocks = []
    for s1, s2, s3 in mesh.segments():
        nx = (mesh.lens[0][s1], mesh.lens[1][s2], mesh.lens[2][s3])
        b = Block(nx, 4, 3).alloc(["prim", "cons"])
        b["prim"][...] = rng.standard_normal(b["prim"].shape)
        b["cons"][...] = rng.standard_normal(b["cons"].shape)
        blocks.append(b)
    return mesh, blocks


def closed_form(mesh, blocks, mhd=True):
    """Per ghost: the source cell of all axes' maps, signs multiplied."""
    out = [(b["prim"].copy(), b["cons"].copy()) for b in blocks]
    for (P, U), b, seg in zip(out, blocks, mesh.segments()):
        org = [int(mesh.starts[d][seg[d]]) for d in range(3)]
        for k in range(b.n3t):
            for j in range(b.n2t):
                for i in range(b.n1t):
                    loc = (i, j, k)
                    g, sp, su, ghost, physical = [], np.ones(abi.NPRIM), np.ones(abi.NCONS), False, False
                    for d in range(3):
                        if not b.ng <= loc[d] < b.ng + b.nx[d]:
                            ghost = True
                        gg = org[d] + loc[d] - b.ng
                        if gg < 0 or gg >= mesh.n[d]:
                            lo = gg < 0
                            bc = mesh.bc_lo[d] if lo else mesh.bc_hi[d]
                            if bc == abi.BC_PERIODIC:
                                gg += mesh.n[d] if lo else -mesh.n[d]
                            elif bc == abi.BC_OUTFLOW:
                                physical = True
                                gg = 0 if lo else mesh.n[d] - 1
                            else:
                                physical = True
                                gg = -1 - gg if lo else 2 * mesh.n[d] - 1 - gg
                                c = 1 if bc == abi.BC_POLAR else d
                                sp[abi.PVEL + c] *= -1
                                sp[abi.PB + c] *= -1
                                if bc == abi.BC_REFLECT:
                                    su[mo.CMOM + d] *= -1
                                    su[mo.CB + d] *= -1
                        g.append(gg)
                    if not ghost:
                        continue
                    o, (li, lj, lk) = mo._owner_cell(mesh, g)
                    src = blocks[o]
                    P[:, k, j, i] = sp * src["prim"][:, lk + b.ng, lj + b.ng, li + b.ng]
                    U[:, k, j, i] = (su if physical else 1.0) * src["cons"][:, lk + b.ng, lj + b.ng, li + b.ng]
    return out


@pytest.mark.parametrize("name", list(CASES))
def test_face_by_face_equals_composed_maps(name):
    mesh, blocks = host_mesh(CASES[name], seed=11 + list(CASES).index(name))
    want = closed_form(mesh, blocks)
    mo._exchange_neighbours(mesh, blocks, True)
    for b, seg in zip(blocks, mesh.segments()):
        for d, outer, bc in mo._physical_faces(mesh, b, seg):
            mo._apply_face(b, d, outer, bc, True)
    for n, (b, (P, U)) in enumerate(zip(blocks, want)):
        assert not np.isnan(b["prim"]).any(), f"block {n}: a ghost no rule filled"
        np.testing.assert_array_equal(b["prim"], P, err_msg=f"block {n} prim")
        np.testing.assert_array_equal(b["cons"], U, err_msg=f"block {n} cons")
