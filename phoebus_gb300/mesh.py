"""A domain tiled by uneven blocks (tensor product of per-axis segments), the
host description behind phx_mesh (phx_stage_mesh, phx_mesh_exchange).

Block (s1, s2, s3) is blocks[(s3 * nseg2 + s2) * nseg1 + s1]; its interior
is the global cells seg[d][s_d] .. seg[d][s_d + 1] - 1 of each axis.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from .block import Block, GeomTables


def split_axis(n: int, lo: int, hi: int, seed: int, stream: int, step: int = 2) -> list[int]:
    """Segment lengths in [lo, hi] (multiples of step) that sum to n, drawn
    from the SplitMix64 stream.  A draw whose remainder could not be split
    into lengths in range is replaced by the nearest length whose remainder
    can."""
    from .states import uniform

    def splittable(r):  # r = 0, or some m lengths in [lo, hi] sum to r
        return r == 0 or -(-r // hi) <= r // lo

    u = uniform(seed, stream, 4 * n // lo + 8)
    lens, left, k = [], n, 0
    choices = list(range(lo, hi + 1, step))
    while left > hi:
        L = choices[min(int(u[k] * len(choices)), len(choices) - 1)]
        k += 1
        if not splittable(left - L):
            ok = [c for c in choices if c < left and splittable(left - c)]
            L = min(ok, key=lambda c: (abs(c - L), c))
        lens.append(L)
        left -= L
    lens.append(left)
    assert sum(lens) == n and all(lo <= x <= hi for x in lens), lens
    return lens


class TiledMesh:
    """Global interior cells n = (n1, n2, n3) over [xmin, xmax] per axis,
    split into segments; boundary conditions per face (abi.BC_*), the
    exchanged variables (abi.BC_VARS_*; conserved is the reference's
    default), ndim active axes (an inactive axis has n = 1)."""

    def __init__(self, n, segs, xmin, xmax, bc_lo, bc_hi, ng: int = 4, bc_vars: int = abi.BC_VARS_CONSERVED,
                 ndim: int = 3):
        self.ndim = ndim
        self.bc_vars = bc_vars
        self.n = tuple(int(x) for x in n)
        self.lens = [list(map(int, s)) for s in segs]
        self.starts = [np.concatenate([[0], np.cumsum(s)]).astype(np.int32) for s in self.lens]
        for d in range(3):
            assert self.starts[d][-1] == self.n[d]
        self.xmin, self.xmax = tuple(xmin), tuple(xmax)
        self.dx = tuple((self.xmax[d] - self.xmin[d]) / self.n[d] for d in range(3))
        self.bc_lo, self.bc_hi = tuple(bc_lo), tuple(bc_hi)
        self.ng = ng
        self.nseg = tuple(len(s) for s in self.lens)

    @property
    def nblocks(self):
        return self.nseg[0] * self.nseg[1] * self.nseg[2]

    def block_index(self, s1, s2, s3):
        return (s3 * self.nseg[1] + s2) * self.nseg[0] + s1

    def segments(self):
        """(s1, s2, s3) in block order."""
        for s3 in range(self.nseg[2]):
            for s2 in range(self.nseg[1]):
                for s1 in range(self.nseg[0]):
                    yield s1, s2, s3

    def make_blocks(self, device="cuda", geometry: abi.Geometry | None = None, backend: str = "torch"):
        """Allocated blocks (torch on device, or numpy with backend="numpy")
        in block order, with FMKS table storage when geometry is FMKS."""
        blocks = []
        for s1, s2, s3 in self.segments():
            s = (s1, s2, s3)
            nx = tuple(self.lens[d][s[d]] for d in range(3))
            xmin = tuple(self.xmin[d] + self.starts[d][s[d]] * self.dx[d] for d in range(3))
            b = Block(nx, self.ng, self.ndim, xmin, self.dx, backend=backend, device=device).alloc()
            if geometry is not None and geometry.kind == abi.GEOM_FMKS:
                b.geom = GeomTables(geometry, b.n1t, b.n2t, backend, device).alloc()
            blocks.append(b)
        return blocks

    def struct(self) -> abi.Mesh:
        m = abi.Mesh()
        self._keep = [np.ascontiguousarray(x, dtype=np.int32) for x in self.starts]
        for d in range(3):
            m.n[d] = self.n[d]
            m.nseg[d] = self.nseg[d]
            m.seg_start[d] = self._keep[d].ctypes.data_as(C.c_void_p)
            m.bc_lo[d] = self.bc_lo[d]
            m.bc_hi[d] = self.bc_hi[d]
        m.bc_vars = self.bc_vars
        return m
