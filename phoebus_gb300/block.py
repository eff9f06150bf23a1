"""Meshblock storage: SoA FP64 fields in Parthenon's per-variable layout.

A Block owns the arrays the hot path reads and writes (prims, cons, fluxes,
signal speeds, fail flags, sources, EMFs, dU/dt) either as numpy arrays on the
host or as torch CUDA tensors in HBM; `struct()` describes them to the C ABI.
Arrays are shaped (nvar, n3t, n2t, n1t) so a[v, k, j, i] is field(v, k, j, i).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

FIELDS = {  # name -> number of variables
    "prim": abi.NPRIM,
    "cons": abi.NCONS,
    "flux": 3 * abi.NCONS,
    "face_sig": 3,
    "cell_sig": 3,
    "fail": 1,
    "src": 4,
    "emf": 3,
    "dudt": abi.NCONS,
}


def _ptr(a) -> int:
    if a is None:
        return 0
    if isinstance(a, np.ndarray):
        assert a.flags.c_contiguous and a.dtype == np.float64
        return a.ctypes.data
    assert a.is_contiguous() and str(a.dtype) == "torch.float64"
    return a.data_ptr()


@dataclass
class Block:
    nx: tuple[int, int, int]
    ng: int = 4
    ndim: int = 3
    xmin: tuple[float, float, float] = (0.0, 0.0, 0.0)
    dx: tuple[float, float, float] = (1.0, 1.0, 1.0)
    backend: str = "numpy"  # "numpy" (host) or "torch" (CUDA)
    device: str = "cuda"
    arrays: dict = field(default_factory=dict)
    geom: object = None  # GeomTables or None (Minkowski)

    def __post_init__(self):
        nx1, nx2, nx3 = self.nx
        if self.ndim < 2:
            assert nx2 == 1
        if self.ndim < 3:
            assert nx3 == 1
        self.n1t = nx1 + 2 * self.ng
        self.n2t = nx2 + 2 * self.ng if self.ndim >= 2 else 1
        self.n3t = nx3 + 2 * self.ng if self.ndim >= 3 else 1
        self.N = self.n1t * self.n2t * self.n3t
        self._struct = None
        self._gstruct = None

    @property
    def shape(self):
        return (self.n3t, self.n2t, self.n1t)

    def alloc(self, names=None, fill=0.0):
        names = names or list(FIELDS)
        for n in names:
            shp = (FIELDS[n],) + self.shape
            if self.backend == "numpy":
                self.arrays[n] = np.full(shp, fill, dtype=np.float64)
            else:
                import torch

                self.arrays[n] = torch.full(shp, fill, dtype=torch.float64, device=self.device)
        self._struct = None
        return self

    def __getitem__(self, name):
        return self.arrays[name]

    def set(self, name, value):
        self.arrays[name] = value
        self._struct = None

    # index ranges (Parthenon IndexRange, inclusive)
    def interior(self):
        ng = self.ng
        nx1, nx2, nx3 = self.nx
        ib = (ng, ng + nx1 - 1)
        jb = (ng, ng + nx2 - 1) if self.ndim >= 2 else (0, 0)
        kb = (ng, ng + nx3 - 1) if self.ndim >= 3 else (0, 0)
        return ib, jb, kb

    def entire(self):
        return (0, self.n1t - 1), (0, self.n2t - 1), (0, self.n3t - 1)

    def isl(self):
        """numpy/torch slices of the interior (k, j, i)."""
        (i0, i1), (j0, j1), (k0, k1) = self.interior()
        return slice(k0, k1 + 1), slice(j0, j1 + 1), slice(i0, i1 + 1)

    def struct(self, cons=None) -> abi.BlockS:
        s = abi.BlockS()
        s.nx1, s.nx2, s.nx3 = self.nx
        s.ng, s.ndim, s.var_stride = self.ng, self.ndim, 0
        s.x1min, s.x2min, s.x3min = self.xmin
        s.dx1, s.dx2, s.dx3 = self.dx
        for n in FIELDS:
            setattr(s, n, _ptr(self.arrays.get(n)))
        if cons is not None:
            s.cons = _ptr(cons)
        if self.geom is not None:
            self._gstruct = self.geom.struct()
            s.geom = C.pointer(self._gstruct)
        else:
            s.geom = None
        return s

    def to_host(self) -> "Block":
        """A numpy copy of this block (geometry tables included)."""
        h = Block(self.nx, self.ng, self.ndim, self.xmin, self.dx, backend="numpy")
        for n, a in self.arrays.items():
            h.arrays[n] = a.copy() if isinstance(a, np.ndarray) else a.detach().cpu().numpy().copy()
        if self.geom is not None:
            h.geom = self.geom.to_host()
        return h

    def to_device(self, device="cuda") -> "Block":
        import torch

        d = Block(self.nx, self.ng, self.ndim, self.xmin, self.dx, backend="torch", device=device)
        for n, a in self.arrays.items():
            d.arrays[n] = torch.from_numpy(np.ascontiguousarray(a)).to(device) if isinstance(a, np.ndarray) else a.clone()
        if self.geom is not None:
            d.geom = self.geom.to_device(device)
        return d


@dataclass
class GeomTables:
    """FMKS per-block tables (cached geometry, axisymmetric)."""

    params: abi.Geometry
    n1t: int
    n2t: int
    backend: str = "numpy"
    device: str = "cuda"
    arrays: dict = field(default_factory=dict)

    def alloc(self):
        shapes = {
            "cent": (abi.GEOM_NLOC, self.n2t, self.n1t),
            "face1": (abi.GEOM_NLOC, self.n2t, self.n1t + 1),
            "face2": (abi.GEOM_NLOC, self.n2t + 1, self.n1t),
            "deriv": (abi.GEOM_NDER, self.n2t, self.n1t),
        }
        for n, shp in shapes.items():
            if self.backend == "numpy":
                self.arrays[n] = np.zeros(shp)
            else:
                import torch

                self.arrays[n] = torch.zeros(shp, dtype=torch.float64, device=self.device)
        return self

    def struct(self) -> abi.Geometry:
        g = abi.Geometry()
        C.memmove(C.byref(g), C.byref(self.params), C.sizeof(abi.Geometry))
        for n in ("cent", "face1", "face2", "deriv"):
            setattr(g, n, _ptr(self.arrays[n]))
        return g

    def to_host(self):
        h = GeomTables(self.params, self.n1t, self.n2t, "numpy")
        for n, a in self.arrays.items():
            h.arrays[n] = a.copy() if isinstance(a, np.ndarray) else a.detach().cpu().numpy().copy()
        return h

    def to_device(self, device="cuda"):
        import torch

        d = GeomTables(self.params, self.n1t, self.n2t, "torch", device)
        for n, a in self.arrays.items():
            d.arrays[n] = torch.from_numpy(np.ascontiguousarray(a)).to(device) if isinstance(a, np.ndarray) else a.clone()
        return d
