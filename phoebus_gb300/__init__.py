"""GB300-native (sm_103a) GRMHD fluid hot path of phoebus.

Hand-written FP64 CUDA kernels behind the C ABI of include/phx_fluid.h:
reconstruction (PLM, WENO5-Z, MP5) + LLF/HLL Riemann fluxes, the robust
con2prim root find, geometric source terms and the RK stage glue, for
Minkowski and FMKS (cached, axisymmetric) geometry; and the radiation M1 /
Eddington moment transport behind include/phx_radiation.h.  `fluid` and
`radiation` are the host APIs mirroring the reference task names; `states`,
`torus` and `radiation` make seeded initial states.
"""
from . import abi  # noqa: F401
from .block import Block, GeomTables  # noqa: F401

__all__ = ["abi", "Block", "GeomTables"]
