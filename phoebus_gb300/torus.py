"""Magnetised Fishbone-Moncrief torus on a tiled FMKS Kerr-Schild mesh.

The deck of phoebus's torus problem (inputs/torus.pin: FMKS a = 0.9375,
Gamma 13/9, WENO5-Z + HLL, ExpX1RhoSie floors, gr_outflow X1/X2 with
bc_vars = primitive, periodic X3) on a mesh of uneven blocks, and its initial
state through phx_torus_init: the problem generator of pgen/torus.cpp on the
GPU (Fishbone & Moncrief solution, pressure noise, floors, poloidal field
from A_phi, HARM-style normalisation), restated in the oracle for parity.
"""
from __future__ import annotations

import math

from . import abi, states
from .mesh import TiledMesh, split_axis

TORUS_SEED = states.SEED + 5


def _gidx(m, n):
    return abi.G_GCOV + states._flat2(m, n)


def torus_params(Gamma: float = 13.0 / 9.0):
    """Fluid/fixup settings of the torus run: WENO5-Z + HLL, tolerance 1e-10,
    ExpX1RhoSie floors (rho0 1e-6, rho exponent -1.5, sie0 1e-3, sie
    exponent -1), MHD floors, ceilings gamma 10 / sie 1 (torus.pin), c2p
    fixup, FixFluxes and the outer-X1 inflow check (torus.pin:141, 151)."""
    p = abi.default_params(Gamma=Gamma, recon="weno5z", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)
    p.enable_floors, p.enable_mhd_floors, p.enable_ceilings, p.enable_c2p_fixup = 1, 1, 1, 1
    p.enable_flux_fixup, p.enable_ox1_fmks_inflow_check = 1, 1
    p.floor_type = abi.FLOOR["ExpX1RhoSie"]
    p.rho0_floor, p.rho_exp_floor, p.sie0_floor, p.sie_exp_floor = 1e-6, -1.5, 1e-3, -1.0
    p.gam0_ceiling, p.sie0_ceiling = 10.0, 1.0
    return p


def torus_geometry(a: float = 0.9375) -> abi.Geometry:
    return abi.default_geometry(abi.GEOM_FMKS, a=a, derefine_poles=0)


def torus_mesh(n: int = 384, seed: int = TORUS_SEED, lo: int = 32, hi: int = 96, r_in_domain: float = 1.2,
               r_out: float = 250.0) -> TiledMesh:
    """n^3 FMKS cells, X1 = ln r in [ln 1.2, ln 250], X2 in [0, 1],
    X3 in [0, 2 pi), each axis split into segments of lo..hi (even) cells;
    outflow in X1 and X2 (the deck's gr_outflow), periodic in X3, bc_vars =
    primitive (torus.pin:17)."""
    segs = [split_axis(n, lo, hi, seed, 10 + d) for d in range(3)]
    return TiledMesh((n, n, n), segs, (math.log(r_in_domain), 0.0, 0.0), (math.log(r_out), 1.0, 2.0 * math.pi),
                     (abi.BC_OUTFLOW, abi.BC_OUTFLOW, abi.BC_PERIODIC), (abi.BC_OUTFLOW, abi.BC_OUTFLOW, abi.BC_PERIODIC),
                     bc_vars=abi.BC_VARS_PRIMITIVE)


def torus_problem(u_jitter: float = 0.04, seed: int = TORUS_SEED, **over) -> abi.TorusParams:
    """The torus deck's problem parameters (r_in 6, r_max 12, kappa 1e-2,
    HARM-style beta 100) with the benchmark's 4% pressure noise."""
    return abi.default_torus_params(u_jitter=u_jitter, seed=seed, **over)


def fill_torus(ctx, p: abi.Params, mesh: TiledMesh, blocks, tp: abi.TorusParams | None = None):
    """The torus initial state on the GPU: FMKS tables, phx_torus_init (the
    problem generator on every block, prim2con and floors, the field
    normalisation), then the start of the run -- the mesh exchange and
    con2prim with floors on every block."""
    tp = torus_problem() if tp is None else tp
    for b in blocks:
        ctx.GeometryFillFMKS(b)
    fac = ctx.TorusInit(p, tp, blocks)
    ctx.MeshExchange(p, mesh, blocks)
    for b in blocks:
        ctx.ConservedToPrimitive(p, b)
        ctx.ApplyFloors(p, b)
    return {"field_factor": fac}


def _bsq(pr, cent):
    """b^2 = B^2 / W^2 + (B.v)^2 at every cell (gamma_ij from the table)."""
    import torch

    def g(m, n):
        return cent[_gidx(m + 1, n + 1)]

    wv = [pr[abi.PVEL + d] for d in range(3)]
    Bv = [pr[abi.PB + d] for d in range(3)]
    wsq = sum(g(m, n) * wv[m] * wv[n] for m in range(3) for n in range(3))
    W = torch.sqrt(1.0 + wsq)
    Bsq = sum(g(m, n) * Bv[m] * Bv[n] for m in range(3) for n in range(3))
    Bdv = sum(g(m, n) * Bv[m] * wv[n] for m in range(3) for n in range(3)) / W
    return Bsq / (W * W) + Bdv * Bdv
