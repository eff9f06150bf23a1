"""Host API of the GB300 radiation moment transport, mirroring the reference's
radiation package tasks (src/radiation/moments.cpp, moments_source.cpp,
radiation.cpp) for the moment_m1 / moment_eddington methods:

    MomentPrim2Con             moments.cpp:198-275
    MomentCon2Prim             moments.cpp:61-192
    MomentCalculateOpacities   moments.cpp:919-995
    ReconstructEdgeStates +
    CalculateFluxes            moments.cpp:280-736 (fused on the device)
    MomentFluidSource          moments_source.cpp:203-965 (oned; update_fluid either way)
    RadConservedToPrimitiveFixup fixup_radc2p.cpp:45-225
    ApplyFloors (radiation on) fixup.cpp:285-678
    EstimateTimestepBlock      radiation.cpp:585-648
plus the RK stage glue of PhoebusDriver::RungeKuttaStage with the fluid not
evolved (Stage) or evolved with the moments (FluidStage), and the problem
generators radiation_advection (pgen/radiation_advection.cpp, which the
radiation_diffusion regression runs) and radiation_equilibration
(pgen/radiation_equilibration.cpp).
All work runs on the GPU through include/phx_radiation.h; there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import abi
from .block import Block, _ptr
from .fluid import FluidContext, _rng, _stream

RAD_FIELDS = {"rcons": abi.RNCONS, "rprim": abi.RNPRIM, "rflux": 3 * abi.RNCONS, "rdudt": abi.RNCONS}


def alloc_rad(b: Block, fill: float = 0.0) -> Block:
    """Allocate the radiation fields of b on b's backend."""
    for n, nv in RAD_FIELDS.items():
        shp = (nv,) + b.shape
        if b.backend == "numpy":
            b.arrays[n] = np.full(shp, fill, dtype=np.float64)
        else:
            import torch

            b.arrays[n] = torch.full(shp, fill, dtype=torch.float64, device=b.device)
    return b


def rad_struct(b: Block, cons=None) -> abi.RadBlockS:
    s = abi.RadBlockS()
    s.var_stride = 0
    s.cons = _ptr(b.arrays["rcons"] if cons is None else cons)
    s.prim = _ptr(b.arrays["rprim"])
    s.flux = _ptr(b.arrays.get("rflux"))
    s.dudt = _ptr(b.arrays.get("rdudt"))
    return s


class RadiationContext:
    """Radiation tasks on device Blocks, sharing a FluidContext's phx_ctx."""

    def __init__(self, fluid: FluidContext):
        self.fc = fluid
        self.lib = fluid.lib
        self.h = fluid.h

    def _ok(self, st):
        abi.check(self.lib, st)

    def check(self):
        self.fc.check()

    def MomentPrim2Con(self, rp, p, b: Block, ib=None, jb=None, kb=None, stream=None):
        e = b.interior()
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_prim_to_con(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r),
                                              _rng(ib or e[0]), _rng(jb or e[1]), _rng(kb or e[2]), _stream(stream)))

    def MomentCon2Prim(self, rp, p, b: Block, ib=None, jb=None, kb=None, stream=None):
        e = b.entire()
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_con_to_prim(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r),
                                              _rng(ib or e[0]), _rng(jb or e[1]), _rng(kb or e[2]), _stream(stream)))

    def MomentCalculateOpacities(self, rp, p, b: Block, stream=None):
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_calculate_opacities(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r),
                                                      _stream(stream)))

    def CalculateFluxes(self, rp, p, b: Block, stream=None):
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_calculate_fluxes(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r),
                                                   _stream(stream)))

    def Update(self, rp, b: Block, base, out, beta, dt, stream=None):
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_update(self.h, C.byref(rp), C.byref(s), C.byref(r), _ptr(base), _ptr(out),
                                         float(beta), float(dt), _stream(stream)))

    def MomentFluidSource(self, rp, p, b: Block, dt, stream=None):
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_fluid_source(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r),
                                               float(dt), _stream(stream)))

    def RadConservedToPrimitiveFixup(self, rp, p, b: Block, stream=None):
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_c2p_fixup(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r), _stream(stream)))

    def ApplyFloors(self, rp, p, b: Block, ib=None, jb=None, kb=None, stream=None):
        """fixup::ApplyFloors with radiation active (phx_rad_apply_floors)."""
        e = b.entire()
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_apply_floors(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r),
                                               _rng(ib or e[0]), _rng(jb or e[1]), _rng(kb or e[2]), _stream(stream)))

    def FillGhostsPeriodic(self, b: Block, stream=None):
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_fill_ghosts_periodic(self.h, C.byref(s), C.byref(r), _stream(stream)))

    def MeshExchange(self, rp, p, mesh, blocks, stream=None):
        """The radiation fields' boundary exchange of a tiled mesh
        (phx_rad_mesh_exchange); run after the fluid's (FluidContext.MeshExchange)."""
        n = len(blocks)
        arr = (abi.BlockS * n)(*[b.struct() for b in blocks])
        rarr = (abi.RadBlockS * n)(*[rad_struct(b) for b in blocks])
        m = mesh.struct()
        self._ok(self.lib.phx_rad_mesh_exchange(self.h, C.byref(rp), C.byref(p), C.byref(m), arr, rarr, n,
                                                _stream(stream)))

    def FixFluxes(self, rp, p, mesh, blocks, stream=None):
        """FixFluxes' radiation part on the blocks' radiation fluxes
        (phx_rad_fix_fluxes)."""
        n = len(blocks)
        arr = (abi.BlockS * n)(*[b.struct() for b in blocks])
        rarr = (abi.RadBlockS * n)(*[rad_struct(b) for b in blocks])
        m = mesh.struct()
        self._ok(self.lib.phx_rad_fix_fluxes(self.h, C.byref(rp), C.byref(p), C.byref(m), arr, rarr, n,
                                             _stream(stream)))

    def EstimateTimestepBlock(self, rp, p, b: Block, out=None, stream=None) -> float:
        """cfl * min dx / csig; returns a float (synchronising) unless out (a
        one-element CUDA tensor) is given."""
        import torch

        o = out if out is not None else torch.empty(1, dtype=torch.float64, device=b.device)
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_estimate_timestep(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r),
                                                    _ptr(o), _stream(stream)))
        return o if out is not None else float(o.item())

    def Stage(self, rp, p, b: Block, base, out, beta, dt, stream=None):
        """One RK stage (phx_rad_stage): b['rcons'] is the stage input."""
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_stage(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r), _ptr(base),
                                        _ptr(out), float(beta), float(dt), _stream(stream)))

    # ---- composite sequences
    def Initialize(self, rp, p, b: Block):
        """Parthenon's mesh initialisation after the problem generator: the
        ghost exchange, then FillDerived (MomentCon2Prim on the entire block)."""
        self.FillGhostsPeriodic(b)
        self.MomentCon2Prim(rp, p, b)

    def rk2_step(self, rp, p, b: Block, stage_buf, dt):
        """Two stages of Parthenon's rk2 (beta 1, then 1/2); the result is left
        in b['rcons'].  stage_buf: a scratch array shaped like b['rcons']."""
        base = b.arrays["rcons"]
        self.Stage(rp, p, b, base, stage_buf, 1.0, dt)
        b.arrays["rcons"] = stage_buf
        self.Stage(rp, p, b, base, base, 0.5, dt)
        b.arrays["rcons"] = base

    def FluidStage(self, rp, p, b: Block, fbase, fout, rbase, rout, beta, dt, stream=None):
        """One RK stage of the fluid and the moments together
        (phx_rad_fluid_stage): b['cons'] and b['rcons'] are the stage inputs."""
        s, r = b.struct(), rad_struct(b)
        self._ok(self.lib.phx_rad_fluid_stage(self.h, C.byref(rp), C.byref(p), C.byref(s), C.byref(r), _ptr(fbase),
                                              _ptr(fout), _ptr(rbase), _ptr(rout), float(beta), float(dt),
                                              _stream(stream)))

    def rk2_fluid_step(self, rp, p, b: Block, fluid_buf, rad_buf, dt):
        """rk2 of the coupled system; U^{n+1} is left in b['cons'] and
        b['rcons']."""
        fb, rb = b.arrays["cons"], b.arrays["rcons"]
        self.FluidStage(rp, p, b, fb, fluid_buf, rb, rad_buf, 1.0, dt)
        b.arrays["cons"], b.arrays["rcons"] = fluid_buf, rad_buf
        b._struct = None
        self.FluidStage(rp, p, b, fb, fb, rb, rb, 0.5, dt)
        b.arrays["cons"], b.arrays["rcons"] = fb, rb
        b._struct = None


# ---------------------------------------------------------------- problem
def radiation_advection(nx1: int = 512, ng: int = 4, J0: float = 1.0, H=(0.0, 0.0, 0.0), vx: float = 0.3,
                        width: float = 0.0333, tau: float = 1.0e3, boost: bool = True, Cv: float = 1.0):
    """pgen/radiation_advection.cpp on inputs/radiation_advection.pin with the
    radiation_diffusion regression's inputs (tst/regression/
    radiation_diffusion.py): a 1D periodic Minkowski block of nx1 zones on
    [0, 1] (X2, X3 inactive on [-1, 1]), rho = T = 1, u^1 = W vx, the boosted
    diffusion profile of J, H = 0, xi = 0, phi = 1.000001 pi; gray scattering
    kappa = tau / (rho0 dx1) (ProblemModifier), no absorption, scale-free
    units.  The fluid primitives stay zero in the ghost zones: the pgen sets
    the interior only, the fluid is not evolved, and with bc_vars =
    conserved (the deck's bc_vars line sits in <parthenon/mesh>, which
    phoebus does not read: fluid.cpp:153) the primitives carry no FillGhost,
    so the reference's ghost values keep their zero initialisation.  Returns
    (host Block with fluid and radiation fields, fluid params, radiation
    params, tlim)."""
    b = Block((nx1, 1, 1), ng=ng, ndim=1, xmin=(0.0, -1.0, -1.0), dx=(1.0 / nx1, 2.0, 2.0), backend="numpy")
    b.alloc(["prim", "cons", "flux", "face_sig", "cell_sig", "fail", "src", "emf", "dudt"])
    alloc_rad(b)
    kappa = tau / (1.0 * (1.0 - 0.0))
    W = 1 / math.sqrt(1 - vx * vx)
    t0p = 1.5 * kappa * width * width
    t0 = t0p
    x0p = (0.5 - vx * t0) * W
    P, R = b["prim"], b["rprim"]
    sl = b.isl()
    x = (b.xmin[0] + (np.arange(nx1) + 0.5) * b.dx[0])[None, None, :]
    P[abi.PRHO][sl] = 1.0
    P[abi.PTMP][sl] = 1.0
    P[abi.PENG][sl] = 1.0 * (Cv * 1.0)
    P[abi.PVEL][sl] = W * vx
    P[abi.PVEL + 1][sl] = 0.0
    P[abi.PVEL + 2][sl] = 0.0
    tp = W * (t0 - vx * x)
    xp = W * (x - vx * t0)
    R[abi.RXI][sl] = 0.0
    R[abi.RPHI][sl] = math.acos(-1.0) * 1.000001
    if boost:
        R[abi.RJ][sl] = J0 * np.maximum(np.sqrt(t0p / tp) * np.exp(-3 * kappa * (xp - x0p) ** 2 / (4 * tp)), 1.0e-10)
    else:
        R[abi.RJ][sl] = J0 * np.maximum(np.exp(-(((x - 0.5) / width) ** 2) / 2.0), 1.0e-10)
    for d in range(3):
        R[abi.RH + d][sl] = H[d]
    par = dict(Gamma=1.6666666666666666667, Cv=Cv, recon="weno5", riemann="hll", cfl=0.8, mhd=0,
               c2p_max_iter=100)
    rpar = dict(method="moment_m1", recon="linear", cfl=0.5, kappa_s=kappa, kappa_a=0.0, jbb_coeff=0.0)
    return b, par, rpar, 1.0


def radiation_pulse_3d(n: int = 128, ng: int = 4, v=(0.3, 0.0, 0.0), kappa_dx: float = 2.0, kappa_a: float = 1.0,
                       jbb_coeff: float = 1.0e-3, width: float = 0.08, Cv: float = 1.0):
    """A 3D periodic M1 workload in the regime of the radiation_diffusion
    regression: n^3 zones on [0, 1]^3, rho = T = 1, a uniform fluid velocity
    v (u^i = W v^i, also in the ghosts), a Gaussian pulse of J (floor 1e-10)
    with H = 0, gray scattering with kappa dx = kappa_dx (optical depth ~2 per
    zone, so the asymptotic and free-streaming fluxes mix), weak gray
    absorption with JBB = jbb_coeff T^4.  Returns (host Block, fluid params,
    radiation params)."""
    dx = 1.0 / n
    b = Block((n, n, n), ng=ng, ndim=3, xmin=(0.0, 0.0, 0.0), dx=(dx, dx, dx), backend="numpy")
    b.alloc(["prim", "cons", "flux", "face_sig", "cell_sig", "fail", "src", "emf", "dudt"])
    alloc_rad(b)
    vv = np.array(v, dtype=np.float64)
    W = 1 / math.sqrt(1 - float(vv @ vv))
    P, R = b["prim"], b["rprim"]
    P[abi.PRHO] = 1.0
    P[abi.PTMP] = 1.0
    P[abi.PENG] = 1.0 * (Cv * 1.0)
    for d in range(3):
        P[abi.PVEL + d] = W * vv[d]
    x = (np.arange(b.n1t) - ng + 0.5) * dx
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    r2 = (X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2
    R[abi.RJ] = np.maximum(np.exp(-r2 / (2 * width * width)), 1.0e-10)
    R[abi.RXI] = 0.0
    R[abi.RPHI] = math.acos(-1.0)
    par = dict(Gamma=1.6666666666666666667, Cv=Cv, mhd=0)
    rpar = dict(method="moment_m1", recon="linear", cfl=0.5, kappa_s=kappa_dx / dx, kappa_a=kappa_a,
                jbb_coeff=jbb_coeff)
    return b, par, rpar


def radiation_equilibration(nx1: int = 4, ng: int = 4, rho0: float = 1.0, Tg0: float = 1.0, Tr0: float = 1.0e-2,
                            kappa: float = 0.2, Cv: float = 1.0, Gamma: float = 1.6666666666666666667,
                            jbb_coeff: float = 1.0):
    """pgen/radiation_equilibration.cpp on inputs/radiation_equilibration.pin:
    a 1D periodic Minkowski block of nx1 zones on [0, 1] (X2, X3 inactive on
    [-1, 1]), gas at rest with rho = rho0, T = Tg0 (ideal gas, Gamma 5/3,
    Cv 1), radiation J = JBB(Tr0), H = 0, over the entire block; gray
    absorption kappa (the deck's gray_kappa 0.2, no scattering) with
    JBB = jbb_coeff T^4 in the run's units.  The pgen sets every zone, ghosts
    included, and prim2cons the fluid over the entire block
    (fluid::PrimitiveToConserved) and the moments over the entire block;
    the stored c2p guesses (mu, xi, phi) stay zero.  Returns (host Block,
    fluid params, radiation params, tlim)."""
    b = Block((nx1, 1, 1), ng=ng, ndim=1, xmin=(0.0, -1.0, -1.0), dx=(1.0 / nx1, 2.0, 2.0), backend="numpy")
    b.alloc(["prim", "cons", "flux", "face_sig", "cell_sig", "fail", "src", "emf", "dudt"])
    alloc_rad(b)
    gm1 = Gamma - 1.0
    P, R = b["prim"], b["rprim"]
    P[abi.PRHO] = rho0
    P[abi.PTMP] = Tg0
    P[abi.PPRS] = max(0.0, gm1 * rho0 * Cv * Tg0)                      # PressureFromDensityTemperature
    P[abi.PENG] = rho0 * max(0.0, Cv * Tg0)                            # rho * InternalEnergyFromDensityTemperature
    P[abi.PGM1] = max(0.0, Gamma * gm1 * rho0 * Cv * Tg0) / P[abi.PPRS]  # BulkModulus / P
    R[abi.RJ] = jbb_coeff * (Tr0 * Tr0) * (Tr0 * Tr0)
    par = dict(Gamma=Gamma, Cv=Cv, recon="weno5", riemann="hll", cfl=0.8, mhd=0, c2p_max_iter=100)
    rpar = dict(method="moment_eddington", recon="linear", cfl=0.8, kappa_s=0.0, kappa_a=kappa,
                jbb_coeff=jbb_coeff)
    return b, par, rpar, 1.0
