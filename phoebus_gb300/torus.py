"""Magnetised Fishbone-Moncrief torus on a tiled FMKS Kerr-Schild mesh.

The initial state of phoebus's torus problem (pgen/torus.cpp:130-474,
525-740, 743-840), restated from the Fishbone & Moncrief (1976) solution:
constant specific angular momentum l fixed by the pressure maximum r_max
(lfish_calc), log enthalpy ln h(r, theta) relative to the inner edge r_in,
rho = (h - 1)(Gamma - 1) / (kappa Gamma))^(1 / (Gamma - 1)) normalised to
rho = 1 at r_max, u = kappa rho^Gamma / (Gamma - 1); the fluid rotates with
u^phi of the solution (Boyer-Lindquist -> Kerr-Schild -> FMKS: u^r = 0, so
only u^phi survives).  The poloidal field comes from A_phi = max(rho_av - 0.2,
0) at cell corners (rho_av: the mean of the four cells around the corner) and
is scaled so that max P / max (b^2 / 2) = beta (HARM-style normalisation,
torus.cpp:525-560).  Outside the torus the atmosphere sits at the ExpX1RhoSie
floors, rho = 1e-6 r^-1.5 and u = rho 1e-3 / r.  Seeded pressure noise:
u *= 1 + jitter (U - 0.5).

All arithmetic runs on the device in torch (state generation, not the hot
path); the geometry (alpha, beta, gamma_ij, sqrt(gamma)) comes from the
library's FMKS tables of each block.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi, states
from .mesh import TiledMesh, split_axis

TORUS_SEED = states.SEED + 5


def lfish(r: float, a: float) -> float:
    """Specific angular momentum of the FM torus with pressure maximum at r."""
    sr = math.sqrt(r)
    num = (a * a - 2.0 * a * sr + r * r) * (
        (-2.0 * a * r * (a * a - 2.0 * a * sr + r * r)) / math.sqrt(2.0 * a * sr + (r - 3.0) * r)
        + ((a + (r - 2.0) * sr) * (r ** 3 + a * a * (2.0 + r))) / math.sqrt(1.0 + 2.0 * a / r ** 1.5 - 3.0 / r))
    den = r ** 3 * math.sqrt(2.0 * a * sr + (r - 3.0) * r) * (a * a + (r - 2.0) * r)
    return num / den


def _lnh_terms(xp, r, sth, cth, a, l):
    DD = r * r - 2.0 * r + a * a
    AA = (r * r + a * a) ** 2 - DD * a * a * sth * sth
    SS = r * r + a * a * cth * cth
    q = 1.0 + 4.0 * l * l * SS * SS * DD / (AA * AA * sth * sth)
    lnh = 0.5 * xp.log((1.0 + xp.sqrt(q)) / (SS * DD / AA)) - 0.5 * xp.sqrt(q) - 2.0 * a * r * l / AA
    return lnh, DD, AA, SS


def log_enthalpy(r, th, a, rin, l):
    """(ln h, u^phi) of the FM solution at Boyer-Lindquist (r, theta)
    (torch tensors); ln h = -1 for r <= r_in, u^phi = 0 where ln h <= 0."""
    import torch

    sth, cth = torch.sin(th), torch.cos(th)
    lnh, DD, AA, SS = _lnh_terms(torch, r, sth, cth, a, l)
    lin, _, _, _ = _lnh_terms(np, np.float64(rin), np.float64(1.0), np.float64(0.0), a, l)
    lnh = lnh - float(lin)
    lnh = torch.where(r > rin, lnh, torch.full_like(lnh, -1.0))
    expm2chi = SS * SS * DD / (AA * AA * sth * sth)
    up1 = torch.sqrt(((-1.0 + torch.sqrt(1.0 + 4.0 * l * l * expm2chi)) / 2.0).clamp(min=0.0))
    uphi = 2.0 * a * r * torch.sqrt(1.0 + up1 * up1) / torch.sqrt(AA * SS * DD) + torch.sqrt(SS / AA) * up1 / sth
    uphi = torch.where(lnh > 0, uphi, torch.zeros_like(uphi))
    return lnh, uphi


def bl_gcov_tphi(r, th, a):
    """g_tt, g_tphi, g_phiphi of the Boyer-Lindquist Kerr metric."""
    import torch

    sth2 = torch.sin(th) ** 2
    SS = r * r + a * a * torch.cos(th) ** 2
    gtt = -(1.0 - 2.0 * r / SS)
    gtp = -2.0 * a * r * sth2 / SS
    gpp = (r * r + a * a + 2.0 * a * a * r * sth2 / SS) * sth2
    return gtt, gtp, gpp


def ucon0(g00, g03, g33, u3):
    """u^0 from u^mu u_mu = -1 with u^1 = u^2 = 0 (the future-directed root)."""
    A, B, Cc = g00, 2.0 * g03 * u3, 1.0 + g33 * u3 * u3
    return (-B - (B * B - 4.0 * A * Cc).clamp(min=0.0).sqrt()) / (2.0 * A)


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


def fill_torus(ctx, p: abi.Params, mesh: TiledMesh, blocks, a: float = 0.9375, rin: float = 6.0, rmax: float = 12.0,
               kappa: float = 1e-2, beta: float = 100.0, jitter: float = 0.04, seed: int = TORUS_SEED, h: float = 0.3):
    """Write the torus primitives into the interior of every block (tables
    filled first), normalise the field, then PrimitiveToConserved (interior),
    the mesh exchange (ghosts) and con2prim (entire)."""
    import torch

    gam = p.gm1 + 1.0
    l = lfish(rmax, a)
    hm1_max = math.exp(float(log_enthalpy(torch.tensor([rmax], dtype=torch.float64),
                                          torch.tensor([0.5 * math.pi], dtype=torch.float64), a, rin, l)[0][0])) - 1.0
    rho_rmax = (hm1_max * (gam - 1.0) / (kappa * gam)) ** (1.0 / (gam - 1.0))
    pmax, bsqmax = 0.0, 0.0
    off = 0
    for b in blocks:
        ctx.GeometryFillFMKS(b)
    for b in blocks:
        dev = b["prim"].device
        n1t, n2t = b.n1t, b.n2t
        ng = b.ng
        x1 = b.xmin[0] - ng * b.dx[0] + (torch.arange(n1t, dtype=torch.float64, device=dev) + 0.5) * b.dx[0]
        x2 = b.xmin[1] - ng * b.dx[1] + (torch.arange(n2t, dtype=torch.float64, device=dev) + 0.5) * b.dx[1]
        X2, X1 = torch.meshgrid(x2.clamp(1e-9, 1.0 - 1e-9), x1, indexing="ij")  # (j, i) over the whole block
        r = torch.exp(X1)
        th = math.pi * X2 + 0.5 * (1.0 - h) * torch.sin(2.0 * math.pi * X2)
        lnh, uphi = log_enthalpy(r, th, a, rin, l)
        inside = lnh > 0.0
        hm1 = torch.where(inside, torch.exp(lnh) - 1.0, torch.zeros_like(lnh))
        rho_t = (hm1 * (gam - 1.0) / (kappa * gam)).clamp(min=0.0) ** (1.0 / (gam - 1.0))
        u_t = kappa * rho_t ** gam / (gam - 1.0) / rho_rmax
        rho_t = rho_t / rho_rmax
        rho_fl = 1e-6 * r ** -1.5
        u_fl = rho_fl * 1e-3 / r
        rho = torch.where(inside, rho_t, rho_fl).clamp(min=0.0)
        rho = torch.maximum(rho, rho_fl)
        u = torch.where(inside, u_t, u_fl)
        u = torch.maximum(u, rho * 1e-3 / r)
        # rotation: u^3 = u^phi (u^r = u^theta = 0), u^0 from the FMKS metric
        cent = b.geom.arrays["cent"]
        alpha, beta1 = cent[abi.G_ALPHA], cent[abi.G_BETA]
        g00, g03, g33 = cent[_gidx(0, 0)], cent[_gidx(0, 3)], cent[_gidx(3, 3)]
        u3 = torch.where(inside, uphi, torch.zeros_like(uphi))
        u0 = ucon0(g00, g03, g33, u3)
        W = alpha * u0
        wv1 = torch.where(inside, W * beta1 / alpha, torch.zeros_like(W))
        wv3 = u3
        # poloidal field from A_phi at corners of the whole block (j, i) -> (j+1, i+1) corners
        rav = torch.zeros((n2t + 1, n1t + 1), dtype=torch.float64, device=dev)
        rav[1:-1, 1:-1] = 0.25 * (rho[1:, 1:] + rho[1:, :-1] + rho[:-1, 1:] + rho[:-1, :-1])
        A = (rav - 0.2).clamp(min=0.0)
        gdet = cent[abi.G_DETGAM]
        B1 = -(A[:-1, :-1] - A[1:, :-1] + A[:-1, 1:] - A[1:, 1:]) / (2.0 * b.dx[1] * gdet)
        B2 = (A[:-1, :-1] + A[1:, :-1] - A[:-1, 1:] - A[1:, 1:]) / (2.0 * b.dx[0] * gdet)
        pr = b["prim"]
        n3t = b.n3t
        rho3 = rho.expand(n3t, n2t, n1t)
        noise = states.uniform_torch(seed, 0, n3t * n2t * n1t, dev, start=off).reshape(n3t, n2t, n1t)
        off += n3t * n2t * n1t
        u3d = u.expand(n3t, n2t, n1t) * (1.0 + jitter * (noise - 0.5))
        pr[abi.PRHO] = rho3
        pr[abi.PVEL] = wv1.expand(n3t, n2t, n1t)
        pr[abi.PVEL + 1] = 0.0
        pr[abi.PVEL + 2] = wv3.expand(n3t, n2t, n1t)
        pr[abi.PENG] = u3d
        pr[abi.PB] = B1.expand(n3t, n2t, n1t)
        pr[abi.PB + 1] = B2.expand(n3t, n2t, n1t)
        pr[abi.PB + 2] = 0.0
        # normalisation maxima over the interior
        ks, js, is_ = b.isl()
        P = (gam - 1.0) * pr[abi.PENG, ks, js, is_]
        pmax = max(pmax, float(P.max()))
        bsqmax = max(bsqmax, float(_bsq(pr, cent)[ks, js, is_].max()))
    fac = math.sqrt((pmax / (0.5 * bsqmax)) / beta) if bsqmax > 0 else 0.0
    for b in blocks:
        pr = b["prim"]
        pr[abi.PB:abi.PB + 3] *= fac
        rho, u = pr[abi.PRHO], pr[abi.PENG]
        T = (u / rho).clamp(min=0.0)
        pr[abi.PPRS] = ((gam - 1.0) * rho * T).clamp(min=0.0)
        pr[abi.PTMP] = T
        pr[abi.PGM1] = ((gam * (gam - 1.0) * rho * T).clamp(min=0.0)) / pr[abi.PPRS]
        pr[abi.PMU] = 0.0
        ctx.PrimitiveToConserved(p, b, *b.interior())
    ctx.MeshExchange(p, mesh, blocks)
    for b in blocks:
        ctx.ConservedToPrimitive(p, b)
        ctx.ApplyFloors(p, b)
    return {"l": l, "rho_rmax": rho_rmax, "beta_pmax_before": pmax / (0.5 * bsqmax) if bsqmax else None,
            "field_factor": fac}


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
