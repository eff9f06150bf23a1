"""Seeded synthetic initial states for the benchmark configurations.

All randomness comes from a counter-based SplitMix64 (one 64-bit hash per
(seed, stream, zone) counter), so a state is a pure function of its seed and
is generated identically for the GPU run and for the CPU oracle.  States are
written as primitives into a host Block (interior and ghosts: ghosts take the
periodic image), ready for PrimitiveToConserved.

Velocities are phoebus primitives, W v^i (normal-observer 3-velocity times the
Lorentz factor); u = P / (Gamma - 1); gamma1 = bulk modulus / P of the ideal
gas, computed as the EOS does.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .block import Block

SEED = 20261203
_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(seed: int, stream: int, idx: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser of the counter (seed, stream, idx) -> uint64."""
    with np.errstate(over="ignore"):
        z = np.uint64((seed * 0x100000001B3 + stream * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF)
        z = z + (idx.astype(np.uint64) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n uniforms in [0, 1) with 53-bit resolution."""
    z = splitmix64(seed, stream, np.arange(n, dtype=np.uint64))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """Box-Muller standard normals."""
    u1 = uniform(seed, stream, n)
    u2 = uniform(seed, stream + 1000, n)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * np.pi * u2)


def _uni(seed: int, stream: int, n: int, device=None):
    """uniform() on the host (device None) or uniform_torch() on a device."""
    return uniform(seed, stream, n) if device is None else uniform_torch(seed, stream, n, device)


def _xp(a):
    if isinstance(a, np.ndarray):
        return np
    import torch

    return torch


def isotropic(seed: int, stream: int, n: int, device=None):
    """Unit vectors uniform on the sphere, shape (3, n)."""
    cz = 2.0 * _uni(seed, stream, n, device) - 1.0
    ph = 2.0 * np.pi * _uni(seed, stream + 1, n, device)
    xp = _xp(cz)
    s = (1.0 - cz * cz).clip(min=0.0) ** 0.5
    return xp.stack([s * xp.cos(ph), s * xp.sin(ph), cz])


def eos_prims(rho, P, gm1, Cv=1.0):
    """u, T, gamma1 from (rho, P) for the ideal gas (singularity-eos IdealGas)."""
    u = P / gm1
    sie = u / rho
    T = (sie / Cv).clip(min=0.0)
    Pt = (gm1 * rho * Cv * T).clip(min=0.0)
    bmod = ((gm1 + 1) * gm1 * rho * Cv * T).clip(min=0.0)
    return u, T, bmod / Pt


def _fill_periodic_ghosts(b: Block, a: np.ndarray):
    """a: (nvar, n3t, n2t, n1t); copy interior periodic images into ghosts."""
    ng = b.ng
    nx1, nx2, nx3 = b.nx
    a[:, :, :, :ng] = a[:, :, :, nx1:nx1 + ng]
    a[:, :, :, ng + nx1:] = a[:, :, :, ng:2 * ng]
    if b.ndim >= 2:
        a[:, :, :ng, :] = a[:, :, nx2:nx2 + ng, :]
        a[:, :, ng + nx2:, :] = a[:, :, ng:2 * ng, :]
    if b.ndim >= 3:
        a[:, :ng, :, :] = a[:, nx3:nx3 + ng, :, :]
        a[:, ng + nx3:, :, :] = a[:, ng:2 * ng, :, :]


def _set_interior(b: Block, rho, wv, P, B, gm1):
    """Write interior prims (arrays shaped like the interior) and periodic ghosts."""
    pr = b.arrays["prim"]
    ks, js, is_ = b.isl()
    u, T, g1 = eos_prims(rho, P, gm1)
    pr[abi.PRHO, ks, js, is_] = rho
    for d in range(3):
        pr[abi.PVEL + d, ks, js, is_] = wv[d]
        pr[abi.PB + d, ks, js, is_] = B[d]
    pr[abi.PENG, ks, js, is_] = u
    pr[abi.PPRS, ks, js, is_] = P
    pr[abi.PGM1, ks, js, is_] = g1
    pr[abi.PTMP, ks, js, is_] = T
    pr[abi.PMU, ks, js, is_] = 0.0
    _fill_periodic_ghosts(b, pr)


def _cell_centres(b: Block):
    nx1, nx2, nx3 = b.nx
    x = b.xmin[0] + (np.arange(nx1) + 0.5) * b.dx[0]
    y = b.xmin[1] + (np.arange(nx2) + 0.5) * b.dx[1]
    z = b.xmin[2] + (np.arange(nx3) + 0.5) * b.dx[2]
    return np.meshgrid(z, y, x, indexing="ij")  # (k, j, i)


def blast_wave(n: int = 64, seed: int = SEED + 1, ng: int = 4) -> tuple[Block, dict]:
    """Special-relativistic MHD blast wave on one n^3 block in [-1, 1]^3:
    rho = 1e-2 (1 + 1e-6 U(-1, 1)), P = 1 inside r < 0.1 and 1e-3 outside,
    v = 0, B = (0.1, 0, 0), Gamma = 4/3."""
    dx = 2.0 / n
    b = Block((n, n, n), ng, 3, (-1.0, -1.0, -1.0), (dx, dx, dx)).alloc()
    Z, Y, X = _cell_centres(b)
    r = np.sqrt(X * X + Y * Y + Z * Z)
    N = n ** 3
    rho = 1.0e-2 * (1.0 + 1.0e-6 * (2.0 * uniform(seed, 0, N) - 1.0)).reshape(r.shape)
    P = np.where(r < 0.1, 1.0, 1.0e-3)
    z0 = np.zeros_like(r)
    _set_interior(b, rho, (z0, z0, z0), P, (0.1 + z0, z0, z0), 4.0 / 3.0 - 1.0)
    par = dict(Gamma=4.0 / 3.0, recon="linear", riemann="llf", cfl=0.3, c2p_tol=1.0e-10, c2p_max_iter=100)
    return b, par


def kelvin_helmholtz(n: int = 256, seed: int = SEED + 2, ng: int = 4) -> tuple[Block, dict]:
    """Shear layer on one n^3 block in [0, 1]^3: v_x = 0.5 tanh((y - 1/2)/0.01),
    rho = 1.5 + 0.5 tanh((y - 1/2)/0.01) (1 below, 2 above), P = 1,
    B = (0.01, 0, 0), Gaussian transverse velocity noise of amplitude 1e-3,
    Gamma = 5/3.  Boundaries are periodic in all three directions."""
    dx = 1.0 / n
    b = Block((n, n, n), ng, 3, (0.0, 0.0, 0.0), (dx, dx, dx)).alloc()
    Z, Y, X = _cell_centres(b)
    N = n ** 3
    t = np.tanh((Y - 0.5) / 0.01)
    vx = 0.5 * t
    vy = 1.0e-3 * normal(seed, 0, N).reshape(t.shape)
    vz = 1.0e-3 * normal(seed, 10, N).reshape(t.shape)
    W = 1.0 / np.sqrt(1.0 - (vx * vx + vy * vy + vz * vz))
    rho = 1.5 + 0.5 * t
    P = np.ones_like(t)
    z0 = np.zeros_like(t)
    _set_interior(b, rho, (W * vx, W * vy, W * vz), P, (0.01 + z0, z0, z0), 5.0 / 3.0 - 1.0)
    par = dict(Gamma=5.0 / 3.0, recon="weno5z", riemann="hll", cfl=0.4, c2p_tol=1.0e-10, c2p_max_iter=100)
    return b, par


def random_zones_prims(N: int, seed: int, logrho=(-4.0, 0.0), logT=(-3.0, 0.0), W=(1.0, 5.0),
                       sigma=(1.0e-3, 10.0), device=None):
    """Per-zone random primitives: log10 rho ~ U, log10 P/rho ~ U, Lorentz
    factor ~ U with isotropic direction, |B|^2/rho log-uniform with isotropic
    direction.  device None draws with numpy, else on that torch device."""
    rho = 10.0 ** (logrho[0] + (logrho[1] - logrho[0]) * _uni(seed, 0, N, device))
    P = rho * 10.0 ** (logT[0] + (logT[1] - logT[0]) * _uni(seed, 1, N, device))
    Wl = W[0] + (W[1] - W[0]) * _uni(seed, 2, N, device)
    nv = isotropic(seed, 3, N, device)
    wv = (Wl * Wl - 1.0) ** 0.5 * nv
    ls = np.log10(sigma[0]) + (np.log10(sigma[1]) - np.log10(sigma[0])) * _uni(seed, 5, N, device)
    Bm = (10.0 ** ls * rho) ** 0.5
    nb = isotropic(seed, 6, N, device)
    return rho, wv, P, Bm * nb


def random_block(n: int, seed: int, ng: int = 4, Gamma: float = 4.0 / 3.0, device=None) -> Block:
    """One periodic n^3 block of per-zone random primitives (host arrays, or
    arrays on a torch device drawn there)."""
    dx = 1.0 / n
    if device is None:
        b = Block((n, n, n), ng, 3, (0.0, 0.0, 0.0), (dx, dx, dx)).alloc()
    else:
        b = Block((n, n, n), ng, 3, (0.0, 0.0, 0.0), (dx, dx, dx), backend="torch", device=device).alloc()
    rho, wv, P, B = random_zones_prims(n ** 3, seed, device=device)
    shp = (n, n, n)
    _set_interior(b, rho.reshape(shp), [w.reshape(shp) for w in wv], P.reshape(shp), [x.reshape(shp) for x in B],
                  Gamma - 1.0)
    return b


def uneven_blocks(nblocks: int = 1024, seed: int = SEED + 3, device="cuda", Gamma: float = 4.0 / 3.0):
    """The batched-meshblock state: nblocks periodic blocks with edges drawn
    by uneven_block_sizes and per-zone random primitives, drawn in one pass
    over all interior zones (block b's zones follow block b-1's in the
    counter order) on the device (or the host for device None)."""
    sizes = uneven_block_sizes(nblocks, seed)
    total = sum(n ** 3 for n in sizes)
    rho, wv, P, B = random_zones_prims(total, seed + 7, device=device)
    blocks, off = [], 0
    for n in sizes:
        dx = 1.0 / n
        kw = {} if device is None else dict(backend="torch", device=device)
        b = Block((n, n, n), 4, 3, (0.0, 0.0, 0.0), (dx, dx, dx), **kw).alloc()
        sl = slice(off, off + n ** 3)
        shp = (n, n, n)
        _set_interior(b, rho[sl].reshape(shp), [w[sl].reshape(shp) for w in wv], P[sl].reshape(shp),
                      [x[sl].reshape(shp) for x in B], Gamma - 1.0)
        blocks.append(b)
        off += n ** 3
    return blocks


def uneven_block_sizes(nblocks: int = 1024, seed: int = SEED + 3, sizes=(16, 32, 64), probs=(0.5, 0.35, 0.15)):
    """Per-block edge lengths drawn from sizes with the given probabilities."""
    u = uniform(seed, 99, nblocks)
    edges = np.cumsum(probs)
    return [int(sizes[int(np.searchsorted(edges, x, side="right"))]) for x in u]


def linear_modes_2d(n: int = 64, ng: int = 4, amp: float = 1.0e-5, gam: float = 1.333333333333333333):
    """Problem generator linear_modes (pgen/linear_modes.cpp:21-307) for the
    2D hydro sound mode on [0, 1]^2 (the regression deck inputs/linear_modes.pin
    with nx = 64, fluid/mhd = true, hydro_modes/physics = hydro): primitives set
    on the entire block from the analytic mode at each cell's own coordinates
    (ghosts included, as the reference does).  Returns (block, params, tlim)
    with tlim = one wave period, which the generator writes over parthenon/time/tlim."""
    kk = 2.0 * np.pi
    omega_im = 3.8780661653218766
    drho, dug, du1, du2 = 0.5804294924639213, 0.7739059899518947, 0.1791244302079596, 0.1791244302079596
    dx = 1.0 / n
    b = Block((n, n, 1), ng, 2, (0.0, 0.0, -1.0), (dx, dx, 2.0)).alloc()
    x0 = 0.0 - ng * dx
    xs = x0 + (np.arange(b.n1t) + 0.5) * dx
    ys = x0 + (np.arange(b.n2t) + 0.5) * dx
    Y, X = np.meshgrid(ys, xs, indexing="ij")
    # the C library's cos (as the reference's std::cos), not numpy's vectorised one
    arg = kk * X + kk * Y
    mode = amp * np.array([math.cos(a) for a in arg.ravel()]).reshape(arg.shape)
    rho = 1.0 + drho * mode
    ug = 1.0 + dug * mode
    gm1 = gam - 1.0
    Pg = (gam - 1.0) * ug
    T = np.maximum(0.0, (ug / rho) / 1.0)
    bmod = np.maximum(0.0, (gm1 + 1) * gm1 * rho * 1.0 * T)
    pr = b.arrays["prim"]
    pr[abi.PRHO, 0] = rho
    pr[abi.PENG, 0] = ug
    pr[abi.PPRS, 0] = Pg
    pr[abi.PTMP, 0] = T
    pr[abi.PGM1, 0] = bmod / Pg
    pr[abi.PVEL, 0] = 0.0 + du1 * mode
    pr[abi.PVEL + 1, 0] = 0.0 + du2 * mode
    pr[abi.PVEL + 2, 0] = 0.0
    pr[abi.PB:abi.PB + 3, 0] = 0.0
    par = dict(Gamma=gam, recon="linear", riemann="hll", cfl=0.4, c2p_tol=1.0e-12, c2p_max_iter=100, mhd=1)
    tlim = 2.0 * np.pi / omega_im
    return b, par, tlim


class TimeControl:
    """PhoebusDriver::Step (phoebus_driver.cpp:121-143) and Parthenon's
    EvolutionDriver timestep control: dt_0 from the cell-speed estimate after
    initialisation; the first step uses dt_init_fact * dt; afterwards the new
    estimate (growth_cap = True also limits growth to 2x per step, a variant of
    the driver the reference's linear-modes gold does not match); every step
    is clipped to end at tlim."""

    def __init__(self, tlim: float, dt0: float, dt_init_fact: float = 1.0, growth_cap: bool = False):
        self.tlim, self.time, self.ncycle = tlim, 0.0, 0
        self.dt_init_fact = dt_init_fact
        self.growth_cap = growth_cap
        big = np.finfo(np.float64).max
        self.dt = min(big, dt0)
        if self.time < self.tlim and (self.tlim - self.time) < self.dt:
            self.dt = self.tlim - self.time

    def keep_going(self):
        return self.time < self.tlim

    def begin_step(self) -> float:
        dt = min(self.dt, 1.0e300)
        dt *= self.dt_init_fact
        self.dt_init_fact = 1.0
        if self.time + dt > self.tlim:
            dt = self.tlim - self.time
        self.dt = dt
        return dt

    def end_step(self, new_dt: float):
        self.ncycle += 1
        self.time += self.dt
        if self.growth_cap and self.dt < 0.1 * np.finfo(np.float64).max:
            self.dt *= 2.0
            self.dt = min(self.dt, new_dt)
        else:
            self.dt = new_dt
        if self.time < self.tlim and (self.tlim - self.time) < self.dt:
            self.dt = self.tlim - self.time


def p2c2p_fmks(n: int = 512, ng: int = 4):
    """Problem generator p2c2p (pgen/p2c2p.cpp:21-136) on its deck
    inputs/p2c2p.pin: a 1D FMKS block, X1 in [1, 2] (r in [e, e^2]), one X2
    zone on [-1, 1], a = 0.9375, derefine_poles = false, Gamma = 5/3, MHD.
    Primitives are smooth functions of X1 set on the entire block.  Returns
    (block with FMKS parameters, params, analytic functions)."""
    from .block import GeomTables

    dx = 1.0 / n
    b = Block((n, 1, 1), ng, 1, (1.0, -1.0, -1.0), (dx, 2.0, 2.0)).alloc()
    g = abi.default_geometry(abi.GEOM_FMKS, a=0.9375, derefine_poles=0, x0=min(1.0, max(0.0, 1.0 - ng * dx)))
    b.geom = GeomTables(g, b.n1t, b.n2t).alloc()
    x = (1.0 - ng * dx) + (np.arange(b.n1t) + 0.5) * dx
    f = {
        "rho": lambda x: 1.0 + 0.3 * np.sin(x), "u": lambda x: 1.0 + 0.3 * np.cos(x),
        "v1": lambda x: 0.5 + 0.2 * np.sin(x - 0.3), "v2": lambda x: 0.3 + 0.2 * np.cos(x - 0.2),
        "v3": lambda x: 0.4 + 0.3 * np.sin(x + 0.1), "b1": lambda x: 0.3 + 0.1 * np.sin(x),
        "b2": lambda x: 0.4 + 0.2 * np.cos(x), "b3": lambda x: 0.5 + 0.3 * np.sin(x - 0.1),
    }
    gm1 = 5.0 / 3.0 - 1.0
    pr = b.arrays["prim"]
    rho, u = f["rho"](x), f["u"](x)
    pr[abi.PRHO, 0, 0] = rho
    pr[abi.PENG, 0, 0] = u
    for d, k in enumerate(("v1", "v2", "v3")):
        pr[abi.PVEL + d, 0, 0] = f[k](x)
    for d, k in enumerate(("b1", "b2", "b3")):
        pr[abi.PB + d, 0, 0] = f[k](x)
    sie = u / rho
    P = np.maximum(0.0, gm1 * rho * sie)
    T = np.maximum(0.0, sie / 1.0)
    pr[abi.PPRS, 0, 0] = P
    pr[abi.PTMP, 0, 0] = T
    pr[abi.PGM1, 0, 0] = np.maximum(0.0, (gm1 + 1) * gm1 * rho * 1.0 * T) / P
    par = dict(Gamma=5.0 / 3.0, recon="weno5z", riemann="hll", cfl=0.8, c2p_tol=1.0e-14, c2p_max_iter=100, mhd=1)
    return b, par, f, x


def bondi_1d(n: int = 128, ng: int = 4):
    """The Bondi regression deck (inputs/bondi.pin with tst/regression/bondi.py's
    nx1 = 128): one 1D FMKS block, X1 in [0.59, 5], one X2 zone on [0, 1]
    (theta = pi/2), a = 0, derefine_poles = false, x0 from fmks.cpp:72-81,
    hydro only, Gamma 1.4, Cv 2.5, PLM + LLF, cfl 0.8, c2p_tol 1e-8, 100
    iterations, gr_outflow in X1 with bc_vars = conserved, t_lim 100,
    dt_init_fact 1e-6.  Returns (host block with FMKS parameters and table
    storage, params, t_lim); fill the tables, then call bondi_fill."""
    from .block import GeomTables

    x1min, x1max = 0.59, 5.0
    dx = (x1max - x1min) / n
    b = Block((n, 1, 1), ng, 1, (x1min, 0.0, 0.0), (dx, 1.0, 6.28318530718)).alloc()
    g = abi.default_geometry(abi.GEOM_FMKS, a=0.0, derefine_poles=0, x0=min(x1min, max(0.0, x1min - ng * dx)))
    b.geom = GeomTables(g, b.n1t, b.n2t).alloc()
    par = dict(Gamma=1.4, Cv=2.5, recon="linear", riemann="llf", cfl=0.8, c2p_tol=1.0e-8, c2p_max_iter=100, mhd=0)
    return b, par, 100.0


def bondi_mesh(n: int = 128):
    """The Bondi deck's one-block 1D mesh: gr_outflow on both X1 faces
    (reflect in X2 and periodic in X3 are inactive in 1D), bc_vars =
    conserved (the default; bondi.pin sets none)."""
    from .mesh import TiledMesh

    return TiledMesh((n, 1, 1), [[n], [1], [1]], (0.59, 0.0, 0.0), (5.0, 1.0, 6.28318530718),
                     (abi.BC_OUTFLOW, abi.BC_REFLECT, abi.BC_PERIODIC), (abi.BC_OUTFLOW, abi.BC_REFLECT, abi.BC_PERIODIC),
                     bc_vars=abi.BC_VARS_CONSERVED, ndim=1)


def _bondi_temp(r, n, C1, C2, Tc, rc):
    """pgen/bondi.cpp:24-69: bisection for T(r) between the two roots."""
    rtol, ftol = 1.0e-12, 1.0e-14
    Tguess = Tc * (rc / r) ** 0.8
    T0, T1 = (0.1 * Tguess, Tguess) if r < rc else (Tguess, 10.0 * Tguess)

    def f(T):
        return (1.0 + (1.0 + n) * T) ** 2.0 * (1.0 - 2.0 / r + (C1 / (r * r * T ** n)) ** 2.0) - C2

    f0, f1 = f(T0), f(T1)
    if f0 * f1 > 0.0:
        raise RuntimeError(f"Bondi setup failed at r = {r}")
    Th = 0.5 * (T0 + T1)
    fh = f(Th)
    while (T1 - T0) / Th > rtol and abs(fh) > ftol:
        if fh * f0 < 0.0:
            T1, f1 = Th, fh
        else:
            T0, f0 = Th, fh
        Th = 0.5 * (T0 + T1)
        fh = f(Th)
    return Th


def bondi_fill(b: Block, mdot: float = 1.0, rs: float = 8.0, Rhor: float = 2.0, gam: float = 1.4):
    """Problem generator bondi (pgen/bondi.cpp:97-228) on the entire block:
    Michel's accretion solution in Boyer-Lindquist, moved to FMKS and
    renormalised with the block's own metric tables (which must be filled).
    Sets the primitives; conserved variables come from PrimitiveToConserved."""
    geo = b.geom.params
    tab = b.geom.arrays["cent"]
    tab = tab if isinstance(tab, np.ndarray) else tab.detach().cpu().numpy()
    n = 1.0 / (gam - 1.0)
    Cv = n
    uc = math.sqrt(1.0 / (2.0 * rs))
    Vc = -math.sqrt(uc ** 2 / (1.0 - 3.0 * uc ** 2))
    Tc = -n * Vc ** 2 / ((n + 1.0) * (n * Vc ** 2 - 1.0))
    C1 = uc * rs ** 2 * Tc ** n
    C2 = (1.0 + (1.0 + n) * Tc) ** 2 * (1.0 - 2.0 / rs + C1 ** 2 / (rs ** 4 * Tc ** (2 * n)))
    h = geo.hslope
    pr = b.arrays["prim"]
    x0 = b.xmin[0] - b.ng * b.dx[0]
    x2 = b.xmin[1] + 0.5 * b.dx[1]
    for i in range(b.n1t):
        x1 = x0 + (i + 0.5) * b.dx[0]
        r = math.exp(x1)
        while r < Rhor:
            x1 += b.dx[0]
            r = math.exp(x1)
        T = _bondi_temp(r, n, C1, C2, Tc, rs)
        rho = T ** n
        u = rho * T / (gam - 1.0)
        P = (gam - 1.0) * rho * (u / rho)
        bmod = gam * (gam - 1.0) * rho * Cv * T
        ucon_bl = [0.0, -C1 / (T ** n * r ** 2), 0.0, 0.0]
        th = math.pi * x2 + ((1.0 - h) / 2.0) * math.sin(2.0 * math.pi * x2)  # derefine_poles = false
        # Schwarzschild (a = 0) Boyer-Lindquist metric at (r, th)
        gtt, grr = -(1.0 - 2.0 / r), 1.0 / (1.0 - 2.0 / r)
        AA, BB = gtt, 0.0
        CC = 1.0 + grr * ucon_bl[1] * ucon_bl[1]
        ucon_bl[0] = (-BB - math.sqrt(BB * BB - 4.0 * AA * CC)) / (2.0 * AA)
        # BL -> KS (a = 0), then KS -> FMKS: dX1/dr = 1/r, dX2/dth = 1/(dth/dX2), phi unchanged
        idenom = 1.0 / (r * r - 2.0 * r)
        uks = [ucon_bl[0] + 2.0 * r * idenom * ucon_bl[1], ucon_bl[1], ucon_bl[2], ucon_bl[3]]
        dth = math.pi * (1.0 + (1.0 - h) * math.cos(2.0 * math.pi * x2))
        ucon = [uks[0], uks[1] / r, uks[2] / dth, uks[3]]
        # renormalise with the cell's own metric
        t = tab[:, 0, i]
        def gc(m, q):
            hi, lo = max(m, q), min(m, q)
            return t[abi.G_GCOV + hi * (hi + 1) // 2 + lo]
        AA = gc(0, 0)
        BB = 2.0 * (gc(0, 1) * ucon[1] + gc(0, 2) * ucon[2] + gc(0, 3) * ucon[3])
        CC = (1.0 + gc(1, 1) * ucon[1] * ucon[1] + gc(2, 2) * ucon[2] * ucon[2] + gc(3, 3) * ucon[3] * ucon[3] +
              2.0 * (gc(1, 2) * ucon[1] * ucon[2] + gc(1, 3) * ucon[1] * ucon[3] + gc(2, 3) * ucon[2] * ucon[3]))
        discr = BB * BB - 4.0 * AA * CC
        assert discr > 0, "discr < 0"
        ucon[0] = (-BB - math.sqrt(discr)) / (2.0 * AA)
        lapse = t[abi.G_ALPHA]
        W = lapse * ucon[0]
        pr[abi.PRHO, 0, 0, i] = rho
        pr[abi.PENG, 0, 0, i] = u
        pr[abi.PPRS, 0, 0, i] = P
        pr[abi.PTMP, 0, 0, i] = T
        pr[abi.PGM1, 0, 0, i] = bmod / P
        for d in range(3):
            pr[abi.PVEL + d, 0, 0, i] = ucon[d + 1] + W * t[abi.G_BETA + d] / lapse
        pr[abi.PMU, 0, 0, i] = 0.0


def fmks_random_block(nx=(12, 10, 4), seed: int = SEED + 5, ng: int = 4, r=(2.0, 20.0), x2=(0.1, 0.9),
                      a: float = 0.9375, derefine_poles: int = 1, Gamma: float = 4.0 / 3.0):
    """A block of FMKS coordinates (X1 = ln r, X2 in (0, 1), X3 = phi) holding
    per-zone random primitives, with FMKS table storage attached."""
    from .block import GeomTables

    n1, n2, n3 = nx
    x1min, x1max = np.log(r[0]), np.log(r[1])
    dx = ((x1max - x1min) / n1, (x2[1] - x2[0]) / n2, 2.0 * np.pi / n3)
    b = Block(nx, ng, 3, (x1min, x2[0], 0.0), dx).alloc()
    g = abi.default_geometry(abi.GEOM_FMKS, a=a, derefine_poles=derefine_poles, x0=x1min - ng * dx[0])
    b.geom = GeomTables(g, b.n1t, b.n2t).alloc()
    N = n1 * n2 * n3
    rho, wv, P, B = random_zones_prims(N, seed, W=(1.0, 3.0), sigma=(1e-3, 1.0))
    shp = (n3, n2, n1)
    _set_interior(b, rho.reshape(shp), [w.reshape(shp) for w in wv], P.reshape(shp), [x.reshape(shp) for x in B],
                  Gamma - 1.0)
    return b


def uniform_torch(seed: int, stream: int, n: int, device, start: int = 0):
    """uniform() on the GPU: the same SplitMix64 counters in int64 arithmetic
    (wrapping multiplies, logical shifts by masking), bit-identical draws."""
    import torch

    def srl(z, k):
        return (z >> k) & ((1 << (64 - k)) - 1)

    def s64(v):
        v &= 0xFFFFFFFFFFFFFFFF
        return v - (1 << 64) if v >= (1 << 63) else v

    z0 = s64(seed * 0x100000001B3 + stream * 0x9E3779B97F4A7C15)
    idx = torch.arange(start + 1, start + n + 1, dtype=torch.int64, device=device)
    z = z0 + idx * s64(0x9E3779B97F4A7C15)
    z = (z ^ srl(z, 30)) * s64(0xBF58476D1CE4E5B9)
    z = (z ^ srl(z, 27)) * s64(0x94D049BB133111EB)
    z = z ^ srl(z, 31)
    return srl(z, 11).to(torch.float64) * (1.0 / 9007199254740992.0)


def theta_to_x2(theta, h: float = 0.3, iters: int = 50):
    """Invert th = pi X2 + (1 - h)/2 sin(2 pi X2) (FMKS without derefined
    poles, mckinney_gammie_ryan.hpp thG_) for X2 in (0, 1) by Newton
    iteration; numpy or torch arrays."""
    xp = np if isinstance(theta, np.ndarray) else __import__("torch")
    x = theta / np.pi
    for _ in range(iters):
        f = np.pi * x + 0.5 * (1.0 - h) * xp.sin(2.0 * np.pi * x) - theta
        df = np.pi + np.pi * (1.0 - h) * xp.cos(2.0 * np.pi * x)
        x = x - f / df
    return x


KERR_SPIN = 0.9375


def kerr_zones(n: int, seed: int = SEED + 4, device=None, Gamma: float = 4.0 / 3.0, r=(1.5, 50.0),
               logrho=(-6.0, 0.0), logsie=(-4.0, 1.0), W=(1.0, 10.0), logsigma=(-4.0, 2.0), start: int = 0):
    """Independent zones for con2prim in FMKS Kerr-Schild geometry (derefined
    poles off): r ~ U[1.5, 50], theta ~ U(0, pi), log10 rho ~ U[-6, 0],
    log10 u/rho ~ U[-4, 1], Lorentz factor W ~ U[1, 10], magnetisation
    sigma = b^2/rho log-uniform in [1e-4, 1e2], velocity and field directions
    uniform on the sphere.  device=None draws with numpy, else on that torch
    device (the same SplitMix64 draws).  start offsets the zone counter, so a
    large set can be drawn in pieces.  Returns the FMKS coordinates x1 = ln r,
    x2 and the per-zone scalars; kerr_zone_prims maps them to primitives once
    the point metric is known."""
    if device is None:
        U = lambda k: uniform(seed, k, start + n)[start:]  # noqa: E731
        xp = np
    else:
        import torch

        U = lambda k: uniform_torch(seed, k, n, device, start)  # noqa: E731
        xp = torch
    rr = r[0] + (r[1] - r[0]) * U(0)
    th = np.pi * (1e-6 + (1.0 - 2e-6) * U(1))

    def iso(k):
        cz = 2.0 * U(k) - 1.0
        ph = 2.0 * np.pi * U(k + 1)
        sn = (1.0 - cz * cz).clip(min=0.0) ** 0.5
        return [sn * xp.cos(ph), sn * xp.sin(ph), cz]

    return dict(x1=xp.log(rr), x2=theta_to_x2(th),
                rho=10.0 ** (logrho[0] + (logrho[1] - logrho[0]) * U(2)),
                sie=10.0 ** (logsie[0] + (logsie[1] - logsie[0]) * U(3)),
                W=W[0] + (W[1] - W[0]) * U(4), nv=iso(5),
                sigma=10.0 ** (logsigma[0] + (logsigma[1] - logsigma[0]) * U(7)), nb=iso(8),
                gm1=Gamma - 1.0)


def kerr_zone_prims(z: dict, geom):
    """Primitives [12][n] of kerr_zones given the point geometry
    geom[21][n] (numpy or torch).  A direction n is normalised with the
    spatial metric, so gamma_ij v^i v^j = (W^2 - 1) / W^2 exactly as sampled;
    |B| is chosen so that b^2 = B^2 / W^2 + (B.v)^2 equals sigma rho.  The
    ideal-gas P, T and gamma1 follow the EOS; c2p_mu starts at 0."""
    gam = [[geom[abi.G_GCOV + _flat2(m + 1, k + 1)] for k in range(3)] for m in range(3)]

    def dot(a, b):
        return sum(gam[m][k] * a[m] * b[k] for m in range(3) for k in range(3))

    nv, nb = z["nv"], z["nb"]
    inv = dot(nv, nv) ** -0.5
    W = z["W"]
    vmag = (W * W - 1.0) ** 0.5 / W
    v = [vmag * inv * nv[m] for m in range(3)]
    inb = dot(nb, nb) ** -0.5
    bh = [inb * nb[m] for m in range(3)]
    bv = dot(bh, v)
    rho, sie, gm1 = z["rho"], z["sie"], z["gm1"]
    Bmag = (z["sigma"] * rho / (1.0 / (W * W) + bv * bv)) ** 0.5
    u = rho * sie
    T = sie.clip(min=0.0)
    Pt = (gm1 * rho * T).clip(min=0.0)
    bmod = ((gm1 + 1.0) * gm1 * rho * T).clip(min=0.0)
    zero = rho * 0.0
    rows = [rho, W * v[0], W * v[1], W * v[2], u, Bmag * bh[0], Bmag * bh[1], Bmag * bh[2], Pt, bmod / Pt, T, zero]
    if isinstance(rho, np.ndarray):
        return np.stack(rows)
    import torch

    return torch.stack(rows)


def _flat2(m: int, n: int) -> int:
    lo, hi = min(m, n), max(m, n)
    return hi * (hi + 1) // 2 + lo
