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


def isotropic(seed: int, stream: int, n: int) -> np.ndarray:
    """Unit vectors uniform on the sphere, shape (3, n)."""
    cz = 2.0 * uniform(seed, stream, n) - 1.0
    ph = 2.0 * np.pi * uniform(seed, stream + 1, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - cz * cz))
    return np.stack([s * np.cos(ph), s * np.sin(ph), cz])


def eos_prims(rho, P, gm1, Cv=1.0):
    """u, T, gamma1 from (rho, P) for the ideal gas (singularity-eos IdealGas)."""
    u = P / gm1
    sie = u / rho
    T = np.maximum(0.0, sie / Cv)
    Pt = np.maximum(0.0, gm1 * rho * Cv * T)
    bmod = np.maximum(0.0, (gm1 + 1) * gm1 * rho * Cv * T)
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
                       sigma=(1.0e-3, 10.0)):
    """Per-zone random primitives: log10 rho ~ U, log10 P/rho ~ U, Lorentz
    factor ~ U with isotropic direction, |B|^2/rho log-uniform with isotropic
    direction."""
    rho = 10.0 ** (logrho[0] + (logrho[1] - logrho[0]) * uniform(seed, 0, N))
    P = rho * 10.0 ** (logT[0] + (logT[1] - logT[0]) * uniform(seed, 1, N))
    Wl = W[0] + (W[1] - W[0]) * uniform(seed, 2, N)
    nv = isotropic(seed, 3, N)
    wv = np.sqrt(Wl * Wl - 1.0) * nv
    ls = np.log10(sigma[0]) + (np.log10(sigma[1]) - np.log10(sigma[0])) * uniform(seed, 5, N)
    Bm = np.sqrt(10.0 ** ls * rho)
    nb = isotropic(seed, 6, N)
    return rho, wv, P, Bm * nb


def random_block(n: int, seed: int, ng: int = 4, Gamma: float = 4.0 / 3.0) -> Block:
    """One periodic n^3 block of per-zone random primitives."""
    dx = 1.0 / n
    b = Block((n, n, n), ng, 3, (0.0, 0.0, 0.0), (dx, dx, dx)).alloc()
    rho, wv, P, B = random_zones_prims(n ** 3, seed)
    shp = (n, n, n)
    _set_interior(b, rho.reshape(shp), [w.reshape(shp) for w in wv], P.reshape(shp), [x.reshape(shp) for x in B],
                  Gamma - 1.0)
    return b


def uneven_block_sizes(nblocks: int = 1024, seed: int = SEED + 3, sizes=(16, 32, 64), probs=(0.5, 0.35, 0.15)):
    """Per-block edge lengths drawn from sizes with the given probabilities."""
    u = uniform(seed, 99, nblocks)
    edges = np.cumsum(probs)
    return [int(sizes[int(np.searchsorted(edges, x, side="right"))]) for x in u]
