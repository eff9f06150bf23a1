"""Comparison helpers shared by the parity tests."""
from __future__ import annotations

import math

import numpy as np


def face_region(b, d: int):
    """(k, j, i) slices of the faces the CUDA path computes in direction d
    (0-based): along d [s, e+1], transverse active directions [s-1, e+1]."""
    (i0, i1), (j0, j1), (k0, k1) = b.interior()
    dj = 1 if b.ndim >= 2 else 0
    dk = 1 if b.ndim >= 3 else 0
    if d == 0:
        return slice(k0 - dk, k1 + dk + 1), slice(j0 - dj, j1 + dj + 1), slice(i0, i1 + 2)
    if d == 1:
        return slice(k0 - dk, k1 + dk + 1), slice(j0, j1 + 2), slice(i0 - 1, i1 + 2)
    return slice(k0, k1 + 2), slice(j0 - 1, j1 + 2), slice(i0 - 1, i1 + 2)


def divergence_faces(b, d: int):
    """(k, j, i) slices of the faces FluxDivergence reads in direction d."""
    (i0, i1), (j0, j1), (k0, k1) = b.interior()
    if d == 0:
        return slice(k0, k1 + 1), slice(j0, j1 + 1), slice(i0, i1 + 2)
    if d == 1:
        return slice(k0, k1 + 1), slice(j0, j1 + 2), slice(i0, i1 + 1)
    return slice(k0, k1 + 2), slice(j0, j1 + 1), slice(i0, i1 + 1)


def flux_view(a, d, ncons=8):
    """flux array (24, n3t, n2t, n1t) -> (ncons, ...) of direction d."""
    return a[d * 8:d * 8 + ncons]


def host(a):
    if isinstance(a, np.ndarray):
        return a
    if hasattr(a, "detach"):
        return a.detach().cpu().numpy()
    return np.asarray(a, dtype=np.float64)


def assert_bitwise(got, ref, what=""):
    got, ref = host(got), host(ref)
    same = (got == ref) | (np.isnan(got) & np.isnan(ref))
    if not same.all():
        bad = np.argwhere(~same)
        i0 = tuple(bad[0])
        rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
        raise AssertionError(f"{what}: {bad.shape[0]} of {same.size} values differ; first at {i0}: "
                             f"got {got[i0]!r} ref {ref[i0]!r}; max rel {np.nanmax(rel):.3e}")


def rel_err(got, ref, floor):
    """|got - ref| / (|ref| + floor), elementwise."""
    got, ref = host(got), host(ref)
    return np.abs(got - ref) / (np.abs(ref) + floor)


def assert_close(got, ref, rtol, what="", floor=None):
    """Relative agreement with an absolute floor per variable: the floor is
    rtol x (max |ref| of that variable), so a component that is zero in the
    reference (e.g. the flux of a zero field component) is compared on the
    scale of the variable rather than relative to zero."""
    got, ref = host(got), host(ref)
    if floor is None:
        floor = np.max(np.abs(ref)) if ref.size else 0.0
    err = np.abs(got - ref)
    lim = rtol * (np.abs(ref) + floor)
    bad = ~(err <= lim)
    if bad.any():
        idx = np.argwhere(bad)[0]
        i0 = tuple(idx)
        raise AssertionError(f"{what}: {bad.sum()} of {bad.size} beyond rtol {rtol:g}; first {i0}: got "
                             f"{got[i0]!r} ref {ref[i0]!r}")


def random_rad_block(nx, ndim, seed, vmax=0.4, kappa_s=50.0, kappa_a=5.0, ng=4, hmax=0.6):
    """A host Block with random fluid background (rho, T, u, u^i on the whole
    block) and random radiation primitives J > 0, |H|/J < hmax of one
    species, xi = 0, phi = pi, radiation conserved moments unset."""
    from phoebus_gb300 import abi
    from phoebus_gb300.block import Block
    from phoebus_gb300.radiation import alloc_rad

    rng = np.random.default_rng(seed)
    nxs = tuple(nx[d] if d < ndim else 1 for d in range(3))
    dx = tuple(1.0 / nxs[d] if d < ndim else 1.0 for d in range(3))
    b = Block(nxs, ng=ng, ndim=ndim, xmin=(0.0, 0.0, 0.0), dx=dx, backend="numpy")
    b.alloc(["prim", "cons", "flux", "face_sig", "cell_sig", "fail", "src", "emf", "dudt"])
    alloc_rad(b)
    P, R = b["prim"], b["rprim"]
    shp = b.shape
    P[abi.PRHO] = rng.uniform(0.5, 2.0, shp)
    P[abi.PTMP] = rng.uniform(0.5, 2.0, shp)
    P[abi.PENG] = P[abi.PRHO] * P[abi.PTMP]
    u = rng.uniform(-1, 1, (3,) + shp)
    u *= vmax * rng.uniform(0, 1, shp) / np.maximum(np.sqrt((u * u).sum(0)), 1e-12)
    W = 1 / np.sqrt(1 - (u * u).sum(0))
    for d in range(3):
        P[abi.PVEL + d] = W * u[d] if d < ndim else 0.3 * W * u[d]
    R[abi.RJ] = np.exp(rng.uniform(np.log(1e-3), 0.0, shp))
    h = rng.uniform(-1, 1, (3,) + shp)
    h *= hmax * rng.uniform(0, 1, shp) ** 0.25 / np.maximum(np.sqrt((h * h).sum(0)), 1e-12)
    for d in range(3):
        R[abi.RH + d] = h[d]
    R[abi.RXI] = 0.0
    R[abi.RPHI] = np.pi
    return b


# ---- per-zone comparison with local floors
#
# A production-build value is compared with the oracle's per zone (per face)
# as |got - ref| <= rtol (|ref| + s), where s is the magnitude of the terms
# that form that value at that zone, so a small result of a large local
# cancellation is held to the precision its own inputs carry, and nothing is
# measured against a block-wide maximum.  For an LLF / HLL flux,
# F = (c_r F_l - c_l F_r + c_r c_l (U_r - U_l)) / (c_r - c_l): its terms are
# of size |F_l| + |F_r| + c (|U_l| + |U_r|), and |F| <= (|U| + p_tot) for
# |v| <= 1, so the face scale is (1 + c) (s(L) + s(R)) with the per-cell
# magnitudes s below (the face states are reconstructions bounded by the
# neighbouring cells).  U_r - U_l is a difference of two rounded values, so
# it carries c eps (|U_l| + |U_r|) whatever its size.

def cell_flux_magnitudes(hb):
    """Per-cell magnitude of each conserved variable's flux terms [8][...]:
    D: |D|; S_i: |S| + p + |B|^2 (momentum flux, pressure and Maxwell
    stress); tau: |tau| + |D| + s_S (F_tau = F_E - F_D); B^i: |B| (the
    induction terms B^i v^d - B^d v^i)."""
    U, P = host(hb["cons"]), host(hb["prim"])
    aS = np.abs(U[1]) + np.abs(U[2]) + np.abs(U[3])
    Bp = P[5] * P[5] + P[6] * P[6] + P[7] * P[7]
    sS = aS + np.abs(P[8]) + Bp
    aB = np.abs(U[5]) + np.abs(U[6]) + np.abs(U[7])
    aD = np.abs(U[0])
    return np.stack([aD, sS, sS, sS, np.abs(U[4]) + aD + sS, aB, aB, aB])


def _shift(a, d, k=1):
    """a at the cell k steps lower along direction d (0-based; arrays are
    (..., k3, k2, k1)); wraps at the block edge, which no compared face or
    zone reaches."""
    return np.roll(a, k, axis=a.ndim - 1 - d)


def face_flux_scale(hb, d, mags=None):
    """Local scale [8][...] of the direction-d face fluxes at every face."""
    m = cell_flux_magnitudes(hb) if mags is None else mags
    c = host(hb["face_sig"])[d]
    return (1.0 + np.abs(c)) * (m + _shift(m, d))


def report_close(got, ref, scale, rtol, what="", sl=None):
    """Per-zone check |got - ref| <= rtol (|ref| + scale) (NaN equal NaN);
    returns the largest per-zone ratio |got - ref| / (|ref| + scale), printed
    for the test log."""
    got, ref = host(got), host(ref)
    scale = np.broadcast_to(host(scale), np.shape(ref))  # a scalar floor too
    if sl is not None:
        got, ref, scale = got[sl], ref[sl], scale[sl]
    both_nan = np.isnan(got) & np.isnan(ref)
    err = np.where(both_nan, 0.0, np.abs(got - ref))
    den = np.abs(np.where(both_nan, 1.0, ref)) + scale
    den = np.where(den > 0, den, 1e-300)
    r = err / den
    worst = float(np.nanmax(r)) if r.size else 0.0
    print(f"[per-zone] {what}: max |d| / (|ref| + local scale) = {worst:.3e} (bar {rtol:g})")
    bad = ~(r <= rtol)
    if bad.any():
        i0 = tuple(np.argwhere(bad)[0])
        raise AssertionError(f"{what}: {int(bad.sum())} of {bad.size} beyond {rtol:g} per zone; first {i0}: got "
                             f"{got[i0]!r} ref {ref[i0]!r} scale {scale[i0]!r}")
    return worst


def max_rel(got, ref, sl=None):
    """Largest per-zone |got - ref| / |ref| over zones with ref != 0 (NaN = NaN)."""
    got, ref = host(got), host(ref)
    if sl is not None:
        got, ref = got[sl], ref[sl]
    both_nan = np.isnan(got) & np.isnan(ref)
    nz = (ref != 0) & ~both_nan
    if not nz.any():
        return 0.0
    return float(np.max(np.abs(got[nz] - ref[nz]) / np.abs(ref[nz])))


def prim_floors(hb):
    """Per-zone floors of the primitive comparisons: rho, u, P are positive
    and compared relative to themselves (floor 0); the three-velocity
    components W v^i relative to |W v| plus the zone's largest signal speed
    (a velocity that is zero in exact arithmetic, ahead of a blast wave, is
    measured against the speed at which the zone can change); the field
    components relative to |B|."""
    P, cs = host(hb["prim"]), host(hb["cell_sig"])
    av = np.abs(P[1]) + np.abs(P[2]) + np.abs(P[3])
    c = np.maximum(np.maximum(np.abs(cs[0]), np.abs(cs[1])), np.abs(cs[2]))
    aB = np.abs(P[5]) + np.abs(P[6]) + np.abs(P[7])
    z = np.zeros_like(P[0])
    return {0: z, 1: av + c, 2: av + c, 3: av + c, 4: z, 8: z, 5: aB, 6: aB, 7: aB}


def max_rel_floor(got, ref, floor):
    """Largest per-zone |got - ref| / (|ref| + floor) over zones where the
    denominator is positive (NaN = NaN)."""
    got, ref, floor = host(got), host(ref), host(floor)
    both_nan = np.isnan(got) & np.isnan(ref)
    den = np.abs(ref) + floor
    ok = (den > 0) & ~both_nan
    if not ok.any():
        return 0.0
    return float(np.nanmax(np.abs(got[ok] - ref[ok]) / den[ok]))


def random_rad_block_fmks(nx, ndim, seed, vmax=0.3, hmax=0.6, ng=4, x1=(math.log(4.0), math.log(40.0)),
                          x2=(0.15, 0.85)):
    """random_rad_block on an FMKS block (the torus geometry, a = 0.9375) of
    X1 = ln r in x1, X2 in x2, X3 in [0, 2 pi) with the oracle's tables: the
    fluid's W v^i scaled by 1 / sqrt(gamma_ii) and the radiation's covariant
    H_i / J by sqrt(gamma_ii), so that |v| and xi keep the ranges of the
    Minkowski helper."""
    from oracle.oracle import Oracle
    from phoebus_gb300 import abi, torus
    from phoebus_gb300.block import Block, GeomTables

    b = random_rad_block(nx, ndim, seed, vmax=vmax, hmax=hmax, ng=ng)
    nxs = b.nx
    lo = (x1[0], x2[0], 0.0)
    hi = (x1[1], x2[1], 2 * math.pi)
    dx = tuple((hi[d] - lo[d]) / nxs[d] if d < ndim else (1.0 if d == 1 else 2 * math.pi) for d in range(3))
    fb = Block(b.nx, ng=ng, ndim=ndim, xmin=lo, dx=dx, backend="numpy", arrays=b.arrays)
    fb.geom = GeomTables(torus.torus_geometry(), fb.n1t, fb.n2t, "numpy").alloc()
    Oracle().GeometryFillFMKS(fb)
    cent = fb.geom.arrays["cent"]
    for d in range(3):
        g_dd = cent[abi.G_GCOV + (d + 1) * (d + 2) // 2 + d + 1][None]
        fb["prim"][abi.PVEL + d] /= np.sqrt(g_dd)
        fb["rprim"][abi.RH + d] *= np.sqrt(g_dd)
    return fb
