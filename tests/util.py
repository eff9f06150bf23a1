"""Comparison helpers shared by the parity tests."""
from __future__ import annotations

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
    return a if isinstance(a, np.ndarray) else a.detach().cpu().numpy()


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
