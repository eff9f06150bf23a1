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
