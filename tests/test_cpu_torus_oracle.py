"""The oracle's restatement of the torus problem generator (pgen/torus.cpp)
against the properties the reference states for its own output: the
Fishbone-Moncrief density is normalised to 1 at the pressure maximum
(GetStateFromEnthalpy with rho_rmax), the atmosphere sits at the ExpX1RhoSie
floors, the HARM-style normalisation leaves max P / max (b^2 / 2) = target
beta over the interior (the reference prints it after normalisation,
torus.cpp:740-745), the field is poloidal (B^3 = 0), and the fluid rotates
(W v^3 > 0 inside the torus).  CPU only: host blocks, the oracle's tables."""
import math

import numpy as np
import pytest

from phoebus_gb300 import abi, torus


@pytest.fixture(scope="module")
def torus_state(built):
    from oracle.oracle import Oracle

    orc = Oracle()
    p = torus.torus_params()
    mesh = torus.torus_mesh(n=32, lo=8, hi=16)
    blocks = mesh.make_blocks(geometry=torus.torus_geometry(), backend="numpy")
    for b in blocks:
        orc.GeometryFillFMKS(b)
    tp = torus.torus_problem()
    fac = orc.TorusInit(p, tp, blocks)
    return orc, p, tp, mesh, blocks, fac


def _interior(b, a):
    return a[(slice(None),) + b.isl()] if a.ndim == 4 else a[b.isl()]


def test_torus_density_and_atmosphere(torus_state):
    orc, p, tp, mesh, blocks, fac = torus_state
    rho_max, inside = 0.0, 0
    for b in blocks:
        pr = b["prim"]
        x1 = b.xmin[0] - b.ng * b.dx[0] + (np.arange(b.n1t) + 0.5) * b.dx[0]
        r = np.exp(x1)[None, None, :]
        rho_fl = 1e-6 * r ** -1.5
        rho = pr[abi.PRHO]
        assert np.all(rho >= rho_fl * (1 - 1e-12))
        torus_zone = rho > 1.5 * rho_fl
        inside += int(_interior(b, torus_zone).sum())
        rho_max = max(rho_max, float(_interior(b, rho).max()))
        # atmosphere: rho and u exactly at the floors (u = rho 1e-3 / r)
        atm = ~torus_zone
        assert np.allclose(rho[atm], np.broadcast_to(rho_fl, rho.shape)[atm], rtol=1e-14)
        u_fl = rho * 1e-3 / r
        assert np.all(pr[abi.PENG][atm] >= u_fl[atm] * (1 - 1e-12))
        assert np.all(pr[abi.PB + 2] == 0.0)
        v3 = pr[abi.PVEL + 2]
        assert np.all(v3[torus_zone] > 0)
    assert inside > 100
    assert 0.5 < rho_max <= 1.0 + 1e-12


def test_torus_field_normalisation(torus_state):
    """After the normalisation, max P / max (b^2 / 2) over the interior of
    all blocks is the target beta (b^2 scales as the factor squared)."""
    orc, p, tp, mesh, blocks, fac = torus_state
    assert fac > 0
    pmax, bsqmax = 0.0, 0.0
    for b in blocks:
        pr = b["prim"]
        cent = b.geom.arrays["cent"]
        g = lambda m, n: cent[abi.G_GCOV + {(1, 1): 2, (1, 2): 4, (1, 3): 7, (2, 2): 5, (2, 3): 8, (3, 3): 9}[  # noqa: E731
            (min(m, n), max(m, n))]][None]
        vp = [pr[abi.PVEL + d] for d in range(3)]
        Bp = [pr[abi.PB + d] for d in range(3)]
        W = np.sqrt(1 + sum(g(m + 1, n + 1) * vp[m] * vp[n] for m in range(3) for n in range(3)))
        Bsq = sum(g(m + 1, n + 1) * Bp[m] * Bp[n] for m in range(3) for n in range(3))
        Bdv = sum(g(m + 1, n + 1) * vp[m] / W * Bp[n] for m in range(3) for n in range(3))
        bsq = Bsq / (W * W) + Bdv * Bdv
        pmax = max(pmax, float(_interior(b, pr[abi.PPRS]).max()))
        bsqmax = max(bsqmax, float(_interior(b, bsq).max()))
    beta = pmax / (0.5 * bsqmax)
    assert math.isclose(beta, tp.target_beta, rel_tol=1e-10), beta
