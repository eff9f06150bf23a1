"""Pin the oracle to the reference's own tests and invariants (CPU only).

- linear_modes.gold (tst/regression/linear_modes.py): the whole 2D run of the
  regression deck, compared like regression_test.py:347-391 (p.density then
  p.velocity, flattened, every 10th value, soft_equiv at tol 1e-3).
- pgen/p2c2p.cpp: 100 prim -> con -> prim round trips on the FMKS deck; the
  reference prints the errors, the test bounds them.
- invariants: reconstruction reproduces constants, a uniform state has zero
  flux divergence, Minkowski sources are exactly zero.
"""
from pathlib import Path

import numpy as np
import pytest

from phoebus_gb300 import abi, states

GOLD = Path(__file__).resolve().parent / "golden"


def soft_equiv(val, ref, tol):
    """regression_test.py:48-55."""
    return np.abs(val - ref) / np.maximum(np.abs(ref), 1.0e-10) <= tol


def run_linear_modes(o, growth_cap=False):
    hb, par, tlim = states.linear_modes_2d()
    p = abi.default_params(**par)
    o.Initialize(p, hb)
    tc = states.TimeControl(tlim, o.EstimateTimestepBlock(p, hb, False), dt_init_fact=0.1, growth_cap=growth_cap)
    cs = np.zeros_like(hb["cons"])
    while tc.keep_going():
        dt = tc.begin_step()
        o.rk2_step(p, hb, cs, dt)
        tc.end_step(o.EstimateTimestepBlock(p, hb, True))
    ks, js, is_ = hb.isl()
    pr = hb["prim"]
    vals = np.concatenate([pr[abi.PRHO][ks, js, is_].ravel()] + [pr[abi.PVEL + d][ks, js, is_].ravel() for d in range(3)])
    comp = np.array([vals[10 * n] for n in range(len(vals) // 10)])
    return comp, tc


def test_linear_modes_gold(oracle):
    gold = np.loadtxt(GOLD / "linear_modes.gold")
    comp, tc = run_linear_modes(oracle)
    assert len(comp) == len(gold) == 1638
    assert abs(tc.time - 2.0 * np.pi / 3.8780661653218766) < 1e-14
    ok = soft_equiv(comp, gold, 1.0e-3)
    assert ok.all(), f"{(~ok).sum()} values outside the gold tolerance"
    # density (the 410 first values) agrees far inside the tolerance
    assert np.max(np.abs(comp[:410] - gold[:410]) / np.abs(gold[:410])) < 1e-7


def run_bondi(o, b=None):
    """The Bondi regression run on the oracle: pgen, initialisation, RK2 steps
    to t = 100 with the gr_outflow (bc_vars = conserved) exchange of the
    mesh oracle.  b: a host block from states.bondi_1d with tables filled
    (default: tables from the oracle)."""
    from oracle.mesh_oracle import mesh_exchange

    if b is None:
        b, _, _ = states.bondi_1d()
        o.GeometryFillFMKS(b)
    _, par, tlim = states.bondi_1d()
    states.bondi_fill(b)
    p = abi.default_params(**par)
    mesh = states.bondi_mesh()

    def ex(blk):
        mesh_exchange(o, p, mesh, [blk])

    o.Initialize(p, b, ex)
    tc = states.TimeControl(tlim, o.EstimateTimestepBlock(p, b, False), dt_init_fact=1.0e-6)
    cs = np.zeros_like(b["cons"])
    dts = []
    while tc.keep_going():
        dt = tc.begin_step()
        dts.append(dt)
        o.rk2_step(p, b, cs, dt, ex)
        tc.end_step(o.EstimateTimestepBlock(p, b, True))
    return b, tc, dts


def bondi_values(b):
    ks, js, is_ = b.isl()
    pr = b["prim"]
    return np.concatenate([pr[abi.PRHO][ks, js, is_].ravel()] + [pr[abi.PVEL + d][ks, js, is_].ravel() for d in range(3)])


def test_bondi_gold(oracle):
    """tst/regression/bondi.gold: the 128-zone FMKS hydro Bondi run (PLM +
    LLF, geometric sources, gr_outflow with densitised conserved copies) at
    t = 100 agrees with the reference's final state far inside its 1e-5
    tolerance."""
    gold = np.loadtxt(GOLD / "bondi.gold")
    b, tc, _ = run_bondi(oracle)
    comp = bondi_values(b)
    assert len(comp) == len(gold) == 512
    assert tc.time == 100.0
    ok = soft_equiv(comp, gold, 1.0e-5)
    assert ok.all(), f"{(~ok).sum()} values outside the gold tolerance"
    assert np.max(np.abs(comp[:128] - gold[:128]) / gold[:128]) < 1e-7  # density
    assert np.max(np.abs(comp[128:256] - gold[128:256]) / np.abs(gold[128:256])) < 1e-5  # v^1


def test_p2c2p_known_answer(oracle):
    b, par, f, x = states.p2c2p_fmks()
    p = abi.default_params(**par)
    oracle.GeometryFillFMKS(b)
    for _ in range(100):  # p2c2p.cpp:124-127
        oracle.PrimitiveToConserved(p, b)
        assert oracle.ConservedToPrimitive(p, b) == 0
    pr = b["prim"]
    sl = slice(b.ng, b.ng + 512)
    bounds = {"rho": (abi.PRHO, 1e-9), "v1": (abi.PVEL, 1e-9), "v2": (abi.PVEL + 1, 1e-9),
              "v3": (abi.PVEL + 2, 1e-9), "u": (abi.PENG, 2e-9), "b1": (abi.PB, 1e-13), "b2": (abi.PB + 1, 1e-13),
              "b3": (abi.PB + 2, 1e-13)}
    for name, (v, tol) in bounds.items():
        ref = f[name](x)[sl]
        err = np.max(np.abs(ref - pr[v, 0, 0, sl]) / np.abs(ref))
        assert err < tol, (name, err)
    assert b["fail"].min() == 1.0


@pytest.mark.parametrize("recon", ["constant", "linear", "weno5z", "mp5"])
def test_uniform_state_is_stationary(oracle, recon):
    """Reconstruction reproduces a constant exactly, so every face of a
    uniform moving state carries the same flux and the divergence is 0."""
    b = states.random_block(6, 1)
    pr = b["prim"]
    for v in range(abi.NPRIM):
        pr[v] = pr[v, 4, 4, 4]
    p = abi.default_params(recon=recon, c2p_tol=1e-12, c2p_max_iter=100)
    oracle.PrimitiveToConserved(p, b)
    oracle.CalculateFluxes(p, b)
    oracle.FluxCT(p, b)
    oracle.CalculateFluidSourceTerms(p, b)
    oracle.FluxDivergence(p, b)
    ks, js, is_ = b.isl()
    assert np.all(b["dudt"][:, ks, js, is_] == 0.0)
    assert np.all(b["src"][:, ks, js, is_] == 0.0)


def test_fmks_geometry_known_answer(oracle):
    """tst/unit/geometry/test_geometry.cpp "Modified Kerr-Schild": FMKS with
    a = 0.8, pole derefinement, hslope 0.3, poly_xt 0.82, poly_alpha 14,
    smooth 0.5, x0 = -0.4409148982097008 at X = (1.13248983, 0.26388889,
    3.27249235): lapse, det g, g_mu nu and g^mu nu within the test's
    GetDifference < 1e-5 (and |value| < 1e-5 where it requires zero)."""
    g = abi.default_geometry(abi.GEOM_FMKS, a=0.8, derefine_poles=1, hslope=0.3, poly_xt=0.82, poly_alpha=14.0,
                             smooth=0.5, x0=-0.4409148982097008)
    out = oracle.fmks_point(g, 1.1324898310315077, 0.2638888888888889, 3.2724923474893677)
    ind = [[0, 1, 3, 6], [1, 2, 4, 7], [3, 4, 5, 8], [6, 7, 8, 9]]
    ind3 = [[0, 1, 3], [1, 2, 4], [3, 4, 5]]
    gc = np.array([[out[abi.G_GCOV + ind[m][n]] for n in range(4)] for m in range(4)])
    alpha = out[abi.G_ALPHA]
    beta = out[abi.G_BETA:abi.G_BETA + 3]
    gam = np.array([[out[abi.G_GAMCON + ind3[a][b]] for b in range(3)] for a in range(3)])
    gi = np.zeros((4, 4))  # spacetime inverse from lapse, shift, gamma^ij
    gi[0, 0] = -1 / alpha**2
    gi[0, 1:] = gi[1:, 0] = beta / alpha**2
    gi[1:, 1:] = gam - np.outer(beta, beta) / alpha**2

    def diff(a, b):  # test_geometry.cpp GetDifference
        return 2 * abs(b - a) / (abs(b) + abs(a) + 1e-300)

    assert diff(alpha, 0.7811769941965497) < 1e-5
    assert diff(alpha * out[abi.G_DETGAM], 64.40965903079623) < 1e-5
    for (m, n), ref in {(0, 0): -0.3612937485396168, (0, 1): 1.9821442243860723, (1, 1): 15.78288823,
                        (1, 2): -0.17903916, (1, 3): -3.51690001, (2, 2): 51.27859056, (3, 3): 9.18405881}.items():
        assert diff(gc[m, n], ref) < 1e-5 and diff(gc[n, m], ref) < 1e-5, (m, n)
    assert abs(gc[0, 2]) < 1e-5 and abs(gc[2, 3]) < 1e-5
    for (m, n), ref in {(0, 0): -1.63870625, (0, 1): 2.05810289e-01, (1, 1): 4.34252153e-02,
                        (1, 2): 0.00015161910494636605, (1, 3): 2.65272964e-02, (2, 2): 1.95018454e-02,
                        (3, 3): 1.19042557e-01}.items():
        assert diff(gi[m, n], ref) < 1e-5, (m, n)
    assert abs(gi[0, 3]) < 1e-5
    assert np.allclose(gc @ gi, np.eye(4), atol=1e-12)


def test_lorentz_factor_known_answer(oracle):
    """tst/unit/phoebus_utils/test_relativity_utils.cpp "RELATIVITY": for the
    primitive velocity W (0.7, 0.2, 0.1) on Minkowski, W = 1.474419561548971247
    (SoftEquiv at 1e-8); through prim2con, D = rho W and S_i = (rho h + b^2)
    W^2 v_i."""
    W_ref = 1.474419561548971247e+00
    prim = np.zeros((abi.NPRIM, 1))
    prim[abi.PRHO] = 1.0
    prim[abi.PENG] = 1.0e-3
    prim[abi.PPRS] = (5.0 / 3.0 - 1.0) * 1.0e-3
    prim[abi.PGM1] = 5.0 / 3.0
    prim[abi.PVEL:abi.PVEL + 3, 0] = np.array([0.7, 0.2, 0.1]) * W_ref
    p = abi.default_params(Gamma=5.0 / 3.0, mhd=0)
    cons = oracle.PrimitiveToConservedZones(p, prim)
    assert abs(cons[abi.CRHO, 0] - W_ref) < 1e-8 * W_ref / 2
    h = 1.0 + (1.0e-3 + prim[abi.PPRS, 0]) / 1.0
    for d, vd in enumerate((0.7, 0.2, 0.1)):
        assert abs(cons[abi.CMOM + d, 0] - h * W_ref**2 * vd) < 1e-8 * abs(h * W_ref**2 * vd)
