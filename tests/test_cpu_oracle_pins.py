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
