"""GPU parity of fixup::ConservedToPrimitiveFixup and fixup::ApplyFloors
(fixup_c2p.cpp:170-353, fixup.cpp:370-540) against the oracle, exact build.

Failures are made on the host: NaN conserved states make con2prim flag zones
(fail = 0), which the fixup then repairs from their neighbours.  Floors and
ceilings are set tight enough that a large share of the random zones trip
them, including the re-inversion inside ApplyFloors.  The bitwise tests use
ConstantRhoSie floors (IEEE arithmetic only); the ExpX1RhoSie floors of the
torus deck call exp(), where CUDA's and glibc's results can differ by an ulp,
so that variant is compared to tolerance.
"""
import numpy as np
import pytest

from phoebus_gb300 import abi, states
from tests.util import assert_bitwise

pytestmark = pytest.mark.gpu


def _params(**over):
    base = dict(Gamma=4.0 / 3.0, c2p_tol=1e-10, c2p_max_iter=100, enable_floors=1, enable_c2p_fixup=1,
                enable_mhd_floors=1, enable_ceilings=1, floor_type="ConstantRhoSie", rho0_floor=5e-3, sie0_floor=1e-2,
                rho_exp_floor=-2.0, sie_exp_floor=-1.0, gam0_ceiling=3.0, sie0_ceiling=0.5, bsqorho0_ceiling=2.0,
                bsqou0_ceiling=50.0, recon="weno5z", riemann="hll")
    base.update(over)
    return abi.default_params(**base)


def test_c2p_fixup_exact(oracle, ctx_exact):
    p = _params()
    hb = states.random_block(10, 61)
    oracle.PrimitiveToConserved(p, hb)
    rng = np.random.default_rng(5)
    for _ in range(40):  # isolated and clustered failures
        k, j, i = rng.integers(3, 15, size=3)
        hb["cons"][abi.CRHO, k, j, i] = np.nan
    db = hb.to_device()
    oracle.ConservedToPrimitive(p, hb)
    ctx_exact.ConservedToPrimitive(p, db)
    assert (hb["fail"] == 0.0).sum() >= 30
    assert_bitwise(db["fail"], hb["fail"], "fail")
    oracle.ConservedToPrimitiveFixup(p, hb)
    ctx_exact.ConservedToPrimitiveFixup(p, db)
    ctx_exact.check()
    assert_bitwise(db["prim"], hb["prim"], "prim after fixup")
    assert_bitwise(db["cons"], hb["cons"], "cons after fixup")
    ks, js, is_ = hb.isl()
    assert np.isfinite(hb["cons"][:5, ks, js, is_]).all()


@pytest.mark.parametrize("mhd_floors", [0, 1])
def test_apply_floors_exact(oracle, ctx_exact, mhd_floors):
    p = _params(enable_mhd_floors=mhd_floors)
    hb = states.random_block(10, 62)
    hb.xmin = (-1.0, -1.0, -1.0)  # X1 < 0 raises the ExpX1 floors
    oracle.PrimitiveToConserved(p, hb)
    oracle.ConservedToPrimitive(p, hb)
    before = hb.to_host()
    db = hb.to_device()
    n_fail = oracle.ApplyFloors(p, hb)
    ctx_exact.ApplyFloors(p, db)
    ctx_exact.check()
    changed = ~np.all(before["prim"] == hb["prim"], axis=0)
    assert changed.mean() > 0.2, changed.mean()
    assert_bitwise(db["prim"], hb["prim"], "prim after floors")
    assert_bitwise(db["cons"], hb["cons"], "cons after floors")
    assert_bitwise(db["cell_sig"], hb["cell_sig"], "cell_sig after floors")


def test_stage_with_fixup_and_floors(oracle, ctx_exact):
    import torch

    p = _params()
    hb = states.random_block(10, 63)
    oracle.Initialize(p, hb)
    oracle.ApplyFloors(p, hb)
    db = hb.to_device()
    dt = 0.05 * oracle.EstimateTimestepBlock(p, hb, False)
    hs = np.zeros_like(hb["cons"])
    ds = torch.zeros_like(db["cons"])
    oracle.Stage(p, hb, hb["cons"], hs, 1.0, dt)
    ctx_exact.Stage(p, db, db["cons"], ds, 1.0, dt)
    ctx_exact.check()
    assert_bitwise(ds, hs, "stage cons")
    assert_bitwise(db["prim"], hb["prim"], "stage prims")
    assert_bitwise(db["fail"], hb["fail"], "stage fail")


def test_apply_floors_expx1_exact(oracle, ctx_exact):
    """ExpX1RhoSie floors (rho0 e^{-2 x1}-type exponentials): each side runs
    prim2con, con2prim and ApplyFloors from the same primitives.  The floors'
    exp is the library's written-out one, which the oracle evaluates too, so
    the floored state is bit for bit the oracle's (more than a fifth of the
    zones are floored)."""
    p = _params(floor_type="ExpX1RhoSie", rho0_floor=2e-3, sie0_floor=1e-2)
    hb = states.random_block(10, 64)
    hb.xmin = (-1.0, -1.0, -1.0)
    before = hb.to_host()
    db = hb.to_device()
    for side in (oracle, ctx_exact):
        blk = hb if side is oracle else db
        side.PrimitiveToConserved(p, blk)
        side.ConservedToPrimitive(p, blk)
        side.ApplyFloors(p, blk)
    ctx_exact.check()
    assert (~np.all(before["prim"] == hb["prim"], axis=0)).mean() > 0.2
    for name in ("fail", "prim", "cons"):
        assert_bitwise(db[name], hb[name], name)
