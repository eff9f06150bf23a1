"""The Bondi regression run (tst/regression/bondi.py: inputs/bondi.pin with
128 zones) through phx_stage_mesh on the GPU: a 1D FMKS block with
gr_outflow boundaries exchanging densitised conserved variables.  The exact
build follows the oracle bit for bit, step by step, and so lands inside the
reference gold's tolerance; the production build stays within it too."""
import numpy as np
import pytest

from phoebus_gb300 import abi, states
from phoebus_gb300.fluid import MeshRK2
from tests.test_cpu_oracle_pins import GOLD, bondi_values, run_bondi, soft_equiv
from tests.util import assert_bitwise, host

pytestmark = pytest.mark.gpu


def gpu_bondi(ctx, checker=None):
    """Tables on the GPU, the pgen on the host with those tables, then the run
    on the GPU.  checker(step, dt): called with the GPU's dt of every step."""
    hb, par, tlim = states.bondi_1d()
    db = hb.to_device()
    ctx.GeometryFillFMKS(db)
    for k, a in db.geom.arrays.items():
        hb.geom.arrays[k] = host(a).copy()
    states.bondi_fill(hb)
    db["prim"].copy_(__import__("torch").from_numpy(hb["prim"]))
    p = abi.default_params(**par)
    rk = MeshRK2(ctx, p, states.bondi_mesh(), [db])
    rk.initialize()
    tc = states.TimeControl(tlim, rk.estimate_dt(False), dt_init_fact=1.0e-6)
    n = 0
    while tc.keep_going():
        dt = tc.begin_step()
        if checker:
            checker(n, dt)
        rk.step(dt)
        tc.end_step(rk.estimate_dt(True))
        n += 1
    ctx.check()
    return db, hb, tc


def test_bondi_gpu_bitwise_and_gold(oracle, ctx_exact):
    gpu_dts = []
    db, hb, tc = gpu_bondi(ctx_exact, lambda n, dt: gpu_dts.append(dt))
    # the oracle from the same tables and initial state
    ob, otc, odts = run_bondi(oracle, hb)
    assert len(gpu_dts) == len(odts) == tc.ncycle
    assert gpu_dts == odts, "time step sequences differ"
    assert_bitwise(db["prim"], ob["prim"], "prim at t = 100")
    assert_bitwise(db["cons"], ob["cons"], "cons at t = 100")
    gold = np.loadtxt(GOLD / "bondi.gold")
    assert soft_equiv(bondi_values(db.to_host()), gold, 1.0e-5).all()


def test_bondi_gpu_production_gold(ctx_fast):
    db, _, tc = gpu_bondi(ctx_fast)
    assert tc.time == 100.0
    comp = bondi_values(db.to_host())
    gold = np.loadtxt(GOLD / "bondi.gold")
    ok = soft_equiv(comp, gold, 1.0e-5)
    assert ok.all(), f"{(~ok).sum()} values outside the gold tolerance"
