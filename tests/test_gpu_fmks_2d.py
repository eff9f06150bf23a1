"""GPU parity on the FMKS (Kerr-Schild) path and on the 2D linear-modes run.

FMKS geometry is read from tables (the reference's cached, axisymmetric
geometry).  The tables call exp, sin, cos and pow, which the GPU and the
oracle both evaluate through phoebus_gb300/csrc/phx_math.h with the same IEEE
operations, and the table kernels are compiled without contraction in both
library builds: the tables built on the GPU equal the oracle's bit for bit,
finite-difference derivatives included, and so do the hot-path tasks that
read them.
"""
import numpy as np
import pytest

from phoebus_gb300 import abi, states
from tests.util import assert_bitwise, face_region, flux_view, report_close

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("derefine", [0, 1])
def test_fmks_tables(oracle, ctx_exact, ctx_fast, derefine, exact):
    """GPU tables (both builds) equal the oracle's bit for bit: centre and
    face tables and the finite-difference derivatives, pole derefinement on
    and off (ghost zones at X2 < 0 and > 1 included)."""
    ctx = ctx_exact if exact else ctx_fast
    hb = states.fmks_random_block(derefine_poles=derefine)
    db = hb.to_device()
    oracle.GeometryFillFMKS(hb)
    ctx.GeometryFillFMKS(db)
    for name in ("cent", "face1", "face2", "deriv"):
        assert_bitwise(db.geom.arrays[name], hb.geom.arrays[name], f"{name} table")


def _shared_tables(oracle, hb):
    oracle.GeometryFillFMKS(hb)
    return hb.to_device()


def test_fmks_hot_path_exact(oracle, ctx_exact):
    p = abi.default_params(Gamma=4.0 / 3.0, recon="weno5z", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)
    hb = states.fmks_random_block(seed=77)
    db = _shared_tables(oracle, hb)
    oracle.PrimitiveToConserved(p, hb)
    ctx_exact.PrimitiveToConserved(p, db)
    assert_bitwise(db["cons"], hb["cons"], "cons")
    assert_bitwise(db["cell_sig"], hb["cell_sig"], "cell_sig")
    oracle.ConservedToPrimitive(p, hb)
    ctx_exact.ConservedToPrimitive(p, db)
    ctx_exact.check()
    assert_bitwise(db["prim"], hb["prim"], "prim")
    assert_bitwise(db["fail"], hb["fail"], "fail")
    oracle.CalculateFluxes(p, hb)
    ctx_exact.CalculateFluxes(p, db)
    for d in range(3):
        r = face_region(hb, d)
        assert_bitwise(flux_view(db["flux"], d)[(slice(None),) + r], flux_view(hb["flux"], d)[(slice(None),) + r],
                       f"flux d={d}")
    oracle.CalculateFluidSourceTerms(p, hb)
    ctx_exact.CalculateFluidSourceTerms(p, db)
    ks, js, is_ = hb.isl()
    assert_bitwise(db["src"][:, ks, js, is_], hb["src"][:, ks, js, is_], "src")
    assert np.abs(hb["src"][:, ks, js, is_]).max() > 0.0


def test_fmks_sources_fast(oracle, ctx_fast):
    """Production build on tables it built itself: sources per zone within
    1e-12 of the zone's source scale (|S_t| + |S_r| + |S_theta| + |tau|
    source magnitudes; S_phi vanishes analytically in axisymmetric Kerr and
    both builds give rounding residuals on that scale)."""
    p = abi.default_params(Gamma=4.0 / 3.0, c2p_tol=1e-10, c2p_max_iter=100)
    hb = states.fmks_random_block(seed=78)
    db = hb.to_device()
    oracle.GeometryFillFMKS(hb)
    ctx_fast.GeometryFillFMKS(db)
    assert_bitwise(db.geom.arrays["deriv"], hb.geom.arrays["deriv"], "deriv table (production build)")
    oracle.CalculateFluidSourceTerms(p, hb)
    ctx_fast.CalculateFluidSourceTerms(p, db)
    ks, js, is_ = hb.isl()
    got, ref = db["src"][:, ks, js, is_].cpu().numpy(), hb["src"][:, ks, js, is_]
    scale = np.abs(ref[0]) + np.abs(ref[1]) + np.abs(ref[3])
    for v in range(4):
        report_close(got[v], ref[v], scale, 1e-12, f"FMKS src {v}")


def test_p2c2p_known_answer_gpu(oracle, ctx_exact):
    b, par, f, x = states.p2c2p_fmks()
    p = abi.default_params(**par)
    db = _shared_tables(oracle, b)
    for _ in range(100):
        oracle.PrimitiveToConserved(p, b)
        oracle.ConservedToPrimitive(p, b)
        ctx_exact.PrimitiveToConserved(p, db)
        ctx_exact.ConservedToPrimitive(p, db)
    ctx_exact.check()
    assert_bitwise(db["prim"], b["prim"], "prim after 100 round trips")
    assert_bitwise(db["cons"], b["cons"], "cons after 100 round trips")


def test_linear_modes_run_gpu(oracle, ctx_exact):
    """The whole regression run on the GPU: bit-identical to the oracle, and
    so within the reference gold's tolerance."""
    import torch

    from phoebus_gb300.fluid import rk2_step
    from tests.test_cpu_oracle_pins import GOLD, soft_equiv

    hb, par, tlim = states.linear_modes_2d()
    p = abi.default_params(**par)
    db = hb.to_device()
    oracle.Initialize(p, hb)
    ctx_exact.Initialize(p, db)
    dt_h = oracle.EstimateTimestepBlock(p, hb, False)
    assert ctx_exact.EstimateTimestepBlock(p, db, False).item() == dt_h
    tc = states.TimeControl(tlim, dt_h, dt_init_fact=0.1)
    hs = np.zeros_like(hb["cons"])
    ds = torch.zeros_like(db["cons"])
    while tc.keep_going():
        dt = tc.begin_step()
        oracle.rk2_step(p, hb, hs, dt)
        rk2_step(ctx_exact, p, db, ds, dt)
        new_h = oracle.EstimateTimestepBlock(p, hb, True)
        assert ctx_exact.EstimateTimestepBlock(p, db, True).item() == new_h
        tc.end_step(new_h)
    ctx_exact.check()
    assert_bitwise(db["prim"], hb["prim"], "prim at t_lim")
    ks, js, is_ = hb.isl()
    pr = db["prim"].cpu().numpy()
    vals = np.concatenate([pr[abi.PRHO][ks, js, is_].ravel()] + [pr[abi.PVEL + d][ks, js, is_].ravel() for d in range(3)])
    comp = np.array([vals[10 * n] for n in range(len(vals) // 10)])
    assert soft_equiv(comp, np.loadtxt(GOLD / "linear_modes.gold"), 1e-3).all()
