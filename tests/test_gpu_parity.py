"""GPU parity of each hot-path kernel against the CPU oracle, through the C ABI.

The exact build (nvcc -fmad=false) must reproduce the oracle (g++
-ffp-contract=off) bit for bit on every value the reference computes with
IEEE arithmetic: Minkowski everywhere, and FMKS given the same geometry
tables.  The production build (FMA contraction) is held to the tolerances
the path specifies: 1e-12 relative per zone on fluxes and sources, the
con2prim tolerance on primitives, and identical fail flags.
"""
import numpy as np
import pytest

from phoebus_gb300 import abi, states
from phoebus_gb300.block import Block
from tests.util import assert_bitwise, assert_close, divergence_faces, face_region, flux_view

pytestmark = pytest.mark.gpu

RECONS = ["constant", "linear", "weno5z", "mp5"]
SOLVERS = ["llf", "hll"]


def _random_state(n=10, seed=7, oracle=None, p=None):
    hb = states.random_block(n, seed)
    if oracle is not None:
        oracle.Initialize(p, hb)
    return hb


def _smooth_state(n=12):
    hb, par = states.kelvin_helmholtz(n=n, seed=11)
    return hb, par


@pytest.mark.parametrize("exact", [True, False])
def test_prim_to_con(oracle, ctx_exact, ctx_fast, exact):
    ctx = ctx_exact if exact else ctx_fast
    p = abi.default_params(Gamma=4.0 / 3.0)
    hb = states.random_block(10, 3)
    db = hb.to_device()
    oracle.PrimitiveToConserved(p, hb)
    ctx.PrimitiveToConserved(p, db)
    if exact:
        assert_bitwise(db["cons"], hb["cons"], "cons")
        assert_bitwise(db["cell_sig"], hb["cell_sig"], "cell_sig")
    else:
        for m in range(8):
            assert_close(db["cons"][m], hb["cons"][m], 1e-12, f"cons {m}")


@pytest.mark.parametrize("tol,maxit", [(1e-10, 100), (1e-8, 20)])
def test_con_to_prim_exact(oracle, ctx_exact, tol, maxit):
    p = abi.default_params(Gamma=4.0 / 3.0, c2p_tol=tol, c2p_max_iter=maxit)
    hb = states.random_block(12, 5)
    oracle.PrimitiveToConserved(p, hb)
    db = hb.to_device()
    iters = np.zeros(hb.shape, dtype=np.int32)
    oracle.ConservedToPrimitive(p, hb, iters=iters)
    ctx_exact.c2p_stats(reset=True)
    ctx_exact.ConservedToPrimitive(p, db)
    ctx_exact.check()
    assert_bitwise(db["prim"], hb["prim"], "prim")
    assert_bitwise(db["fail"], hb["fail"], "fail")
    assert_bitwise(db["cons"], hb["cons"], "cons")
    assert_bitwise(db["cell_sig"], hb["cell_sig"], "cell_sig")
    st = ctx_exact.c2p_stats()
    assert st["zones"] == hb.N
    assert st["iterations"] == int(iters.sum())
    hist = np.bincount(np.minimum(iters.ravel(), abi.C2P_HIST - 1), minlength=abi.C2P_HIST)
    assert list(hist) == st["hist"]


def test_con_to_prim_fast(oracle, ctx_fast):
    """Production build: the root mu agrees to the con2prim tolerance, fail
    flags are identical, and the primitives differ by no more than two valid
    solutions can: each is within the tolerance-induced deviation delta of
    the exact root, measured here per variable as the oracle at tol against
    the oracle at 1e-15 (the state's conditioning amplifies d mu into the
    prims, ~W^2 for Lorentz factors up to 5)."""
    tol = 1e-10
    p = abi.default_params(Gamma=4.0 / 3.0, c2p_tol=tol, c2p_max_iter=100)
    hb = states.random_block(12, 9)
    oracle.PrimitiveToConserved(p, hb)
    db = hb.to_device()
    tight = hb.to_host()
    oracle.ConservedToPrimitive(p, hb)
    oracle.ConservedToPrimitive(abi.default_params(Gamma=4.0 / 3.0, c2p_tol=1e-15, c2p_max_iter=300), tight)
    ctx_fast.ConservedToPrimitive(p, db)
    ctx_fast.check()
    assert_bitwise(db["fail"], hb["fail"], "fail")
    got, ref, exact = db["prim"].cpu().numpy(), hb["prim"], tight["prim"]
    # mu is the root itself: |mu_gpu - mu_cpu| <= 2 tol (both within tol of the root)
    assert np.max(np.abs(got[abi.PMU] - ref[abi.PMU])) <= 2 * tol
    for v in (abi.PRHO, abi.PENG, abi.PPRS, abi.PVEL, abi.PVEL + 1, abi.PVEL + 2):
        delta = np.max(np.abs(ref[v] - exact[v]) / np.abs(exact[v]))
        err = np.max(np.abs(got[v] - ref[v]) / np.abs(ref[v]))
        assert err <= 2.5 * delta + 1e-14, (v, err, delta)


def test_con_to_prim_nan_and_guess(oracle, ctx_exact):
    """NaN conserved input -> fail flag 0, prims untouched (the reference
    returns failure before writing)."""
    p = abi.default_params(Gamma=4.0 / 3.0, c2p_tol=1e-10, c2p_max_iter=100)
    hb = states.random_block(8, 21)
    oracle.PrimitiveToConserved(p, hb)
    hb["cons"][abi.CRHO, 5, 6, 7] = np.nan
    hb["cons"][abi.CENG, 9, 9, 9] = np.nan
    hb["prim"][abi.PMU] = 0.37  # warm-start guess everywhere
    db = hb.to_device()
    oracle.ConservedToPrimitive(p, hb)
    ctx_exact.ConservedToPrimitive(p, db)
    ctx_exact.check()
    assert hb["fail"][0, 5, 6, 7] == 0.0 and hb["fail"][0, 9, 9, 9] == 0.0
    assert_bitwise(db["prim"], hb["prim"], "prim")
    assert_bitwise(db["fail"], hb["fail"], "fail")


@pytest.mark.parametrize("recon", RECONS)
@pytest.mark.parametrize("solver", SOLVERS)
def test_fluxes_exact(oracle, ctx_exact, recon, solver):
    p = abi.default_params(Gamma=5.0 / 3.0, recon=recon, riemann=solver, c2p_tol=1e-10, c2p_max_iter=100)
    hb, _ = _smooth_state(12)
    oracle.Initialize(p, hb)
    db = hb.to_device()
    oracle.CalculateFluxes(p, hb)
    ctx_exact.CalculateFluxes(p, db)
    ctx_exact.check()
    for d in range(3):
        r = face_region(hb, d)
        assert_bitwise(flux_view(db["flux"], d)[(slice(None),) + r], flux_view(hb["flux"], d)[(slice(None),) + r],
                       f"flux d={d}")
        assert_bitwise(db["face_sig"][d][r], hb["face_sig"][d][r], f"face_sig d={d}")


@pytest.mark.parametrize("recon", ["weno5z", "mp5", "linear"])
def test_fluxes_random_state(oracle, ctx_exact, recon):
    """Discontinuous per-zone random state (limiters and MP5 branches)."""
    p = abi.default_params(Gamma=4.0 / 3.0, recon=recon, riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)
    hb = states.random_block(10, 33)
    oracle.Initialize(p, hb)
    db = hb.to_device()
    oracle.CalculateFluxes(p, hb)
    ctx_exact.CalculateFluxes(p, db)
    for d in range(3):
        r = face_region(hb, d)
        assert_bitwise(flux_view(db["flux"], d)[(slice(None),) + r], flux_view(hb["flux"], d)[(slice(None),) + r],
                       f"flux d={d}")


@pytest.mark.parametrize("staging", ["tensor", "bulk", "loads"])
@pytest.mark.parametrize("shape", [(10, 10, 10), (256, 6, 6)])
def test_fluxes_x1_staging(oracle, ctx_exact, staging, shape, monkeypatch):
    """The X1 kernel's three ways of staging pencils in shared memory (tiled
    TMA through a tensor map, 1-D bulk copies, plain loads) give the oracle's
    fluxes bit for bit; (256, 6, 6) has 264-cell pencils, which the tensor
    map splits in two 132-cell rows (a TMA box dimension is at most 256)."""
    from phoebus_gb300.block import Block

    monkeypatch.setenv("PHX_X1_STAGING", staging)
    p = abi.default_params(Gamma=4.0 / 3.0, recon="weno5z", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)
    ref = states.random_block(6, 35)
    hb = Block(shape, 4, 3, (0.0, 0.0, 0.0), tuple(1.0 / n for n in shape)).alloc()
    rng = np.random.default_rng(36)
    for v in range(hb["prim"].shape[0]):  # tile the random state over the larger block
        src = ref["prim"][v]
        reps = [int(np.ceil(t / s)) for t, s in zip(hb["prim"][v].shape, src.shape)]
        hb["prim"][v] = np.tile(src, reps)[tuple(slice(0, t) for t in hb["prim"][v].shape)]
    hb["prim"][abi.PRHO] *= 1.0 + 0.01 * rng.random(hb["prim"][abi.PRHO].shape)
    oracle.Initialize(p, hb)
    db = hb.to_device()
    oracle.CalculateFluxes(p, hb)
    ctx_exact.CalculateFluxes(p, db)
    ctx_exact.check()
    r = face_region(hb, 0)
    assert_bitwise(flux_view(db["flux"], 0)[(slice(None),) + r], flux_view(hb["flux"], 0)[(slice(None),) + r],
                   f"flux d=0 ({staging})")
    assert_bitwise(db["face_sig"][0][r], hb["face_sig"][0][r], f"face_sig d=0 ({staging})")


@pytest.mark.parametrize("recon,solver,state", [("weno5z", "hll", "smooth"), ("mp5", "hll", "smooth"),
                                                ("linear", "llf", "smooth"), ("weno5z", "hll", "random"),
                                                ("mp5", "hll", "random"), ("linear", "llf", "random")])
def test_fluxes_fast_tolerance(oracle, ctx_fast, recon, solver, state):
    """Production build: every face flux within 1e-12 of the oracle's relative
    to the face's own scale (the magnitudes of the terms that form it there,
    tests/util.py face_flux_scale), on the smooth shear state and on the
    per-zone random discontinuous state (limiters, MP5 branches, WENO5-Z
    weights far from linear)."""
    from tests.util import face_flux_scale, report_close

    p = abi.default_params(Gamma=5.0 / 3.0, recon=recon, riemann=solver, c2p_tol=1e-10, c2p_max_iter=100)
    hb = _smooth_state(12)[0] if state == "smooth" else states.random_block(10, 33)
    oracle.Initialize(p, hb)
    db = hb.to_device()
    oracle.CalculateFluxes(p, hb)
    ctx_fast.CalculateFluxes(p, db)
    for d in range(3):
        r = face_region(hb, d)
        sl = (slice(None),) + r
        scale = face_flux_scale(hb, d)
        report_close(flux_view(db["flux"], d)[sl], flux_view(hb["flux"], d)[sl], scale[sl], 1e-12,
                     f"{recon}/{solver} {state} flux d={d}")


def test_flux_ct_and_update(oracle, ctx_exact):
    p = abi.default_params(Gamma=5.0 / 3.0, recon="weno5z", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)
    hb, _ = _smooth_state(12)
    oracle.Initialize(p, hb)
    db = hb.to_device()
    oracle.CalculateFluxes(p, hb)
    oracle.FluxCT(p, hb)
    oracle.CalculateFluidSourceTerms(p, hb)
    oracle.FluxDivergence(p, hb)
    ctx_exact.CalculateFluxes(p, db)
    ctx_exact.FluxCT(p, db)
    ctx_exact.CalculateFluidSourceTerms(p, db)
    ctx_exact.UpdateStage(db, None, None, 1.0, 0.0)  # dU/dt only
    for d in range(3):
        r = divergence_faces(hb, d)
        assert_bitwise(flux_view(db["flux"], d)[(slice(None),) + r], flux_view(hb["flux"], d)[(slice(None),) + r],
                       f"flux after FluxCT d={d}")
    ks, js, is_ = hb.isl()
    assert_bitwise(db["src"][:, ks, js, is_], hb["src"][:, ks, js, is_], "src")
    assert np.all(hb["src"][:, ks, js, is_] == 0.0)  # Minkowski: exactly zero
    assert_bitwise(db["dudt"][:, ks, js, is_], hb["dudt"][:, ks, js, is_], "dudt")


def test_ghosts_and_dt(oracle, ctx_exact):
    import torch

    p = abi.default_params(Gamma=4.0 / 3.0, c2p_tol=1e-10, c2p_max_iter=100, cfl=0.3)
    hb = states.random_block(8, 44)
    oracle.PrimitiveToConserved(p, hb)
    hb["cons"][:, :4] = -1.0  # dirty ghosts
    db = hb.to_device()
    oracle.FillGhostsPeriodic(hb, hb["cons"], 8)
    ctx_exact.FillGhostsPeriodic(db, db["cons"], 8)
    assert_bitwise(db["cons"], hb["cons"], "cons after ghost exchange")
    oracle.ConservedToPrimitive(p, hb)
    ctx_exact.ConservedToPrimitive(p, db)
    oracle.CalculateFluxes(p, hb)
    ctx_exact.CalculateFluxes(p, db)
    for face in (False, True):
        ref = oracle.EstimateTimestepBlock(p, hb, face)
        got = ctx_exact.EstimateTimestepBlock(p, db, face)
        torch.cuda.synchronize()
        assert got.item() == ref


@pytest.mark.parametrize("recon,solver", [("weno5z", "hll"), ("linear", "llf"), ("mp5", "hll")])
def test_stage_exact(oracle, ctx_exact, recon, solver):
    import torch

    p = abi.default_params(Gamma=5.0 / 3.0, recon=recon, riemann=solver, c2p_tol=1e-10, c2p_max_iter=100)
    hb, _ = _smooth_state(12)
    oracle.Initialize(p, hb)
    db = hb.to_device()
    dt = 0.3 * oracle.EstimateTimestepBlock(p, hb, False)
    hs = np.zeros_like(hb["cons"])
    ds = torch.zeros_like(db["cons"])
    for beta, (hin, hout, din, dout) in [(1.0, (hb["cons"], hs, db["cons"], ds)),
                                         (0.5, (hs, hb["cons"], ds, db["cons"]))]:
        base_h, base_d = hb["cons"], db["cons"]
        hb.arrays["cons"], db.arrays["cons"] = hin, din
        oracle.Stage(p, hb, base_h, hout, beta, dt)
        ctx_exact.Stage(p, db, base_d, dout, beta, dt)
        hb.arrays["cons"], db.arrays["cons"] = base_h, base_d
    ctx_exact.check()
    assert_bitwise(db["cons"], hb["cons"], "cons after RK2 step")
    assert_bitwise(db["prim"], hb["prim"], "prim after RK2 step")
    assert_bitwise(db["fail"], hb["fail"], "fail after RK2 step")


def test_blast_wave_steps(oracle, ctx_exact):
    """Config 1 shape at reduced size: SR-MHD blast wave, PLM + LLF, RK2,
    CFL 0.3, several steps with the reference's timestep control (dt grows
    at most 2x per step; first estimate from cell speeds, then face speeds)."""
    import torch

    from phoebus_gb300.fluid import rk2_step

    hb, par = states.blast_wave(24)
    p = abi.default_params(**par)
    db = hb.to_device()
    oracle.Initialize(p, hb)
    ctx_exact.Initialize(p, db)
    assert_bitwise(db["prim"], hb["prim"], "prim after init")
    dt = oracle.EstimateTimestepBlock(p, hb, False)
    dt_d = ctx_exact.EstimateTimestepBlock(p, db, False).item()
    assert dt == dt_d
    hs = np.zeros_like(hb["cons"])
    ds = torch.zeros_like(db["cons"])
    for step in range(4):
        oracle.rk2_step(p, hb, hs, dt)
        rk2_step(ctx_exact, p, db, ds, dt)
        ctx_exact.check()
        assert_bitwise(db["cons"], hb["cons"], f"cons step {step}")
        dt_new = oracle.EstimateTimestepBlock(p, hb, True)
        assert ctx_exact.EstimateTimestepBlock(p, db, True).item() == dt_new
        dt = min(2 * dt, dt_new)
    assert_bitwise(db["prim"], hb["prim"], "prim")
    assert_bitwise(db["fail"], hb["fail"], "fail")
