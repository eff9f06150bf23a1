"""Radiation moments on the GPU against the oracle (exact build: bit for bit).

Every task of include/phx_radiation.h on random 1D/2D/3D states (M1 and
Eddington closures, each reconstruction), full RK stages, the source with
the coupled fluid update and the coupled fluid + moment stage
(radiation_equilibration and a moving fluid), and the radiation_diffusion
regression run (512 zones to t = 1, 655 steps): the exact
build equals the oracle bit for bit, the production build stays within the
oracle's agreement bands with the reference gold.
"""
import numpy as np
import pytest

from phoebus_gb300 import abi, radiation, states
from phoebus_gb300.radiation import RadiationContext
from tests.test_cpu_m1_oracle import GOLD, diffusion_values, run_diffusion
from tests.util import assert_bitwise, host, random_rad_block

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rad_oracle(built):
    from oracle.oracle import RadOracle

    return RadOracle()


@pytest.fixture(scope="module")
def rx(ctx_exact):
    return RadiationContext(ctx_exact)


@pytest.fixture(scope="module")
def rf(ctx_fast):
    return RadiationContext(ctx_fast)


def _pair(nx, ndim, seed, **kw):
    hb = random_rad_block(nx, ndim, seed, **kw)
    return hb, hb.to_device()


def _cmp(db, hb, names, what, region=None):
    for n in names:
        g, r = host(db[n]), hb[n]
        if region is not None:
            g, r = g[(slice(None),) + region], r[(slice(None),) + region]
        assert_bitwise(g, r, f"{what}: {n}")


CASES = [("moment_m1", "linear", 1), ("moment_m1", "linear", 3), ("moment_m1", "weno5z", 2),
         ("moment_m1", "mp5", 3), ("moment_m1", "constant", 2), ("moment_eddington", "linear", 3),
         ("moment_eddington", "weno5z", 1)]


@pytest.mark.parametrize("method,recon,ndim", CASES)
def test_tasks_bitwise(rx, rad_oracle, method, recon, ndim):
    nx = {1: (64, 1, 1), 2: (24, 20, 1), 3: (12, 10, 8)}[ndim]
    hb, db = _pair(nx, ndim, seed=11 + ndim)
    rp = abi.default_rad_params(method=method, recon=recon, cfl=0.5, kappa_s=40.0, kappa_a=3.0, jbb_coeff=0.7)
    p = abi.default_params(Cv=1.3)
    e = hb.entire()
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentPrim2Con(rp, p, b, *e)
    _cmp(db, hb, ["rcons"], "prim2con")
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentCon2Prim(rp, p, b)
    _cmp(db, hb, ["rcons", "rprim"], "con2prim")
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentCalculateOpacities(rp, p, b)
    _cmp(db, hb, ["rprim"], "opacities")
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.CalculateFluxes(rp, p, b)
    ks, js, is_ = hb.isl()
    for d in range(ndim):
        reg = (slice(ks.start, ks.stop + (d == 2)), slice(js.start, js.stop + (d == 1)),
               slice(is_.start, is_.stop + (d == 0)))
        g = host(db["rflux"])[4 * d:4 * d + 4][(slice(None),) + reg]
        assert_bitwise(g, hb["rflux"][4 * d:4 * d + 4][(slice(None),) + reg], f"fluxes d={d}")
    import torch

    base_h = hb["rcons"] * 1.01
    out_h = np.zeros_like(base_h)
    base_d = torch.from_numpy(base_h).cuda()
    out_d = torch.zeros_like(base_d)
    rad_oracle.Update(rp, hb, base_h, out_h, 0.5, 1.0e-3)
    rx.Update(rp, db, base_d, out_d, 0.5, 1.0e-3)
    assert_bitwise(host(out_d)[(slice(None), ks, js, is_)], out_h[(slice(None), ks, js, is_)], "update out")
    _cmp(db, hb, ["rcons"], "update in place", (ks, js, is_))
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentFluidSource(rp, p, b, 2.0e-3)
    _cmp(db, hb, ["rcons", "rprim"], "fluid source", (ks, js, is_))
    dt_h = rad_oracle.EstimateTimestepBlock(rp, p, hb)
    dt_d = rx.EstimateTimestepBlock(rp, p, db)
    assert dt_d == dt_h
    rx.check()


@pytest.mark.parametrize("method,ndim", [("moment_m1", 3), ("moment_eddington", 2), ("moment_m1", 1)])
def test_rk2_steps_bitwise(rx, rad_oracle, method, ndim):
    nx = {1: (48, 1, 1), 2: (16, 16, 1), 3: (10, 8, 8)}[ndim]
    hb, db = _pair(nx, ndim, seed=23, vmax=0.3)
    rp = abi.default_rad_params(method=method, recon="linear", cfl=0.5, kappa_s=30.0, kappa_a=2.0, jbb_coeff=0.5)
    p = abi.default_params(Cv=1.0)
    import torch

    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentPrim2Con(rp, p, b)
        o.Initialize(rp, p, b)
    _cmp(db, hb, ["rcons", "rprim"], "initialize")
    buf_h = np.zeros_like(hb["rcons"])
    buf_d = torch.zeros_like(db["rcons"])
    for step in range(3):
        dt = rad_oracle.EstimateTimestepBlock(rp, p, hb)
        assert rx.EstimateTimestepBlock(rp, p, db) == dt
        rad_oracle.rk2_step(rp, p, hb, buf_h, dt)
        rx.rk2_step(rp, p, db, buf_d, dt)
        _cmp(db, hb, ["rcons", "rprim"], f"step {step}")
    rx.check()


BRANCHES = [
    # the radiation floors force the fluid floors on (fixup.cpp:130-134), so
    # ApplyFloors runs with its radiation part
    dict(rad=dict(enable_rad_floors=1, J0_floor=0.05, enable_rad_ceilings=1, xi0_ceiling=0.3, tau0_ceiling=0.5),
         fluid=dict(enable_ceilings=1, gam0_ceiling=1.05, enable_floors=1)),
    dict(rad=dict(closure_frail=1, oned_fixup_strategy="ignore_all"), fluid={}),
    dict(rad=dict(oned_fixup_strategy="ignore_dJ", recon_fixup_bounds=0), fluid={}),
    dict(rad=dict(method="moment_eddington", oned_fixup_strategy="ignore_dJ", enable_rad_ceilings=1,
                  xi0_ceiling=0.5, tau0_ceiling=2.0), fluid={}),
]


@pytest.mark.parametrize("case", range(len(BRANCHES)))
def test_branches_bitwise(rx, rad_oracle, case):
    """Bounds, ceilings, the W ceiling, the frail closure and the oned fixup
    strategies on states with |H|/J up to 0.999 (inversions that fail or are
    rewritten), every task and a full stage, bit for bit."""
    import torch

    cfg = BRANCHES[case]
    hb, db = _pair((14, 12, 10), 3, seed=70 + case, vmax=0.45, hmax=0.999)
    rp = abi.default_rad_params(cfl=0.5, kappa_s=60.0, kappa_a=4.0, jbb_coeff=0.8, **cfg["rad"])
    p = abi.default_params(Cv=1.0, **cfg["fluid"])
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentPrim2Con(rp, p, b, *b.entire())
    # every 7th zone gets a flux beyond the free-streaming limit: inversions
    # that the robust strategy rewrites and the frail one fails
    bad = (np.arange(hb.N) % 7 == 3).reshape(hb.shape)
    hb["rcons"][abi.RF:abi.RF + 3][:, bad] *= 1.8
    db["rcons"].copy_(torch.from_numpy(hb["rcons"]))
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentCon2Prim(rp, p, b)
    _cmp(db, hb, ["rcons", "rprim"], "con2prim")
    dt = 3.0e-3
    out_h = np.zeros_like(hb["rcons"])
    out_d = torch.zeros_like(db["rcons"])
    rad_oracle.Stage(rp, p, hb, hb["rcons"].copy(), out_h, 1.0, dt)
    rx.Stage(rp, p, db, db["rcons"].clone(), out_d, 1.0, dt)
    assert_bitwise(out_d, out_h, "stage output")
    _cmp(db, hb, ["rprim"], "stage prims")
    assert rx.EstimateTimestepBlock(rp, p, db) == rad_oracle.EstimateTimestepBlock(rp, p, hb)
    rx.check()


def gpu_diffusion(rc):
    hb, _, _, _ = radiation.radiation_advection()
    return run_diffusion(rc, hb.to_device())


def test_diffusion_run_bitwise(rx, rad_oracle):
    db, tc, dts = gpu_diffusion(rx)
    hb, otc, odts = run_diffusion(rad_oracle)
    assert dts == odts and tc.ncycle == otc.ncycle == 655
    assert_bitwise(db["rprim"][:abi.RFAIL + 1], hb["rprim"][:abi.RFAIL + 1], "prims at t = 1")
    assert_bitwise(db["rcons"], hb["rcons"], "cons at t = 1")
    rx.check()


def test_diffusion_run_production(rf, rad_oracle):
    db, tc, _ = gpu_diffusion(rf)
    assert tc.time == 1.0
    hb, _, _ = run_diffusion(rad_oracle)
    comp, ref = diffusion_values(db.to_host()), diffusion_values(hb)
    gold = np.loadtxt(GOLD / "radiation_diffusion.gold")
    # production (FMA contraction, the closure solve's scaled-tensor
    # residual) against the exact oracle after 655 steps: the closure
    # converges to |f| < 2.2e-10, so agreement is at that level, not bitwise
    m = np.abs(ref[:52]) > 1e-8
    assert np.max(np.abs(comp[:52][m] - ref[:52][m]) / np.abs(ref[:52][m])) < 1e-6
    assert np.abs(comp[52:104] - ref[52:104]).max() < 1e-7
    # and the gold bands of the oracle pin
    rel = np.abs(comp - gold) / np.maximum(np.abs(gold), 1.0e-10)
    assert rel[:52][gold[:52] >= 1.0e-2].max() < 1.5e-2 and rel[:52].max() < 0.15
    rf.check()


def test_rad_configuration_errors(rx):
    hb = random_rad_block((8, 1, 1), 1, seed=1)
    db = hb.to_device()
    p = abi.default_params()
    with pytest.raises(abi.PhxError) as e:
        rx.MomentCon2Prim(abi.default_rad_params(method=7), p, db)
    assert e.value.status == abi.PHX_ERR_INVALID_ARG
    # radiation/src_solver other than oned / fourd (radiation.cpp:403-415)
    with pytest.raises(abi.PhxError, match="src_solver") as e:
        rx.MomentFluidSource(abi.default_rad_params(src_solver=7), p, db, 1e-3)
    assert e.value.status == abi.PHX_ERR_INVALID_ARG
    import torch

    # the radiation floors need the fluid floors (the fixup package forces them on)
    with pytest.raises(abi.PhxError, match="enable_rad_floors") as e:
        rx.Stage(abi.default_rad_params(enable_rad_floors=1), abi.default_params(), db, db["rcons"],
                 torch.zeros_like(db["rcons"]), 1.0, 1e-3)
    assert e.value.status == abi.PHX_ERR_INVALID_ARG
    # the radiation-only stage refuses update_fluid (the fluid stage carries it)
    with pytest.raises(abi.PhxError, match="phx_rad_fluid_stage") as e:
        rx.Stage(abi.default_rad_params(update_fluid=1), p, db, db["rcons"], torch.zeros_like(db["rcons"]), 1.0,
                 1e-3)
    assert e.value.status == abi.PHX_ERR_INVALID_ARG
    with pytest.raises(abi.PhxError, match="enable_rad_floors") as e:
        rx.FluidStage(abi.default_rad_params(enable_rad_floors=1), abi.default_params(), db, db["cons"],
                      torch.zeros_like(db["cons"]), db["rcons"], torch.zeros_like(db["rcons"]), 1.0, 1e-3)
    assert e.value.status == abi.PHX_ERR_INVALID_ARG


@pytest.mark.parametrize("exact", [True, False])
def test_closure_unit_known_answer_gpu(rx, rf, rad_oracle, exact):
    """tst/unit/radiation/test_closure.cpp's 6000-point closure round trip
    through phx_rad_prim_to_con / phx_rad_con_to_prim: the exact build equals
    the oracle bit for bit, both builds meet the reference's 1e-5 bound at
    every point."""
    import torch

    from tests.test_cpu_m1_oracle import closure_unit_block

    rc = rx if exact else rf
    hb, v, x = closure_unit_block()
    rp, p = abi.default_rad_params(method="moment_m1"), abi.default_params()
    db = hb.to_device()
    rad_oracle.MomentPrim2Con(rp, p, hb)
    rc.MomentPrim2Con(rp, p, db)
    sl = hb.isl()
    if exact:
        _cmp(db, hb, ["rcons"], "prim2con")
    E = host(db["rcons"])[abi.RE][sl].ravel()
    F = np.stack([host(db["rcons"])[abi.RF + d][sl].ravel() for d in range(3)])
    xig, phig = rad_oracle.M1GuessesFromEddington(E, F, np.stack([v, 0 * v, 0 * v]))
    for b in (hb, db):
        R = b["rprim"]
        R[abi.RXI][sl] = torch.from_numpy(xig.reshape(R[abi.RXI][sl].shape)).cuda() if b is db else \
            xig.reshape(R[abi.RXI][sl].shape)
        R[abi.RPHI][sl] = (torch.from_numpy((phig / 1.0001).reshape(R[abi.RPHI][sl].shape)).cuda() if b is db else
                           (phig / 1.0001).reshape(R[abi.RPHI][sl].shape))
    rad_oracle.MomentCon2Prim(rp, p, hb, *hb.interior())
    rc.MomentCon2Prim(rp, p, db, *db.interior())
    rc.check()
    if exact:
        _cmp(db, hb, ["rcons", "rprim"], "con2prim", sl)
    J_out = host(db["rprim"])[abi.RJ][sl].ravel()
    H_out = host(db["rprim"])[abi.RH][sl].ravel() * J_out
    H_in = x / np.sqrt(1.0 - v * v)
    wrong = ~((np.abs(1.0 - J_out) < 1.0e-5) & (np.abs(H_in - H_out) < 1.0e-5))
    assert wrong.sum() == 0


def _coupled_pair(nx, ndim, seed, p, vmax=0.3):
    """Host/device blocks with a random moving fluid whose conserved
    variables are its prim2con (entire block) and random moments."""
    from oracle.oracle import Oracle

    hb = random_rad_block(nx, ndim, seed, vmax=vmax)
    P = hb["prim"]
    P[abi.PPRS] = p.gm1 * P[abi.PENG]
    P[abi.PGM1] = p.gm1 + 1.0
    Oracle().PrimitiveToConserved(p, hb, *hb.entire())
    return hb, hb.to_device()


@pytest.mark.parametrize("method,ndim", [("moment_m1", 1), ("moment_m1", 3), ("moment_eddington", 2)])
def test_fluid_source_update_fluid_bitwise(rx, rad_oracle, method, ndim):
    """MomentFluidSource with update_fluid = 1 (exact build): the fluid's tau
    and S_i, its con2prim (prims, cell speeds, cons where bounds were used),
    the closure inversion with the new velocity, and the failure state of a
    zone whose fluid cannot be inverted (NaN D) equal the oracle bit for bit
    in every fluid and radiation field of the interior."""
    nx = {1: (64, 1, 1), 2: (20, 16, 1), 3: (10, 8, 8)}[ndim]
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.0)
    rp = abi.default_rad_params(method=method, kappa_a=4.0, kappa_s=20.0, jbb_coeff=0.6, update_fluid=1)
    hb, db = _coupled_pair(nx, ndim, 61 + ndim, p)
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentPrim2Con(rp, p, b, *b.entire())
        o.MomentCon2Prim(rp, p, b)
        o.MomentCalculateOpacities(rp, p, b)
    ks, js, is_ = hb.isl()
    bad = (ks.start, js.start, is_.start + 3)
    hb["cons"][(abi.CRHO,) + bad] = np.nan
    db["cons"][(abi.CRHO,) + bad] = float("nan")
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentFluidSource(rp, p, b, 0.05)
    rx.check()
    _cmp(db, hb, ["prim", "cons", "cell_sig", "rcons", "rprim"], "update_fluid source", (ks, js, is_))
    assert host(db["rprim"])[(abi.RJ,) + bad] == 10 * np.finfo(np.float64).tiny


@pytest.mark.parametrize("method", ["moment_m1", "moment_eddington"])
@pytest.mark.parametrize("geom,ndim", [("mink", 1), ("mink", 3), ("fmks", 2)])
@pytest.mark.parametrize("upd,backup,maxiter", [(0, 0, 100), (1, 0, 100), (0, 1, 2), (1, 0, 2)])
def test_fourd_source_bitwise(rx, rad_oracle, method, geom, ndim, upd, backup, maxiter):
    """MomentFluidSource with the fourd solver (moments_source.cpp:489-786),
    exact build, equals the oracle bit for bit in every fluid and radiation
    field of the interior: the Newton iterations over (u, W v^i) with the
    finite-difference Jacobian and the 4x4 adjugate inverse, on Minkowski and
    FMKS blocks, with and without the coupled fluid update.  Two Newton steps
    leave most zones unconverged: with src_use_oned_backup they take the oned
    solver (whose root find shares the iteration cap), without it the
    radiation keeps its state (and, with update_fluid, the fluid takes a zero
    exchange)."""
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.0)
    if geom == "mink":
        nx = {1: (48, 1, 1), 3: (8, 8, 6)}[ndim]
        hb, db = _coupled_pair(nx, ndim, 101 + ndim, p, vmax=0.3)
    else:
        from oracle.oracle import Oracle

        from tests.util import random_rad_block_fmks

        hb = random_rad_block_fmks((16, 12, 1), 2, seed=97)
        P = hb["prim"]
        P[abi.PPRS] = p.gm1 * P[abi.PENG]
        P[abi.PGM1] = p.gm1 + 1.0
        Oracle().PrimitiveToConserved(p, hb, *hb.entire())
        db = hb.to_device()
    rp = abi.default_rad_params(method=method, kappa_a=4.0, kappa_s=20.0, jbb_coeff=0.6, update_fluid=upd,
                                src_solver="fourd", src_use_oned_backup=backup, src_rootfind_maxiter=maxiter)
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentPrim2Con(rp, p, b, *b.entire())
        o.MomentCon2Prim(rp, p, b)
        o.MomentCalculateOpacities(rp, p, b)
    r0 = hb["rcons"].copy()
    applied = rad_oracle.MomentFluidSource(rp, p, hb, 0.02)
    rx.MomentFluidSource(rp, p, db, 0.02)
    rx.check()
    ks, js, is_ = hb.isl()
    _cmp(db, hb, ["prim", "cons", "rcons", "rprim"], f"fourd source ({geom}, update_fluid={upd})", (ks, js, is_))
    n = hb["rcons"][0][ks, js, is_].size
    if maxiter == 100:
        assert applied == n  # every zone converged
        assert np.any(hb["rcons"][:, ks, js, is_] != r0[:, ks, js, is_])
    elif not backup:
        assert applied < n


@pytest.mark.parametrize("method", ["moment_m1", "moment_eddington"])
@pytest.mark.parametrize("upd", [0, 1])
def test_fourd_source_production(rf, rad_oracle, method, upd):
    """The fourd solver in the production build (FMA contraction, reciprocal
    products) against the oracle: both Newton iterations stop at a relative
    residual of 1e-12 (src_rootfind_tol), so the conserved radiation and
    fluid variables agree per zone to 1e-9 (the residual's tolerance times the
    Jacobian's conditioning; measured up to 5e-10) and the primitives inverted
    from them to 1e-7 (measured up to 1e-8 in H_i / J and 4e-8 in a fluid
    velocity component near zero)."""
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.0)
    hb, db = _coupled_pair((8, 8, 6), 3, 131 + upd, p, vmax=0.3)
    rp = abi.default_rad_params(method=method, kappa_a=4.0, kappa_s=20.0, jbb_coeff=0.6, update_fluid=upd,
                                src_solver="fourd")
    for o, b in ((rad_oracle, hb), (rf, db)):
        o.MomentPrim2Con(rp, p, b, *b.entire())
        o.MomentCon2Prim(rp, p, b)
        o.MomentCalculateOpacities(rp, p, b)
    applied = rad_oracle.MomentFluidSource(rp, p, hb, 0.02)
    rf.MomentFluidSource(rp, p, db, 0.02)
    rf.check()
    ks, js, is_ = hb.isl()
    assert applied == hb["rcons"][0][ks, js, is_].size
    for name in ("rcons", "rprim", "cons", "prim"):
        g, r = host(db[name])[(slice(None), ks, js, is_)], hb[name][(slice(None), ks, js, is_)]
        n = abi.RFAIL + 1 if name == "rprim" else g.shape[0]
        for v in range(n):
            # per zone, with a floor of 1e-6 of the variable's magnitude for
            # components that pass through zero (velocities, fluxes)
            den = np.abs(r[v]) + 1e-6 * np.abs(r[v]).max() + 1e-300
            err = float(np.max(np.abs(g[v] - r[v]) / den))
            print(f"[per-zone] fourd production {name}[{v}] max rel {err:.2e}")
            # primitives are inversions of the updated conserved variables:
            # the closure's H_i / J of a nearly isotropic field carries the
            # cancellation of F_i - (J terms) into the ratio, and the fluid's
            # con2prim (update_fluid) stops within its 1e-10 bracket
            assert err < (1e-7 if name in ("rprim", "prim") else 1e-9), (name, v, err)


@pytest.mark.parametrize("method,ndim", [("moment_m1", 1), ("moment_eddington", 2), ("moment_m1", 3)])
def test_fluid_stage_rk2_bitwise(rx, rad_oracle, method, ndim):
    """phx_rad_fluid_stage (exact build): three rk2 steps of a moving fluid
    coupled to the moments (both packages' fluxes and updates, FillDerived,
    MomentFluidSource with update_fluid, exchange, FillDerived) equal the
    oracle's composed reference stage bit for bit in every field."""
    import torch

    nx = {1: (48, 1, 1), 2: (16, 16, 1), 3: (10, 8, 8)}[ndim]
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.0, recon="linear", riemann="hll", c2p_tol=1e-10,
                           c2p_max_iter=100)
    rp = abi.default_rad_params(method=method, recon="linear", cfl=0.5, kappa_a=2.0, kappa_s=10.0, jbb_coeff=0.4)
    hb, db = _coupled_pair(nx, ndim, 71 + ndim, p, vmax=0.2)
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentPrim2Con(rp, p, b, *b.entire())
        o.MomentCon2Prim(rp, p, b)
    fh, rh = np.zeros_like(hb["cons"]), np.zeros_like(hb["rcons"])
    fd, rd = torch.zeros_like(db["cons"]), torch.zeros_like(db["rcons"])
    dt = 0.2 * min(hb.dx[d] for d in range(ndim))
    for step in range(3):
        rad_oracle.rk2_fluid_step(rp, p, hb, fh, rh, dt)
        rx.rk2_fluid_step(rp, p, db, fd, rd, dt)
        _cmp(db, hb, ["prim", "cons", "fail", "rcons", "rprim"], f"coupled step {step}")
    rx.check()


def test_equilibration_exact_and_production(rx, rf, rad_oracle):
    """radiation_equilibration through phx_rad_fluid_stage: the exact build
    equals the oracle bit for bit after 60 rk2 steps; the production build
    conserves tau + E per zone to 1e-13 and reaches the oracle's gas
    temperature and J within the con2prim tolerance (c2p_tol 1e-8, the
    deck's default: the fluid inversion stops anywhere inside a bracket of
    that relative width, and both builds take their own path to it)."""
    from oracle.oracle import Oracle

    from tests.test_cpu_m1_oracle import equilibration_run

    hb, _, _, e0 = equilibration_run(rad_oracle, Oracle(), steps=60, nx1=16)
    ctx_e, ctx_f = rx.fc, rf.fc
    db, _, _, _ = equilibration_run(rx, ctx_e, steps=60, nx1=16, b=lambda h: h.to_device())
    _cmp(db, hb, ["prim", "cons", "fail", "rcons", "rprim"], "equilibration (exact)")
    fb, _, _, _ = equilibration_run(rf, ctx_f, steps=60, nx1=16, b=lambda h: h.to_device())
    ks, js, is_ = hb.isl()
    tot = host(fb["cons"])[abi.CENG][ks, js, is_] + host(fb["rcons"])[abi.RE][ks, js, is_]
    assert np.max(np.abs(tot - e0) / e0) < 1e-13
    for name, v in (("prim", abi.PTMP), ("rprim", abi.RJ)):
        g, r = host(fb[name])[v][ks, js, is_], hb[name][v][ks, js, is_]
        err = float(np.max(np.abs(g - r) / np.abs(r)))
        print(f"[per-zone] equilibration production {name}[{v}] max rel {err:.2e}")
        assert err < 1e-8
    rx.check()
    rf.check()


# ---- curved geometry: FMKS tables (the torus' Kerr-Schild metric, a = 0.9375)
@pytest.mark.parametrize("method,recon,ndim", [("moment_m1", "linear", 2), ("moment_eddington", "weno5z", 2),
                                               ("moment_m1", "mp5", 3), ("moment_eddington", "constant", 3)])
def test_fmks_tasks_bitwise(rx, rad_oracle, method, recon, ndim):
    """Every radiation task on an FMKS block (exact build) equals the oracle
    bit for bit: prim2con and con2prim with the LocalThreeGeometry and
    sqrt(gamma), fluxes with the face metric, lapse and shift, the update
    with the geometric source (moments.cpp:764-885), the source step with
    the lapse in the optical depths (both update_fluid settings), and the
    timestep with the metric's signal speeds."""
    import torch

    from tests.util import random_rad_block_fmks

    nx = {2: (20, 16, 1), 3: (12, 10, 8)}[ndim]
    hb = random_rad_block_fmks(nx, ndim, seed=91 + ndim)
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.3)
    P = hb["prim"]
    P[abi.PPRS] = p.gm1 * P[abi.PENG]
    P[abi.PGM1] = p.gm1 + 1.0
    from oracle.oracle import Oracle

    Oracle().PrimitiveToConserved(p, hb, *hb.entire())
    db = hb.to_device()
    rp = abi.default_rad_params(method=method, recon=recon, cfl=0.5, kappa_s=40.0, kappa_a=3.0, jbb_coeff=0.7)
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentPrim2Con(rp, p, b, *b.entire())
    _cmp(db, hb, ["rcons"], "fmks prim2con")
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentCon2Prim(rp, p, b)
    _cmp(db, hb, ["rcons", "rprim"], "fmks con2prim")
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentCalculateOpacities(rp, p, b)
        o.CalculateFluxes(rp, p, b)
    ks, js, is_ = hb.isl()
    for d in range(ndim):
        reg = (slice(ks.start, ks.stop + (d == 2)), slice(js.start, js.stop + (d == 1)),
               slice(is_.start, is_.stop + (d == 0)))
        g = host(db["rflux"])[4 * d:4 * d + 4][(slice(None),) + reg]
        assert_bitwise(g, hb["rflux"][4 * d:4 * d + 4][(slice(None),) + reg], f"fmks fluxes d={d}")
    base_h = hb["rcons"] * 1.01
    out_h = np.zeros_like(base_h)
    base_d = torch.from_numpy(base_h).cuda()
    out_d = torch.zeros_like(base_d)
    rad_oracle.Update(rp, hb, base_h, out_h, 0.5, 1.0e-3)
    rx.Update(rp, db, base_d, out_d, 0.5, 1.0e-3)
    assert_bitwise(host(out_d)[(slice(None), ks, js, is_)], out_h[(slice(None), ks, js, is_)], "fmks update out")
    _cmp(db, hb, ["rcons", "rdudt"], "fmks update (geometric source)", (ks, js, is_))
    src = rad_oracle.GeometricSource(rp, hb)
    assert np.abs(src[0][ks, js, is_]).max() > 0  # the curved source is at work
    for upd in (0, 1):
        rpu = abi.default_rad_params(method=method, recon=recon, cfl=0.5, kappa_s=40.0, kappa_a=3.0,
                                     jbb_coeff=0.7, update_fluid=upd)
        for o, b in ((rad_oracle, hb), (rx, db)):
            o.MomentFluidSource(rpu, p, b, 2.0e-3)
        _cmp(db, hb, ["rcons", "rprim", "cons", "prim"], f"fmks fluid source update_fluid={upd}", (ks, js, is_))
    assert rx.EstimateTimestepBlock(rp, p, db) == rad_oracle.EstimateTimestepBlock(rp, p, hb)
    rx.check()


@pytest.mark.parametrize("method", ["moment_m1", "moment_eddington"])
def test_fmks_stages_bitwise(rx, rad_oracle, method):
    """Two rk2 steps on an FMKS block (periodic ghosts), exact build, bit
    for bit: the moment-only stage, then the coupled fluid + moment stage."""
    import torch

    from oracle.oracle import Oracle
    from tests.util import random_rad_block_fmks

    hb = random_rad_block_fmks((16, 12, 1), 2, seed=7, vmax=0.2)
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.0, recon="linear", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)
    P = hb["prim"]
    P[abi.PPRS] = p.gm1 * P[abi.PENG]
    P[abi.PGM1] = p.gm1 + 1.0
    Oracle().PrimitiveToConserved(p, hb, *hb.entire())
    db = hb.to_device()
    rp = abi.default_rad_params(method=method, recon="linear", cfl=0.5, kappa_s=10.0, kappa_a=2.0, jbb_coeff=0.4)
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentPrim2Con(rp, p, b, *b.entire())
        o.Initialize(rp, p, b)
    dt = 0.2 * min(hb.dx[d] for d in range(2))
    # second-stage containers start as copies of the state (their ghost
    # zones, which FillDerived inverts before the exchange, hold a physical
    # state as after any earlier step)
    rh, rd = hb["rcons"].copy(), db["rcons"].clone()
    fh, fd = hb["cons"].copy(), db["cons"].clone()
    rad_oracle.rk2_step(rp, p, hb, rh, dt)
    rx.rk2_step(rp, p, db, rd, dt)
    _cmp(db, hb, ["rcons", "rprim"], "fmks moment stage")
    rad_oracle.rk2_fluid_step(rp, p, hb, fh, rh, dt)
    rx.rk2_fluid_step(rp, p, db, fd, rd, dt)
    _cmp(db, hb, ["prim", "cons", "rcons", "rprim"], "fmks coupled stage")
    rx.check()


# ---- the radiation parts of the fixups and floors
@pytest.mark.parametrize("geometry", ["minkowski", "fmks"])
@pytest.mark.parametrize("method", ["moment_m1", "moment_eddington"])
def test_rad_fixup_and_floors_bitwise(rx, rad_oracle, method, geometry):
    """RadConservedToPrimitiveFixup (zones marked failed, isolated and
    adjacent, both strategies) and ApplyFloors with the radiation on (fluid
    floors acting in some zones, the J floor and the xi ceiling acting in
    others) equal the oracle bit for bit (exact build)."""
    from oracle.oracle import Oracle
    from tests.util import random_rad_block_fmks

    nx = (16, 12, 1)
    hb = random_rad_block(nx, 2, seed=29, vmax=0.3) if geometry == "minkowski" else \
        random_rad_block_fmks(nx, 2, seed=29, vmax=0.3)
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.0)
    P = hb["prim"]
    P[abi.PPRS] = p.gm1 * P[abi.PENG]
    P[abi.PGM1] = p.gm1 + 1.0
    Oracle().PrimitiveToConserved(p, hb, *hb.entire())
    rp = abi.default_rad_params(method=method)
    rad_oracle.MomentPrim2Con(rp, p, hb, *hb.entire())
    rad_oracle.MomentCon2Prim(rp, p, hb)
    ks, js, is_ = hb.isl()
    F = hb["rprim"][abi.RFAIL]
    F[0, js.start + 2, is_.start + 3] = 0.0
    F[0, js.start + 6, is_.start + 5:is_.start + 7] = 0.0
    F[0, js.start, is_.start] = 0.0  # next to the ghosts
    db = hb.to_device()
    p.enable_c2p_fixup = 1
    for strategy in (0, 1):
        rp.rad_c2p_failure_floors = strategy
        h2, d2 = hb.to_host(), hb.to_device()
        rad_oracle.RadConservedToPrimitiveFixup(rp, p, h2)
        rx.RadConservedToPrimitiveFixup(rp, p, d2)
        _cmp(d2, h2, ["rprim", "rcons"], f"rad c2p fixup strategy {strategy}")
    rp.rad_c2p_failure_floors = 0
    p.enable_floors = 1
    rho = hb["prim"][abi.PRHO]
    p.rho0_floor, p.sie0_floor = float(np.quantile(rho, 0.1)), 1e-6  # some fluid floors act
    rp.enable_rad_floors, rp.J0_floor = 1, float(np.quantile(hb["rprim"][abi.RJ], 0.3))
    rp.enable_rad_ceilings, rp.xi0_ceiling = 1, 0.5
    rad_oracle.ApplyFloors(rp, p, hb)
    rx.ApplyFloors(rp, p, db)
    _cmp(db, hb, ["prim", "cons", "rprim", "rcons"], "apply floors with radiation")
    rx.check()


@pytest.mark.parametrize("geometry,jfloor", [("minkowski", "ConstantJ"), ("fmks", "ConstantJ"),
                                             ("fmks", "ExpX1J"), ("minkowski", "ExpX1J")])
def test_stages_with_fixups_and_floors_bitwise(rx, rad_oracle, geometry, jfloor):
    """The moment stage and the coupled fluid + moment stage with the c2p
    fixups, the fluid floors and the radiation floors (ConstantJ, or ExpX1J:
    J0 exp(J_exp_floor X1) at the zone's X1 in ApplyFloors and at the face's
    X1 on the reconstructed J) and ceilings on: two rk2 steps of each equal
    the oracle bit for bit (exact build)."""
    import torch

    from oracle.oracle import Oracle
    from tests.util import random_rad_block_fmks

    nx = (16, 12, 1)
    hb = random_rad_block(nx, 2, seed=37, vmax=0.2) if geometry == "minkowski" else \
        random_rad_block_fmks(nx, 2, seed=37, vmax=0.2)
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.0, recon="linear", riemann="hll", c2p_tol=1e-10, c2p_max_iter=100)
    P = hb["prim"]
    P[abi.PPRS] = p.gm1 * P[abi.PENG]
    P[abi.PGM1] = p.gm1 + 1.0
    Oracle().PrimitiveToConserved(p, hb, *hb.entire())
    p.enable_floors, p.enable_c2p_fixup, p.enable_ceilings = 1, 1, 1
    p.rho0_floor, p.sie0_floor = float(np.quantile(P[abi.PRHO], 0.05)), 1e-6
    rp = abi.default_rad_params(method="moment_m1", recon="linear", cfl=0.5, kappa_s=10.0, kappa_a=2.0, jbb_coeff=0.4)
    rp.enable_rad_floors, rp.J0_floor = 1, float(np.quantile(hb["rprim"][abi.RJ], 0.1))
    if jfloor == "ExpX1J":  # the floor spans the quantiles across the block's X1 range
        rp.rad_floor_type, rp.J_exp_floor = abi.RAD_FLOOR["ExpX1J"], -1.5
        rp.J0_floor = float(np.quantile(hb["rprim"][abi.RJ], 0.3)) * np.exp(1.5 * hb.xmin[0])
    rp.enable_rad_ceilings, rp.xi0_ceiling, rp.tau0_ceiling = 1, 0.9, 1e3
    db = hb.to_device()
    for o, b in ((rad_oracle, hb), (rx, db)):
        o.MomentPrim2Con(rp, p, b, *b.entire())
        o.Initialize(rp, p, b)
    dt = 0.2 * min(hb.dx[d] for d in range(2))
    rh, rd = hb["rcons"].copy(), db["rcons"].clone()
    fh, fd = hb["cons"].copy(), db["cons"].clone()
    for step in range(2):
        rad_oracle.rk2_step(rp, p, hb, rh, dt)
        rx.rk2_step(rp, p, db, rd, dt)
        _cmp(db, hb, ["prim", "cons", "rprim", "rcons"], f"moment stage with fixups, step {step}")
    for step in range(2):
        rad_oracle.rk2_fluid_step(rp, p, hb, fh, rh, dt)
        rx.rk2_fluid_step(rp, p, db, fd, rd, dt)
        _cmp(db, hb, ["prim", "cons", "fail", "rprim", "rcons"], f"coupled stage with fixups, step {step}")
    rx.check()
