"""Pin the radiation-moment oracle (CPU only).

- radiation_diffusion.gold (tst/regression/radiation_diffusion.py): the
  512-zone M1 diffusion run of the radiation_advection deck to t = 1,
  flattened like regression_test.py:347-391 (r.p.J, then r.p.H components,
  every 10th value).  The gold predates the reference tree (its deck lacks
  the <phoebus> boundary keys the current fluid package requires), and the
  restatement of the current code meets it on the pulse, not at its 1e-5
  tolerance: the bands below are the measured agreement with margin.  With
  the timestep of the free-streaming signal speed (the estimate before its
  diffusion-limit mixing) the agreement is about three times closer.
- the restated tanh against the correctly rounded value;
- closure inversions: prim -> con -> prim round trips (M1, Eddington).
"""
from pathlib import Path

import numpy as np
import pytest

from phoebus_gb300 import abi, radiation, states
from tests.util import random_rad_block

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def rad_oracle(built):
    from oracle.oracle import RadOracle

    return RadOracle()


def run_diffusion(o, b=None, free_streaming_dt=False):
    """The regression run through any object with the RadOracle task names
    (the oracle on host arrays, or a RadiationContext on device arrays).
    free_streaming_dt: the timestep cfl dx / 1 of the signal speed cs_rad = 1
    (the estimate before its diffusion-limit mixing) instead of the current
    EstimateTimestepBlock.  Returns (block, TimeControl, dts)."""
    if b is None:
        b, par, rpar, tlim = radiation.radiation_advection()
    else:
        _, par, rpar, tlim = radiation.radiation_advection(nx1=b.nx[0])
    p, rp = abi.default_params(**par), abi.default_rad_params(**rpar)
    o.MomentPrim2Con(rp, p, b)
    o.Initialize(rp, p, b)
    est = (lambda: rp.cfl * b.dx[0]) if free_streaming_dt else (lambda: o.EstimateTimestepBlock(rp, p, b))
    tc = states.TimeControl(tlim, est(), dt_init_fact=1.0e-6)
    buf = np.zeros_like(b["rcons"]) if isinstance(b["rcons"], np.ndarray) else b["rcons"].clone()
    dts = []
    while tc.keep_going():
        dt = tc.begin_step()
        dts.append(dt)
        o.rk2_step(rp, p, b, buf, dt)
        tc.end_step(est())
    return b, tc, dts


def diffusion_values(b):
    """regression_test.py:347-376 flattening with compression_factor 10."""
    sl = b.isl()
    R = b["rprim"]
    data = np.concatenate([R[abi.RJ][sl].ravel()] + [R[abi.RH + d][sl].ravel() for d in range(3)])
    return np.array([data[10 * n] for n in range(len(data) // 10)])


def test_radiation_diffusion_gold(rad_oracle):
    b, tc, _ = run_diffusion(rad_oracle)
    assert tc.time == 1.0
    comp, gold = diffusion_values(b), np.loadtxt(GOLD / "radiation_diffusion.gold")
    assert comp.shape == gold.shape == (204,)
    rel = np.abs(comp - gold) / np.maximum(np.abs(gold), 1.0e-10)  # soft_equiv's measure
    J, Jg = comp[:52], gold[:52]
    assert rel[:52][Jg >= 1.0e-2].max() < 1.5e-2  # the pulse (measured 9.9e-3)
    assert rel[:52].max() < 0.15  # tails and floor region (measured 0.105)
    # pulse moments
    x = (np.arange(52) * 10 + 0.5) / 512
    m, mg = J > 1e-6, Jg > 1e-6
    c, cg = (x[m] * J[m]).sum() / J[m].sum(), (x[mg] * Jg[mg]).sum() / Jg[mg].sum()
    assert abs(c - cg) < 1.0e-4 and abs(J.max() - Jg.max()) / Jg.max() < 1.0e-3
    assert np.abs(comp[52:104] - gold[52:104]).max() < 4.0e-3  # H_x / J (measured 2.2e-3)
    assert np.abs(comp[104:]).max() < 1.0e-20  # H_y, H_z: round-off only, as in the gold


def test_radiation_diffusion_gold_free_streaming_dt(rad_oracle):
    """The same run with the timestep of the free-streaming signal speed
    (cs_rad = 1, dt = cfl dx: 1025 steps) meets the gold about three times
    closer on every measure: the gold's dt sequence is the earlier estimate's,
    and the time-discretisation error of the operator-split stiff scattering
    source is most of the remaining difference."""
    b, tc, dts = run_diffusion(rad_oracle, free_streaming_dt=True)
    assert tc.time == 1.0 and tc.ncycle == 1025
    comp, gold = diffusion_values(b), np.loadtxt(GOLD / "radiation_diffusion.gold")
    rel = np.abs(comp - gold) / np.maximum(np.abs(gold), 1.0e-10)
    assert rel[:52][gold[:52] >= 1.0e-2].max() < 5.0e-3  # measured 3.7e-3
    assert rel[:52].max() < 3.0e-2  # measured 2.2e-2
    assert np.abs(comp[52:104] - gold[52:104]).max() < 1.0e-3  # measured 7.6e-4


def test_tanh_restatement(rad_oracle):
    import mpmath

    mpmath.mp.dps = 40
    rng = np.random.default_rng(3)
    xs = np.concatenate([rng.uniform(0, 23, 400), 10 ** rng.uniform(-9, 1.4, 400), [0.0, 0.25, 0.5, 21.99, 22.0]])
    worst = 0.0
    for x in xs:
        ex = mpmath.tanh(mpmath.mpf(float(x)))
        t = rad_oracle.tanh(float(x))
        if ex == 0:
            assert t == 0.0
            continue
        worst = max(worst, abs(float((mpmath.mpf(t) - ex) / np.spacing(float(ex)))))
        assert rad_oracle.tanh(-float(x)) == -t
    assert worst <= 4.0


@pytest.mark.parametrize("method", ["moment_m1", "moment_eddington"])
@pytest.mark.parametrize("aligned", [False, True])
def test_closure_round_trip(rad_oracle, method, aligned):
    """MomentPrim2Con then MomentCon2Prim recovers J and H/J where the
    reference's closure solve is exact: fluid at rest, or flux and velocity
    along one axis.  (It holds the angle phi at pi, i.e. takes the rest-frame
    flux along the F / v basis vector g of closure_m1.hpp:326-372; for other
    states the inversion differs from the prim2con closure at the 1e-3 level,
    in the reference as here.)"""
    b = random_rad_block((16, 12, 1), 2, seed=5, vmax=0.4 if aligned else 0.0)
    if aligned:
        for d in (1, 2):
            b["prim"][abi.PVEL + d] = 0.0
            b["rprim"][abi.RH + d] = 0.0
    rp, p = abi.default_rad_params(method=method), abi.default_params(Cv=1.0)
    J0, H0 = b["rprim"][abi.RJ].copy(), b["rprim"][abi.RH:abi.RH + 3].copy()
    rad_oracle.MomentPrim2Con(rp, p, b, *b.entire())
    rad_oracle.MomentCon2Prim(rp, p, b)
    R = b["rprim"]
    assert (R[abi.RFAIL] == 1.0).all()
    tol = 1e-8 if method == "moment_m1" else 1e-13
    assert np.max(np.abs(R[abi.RJ] - J0) / J0) < tol
    assert np.max(np.abs(R[abi.RH:abi.RH + 3] - H0)) < tol


def test_rad_params_default_matches_library(built):
    import ctypes as C

    lib = abi.load()
    r = abi.RadParams()
    lib.phx_rad_params_default(C.byref(r))
    ref = abi.default_rad_params()
    for name, _ in abi.RadParams._fields_:
        assert getattr(r, name) == getattr(ref, name), name


def test_pulse_workload_steps_cleanly(rad_oracle):
    """The bench's 3D M1 workload (radiation.radiation_pulse_3d) at a small
    size: two RK2 steps without failed inversions or NaNs; total E conserved
    where no source exchanges energy with the fluid."""
    b, par, rpar = radiation.radiation_pulse_3d(n=16)
    p, rp = abi.default_params(**par), abi.default_rad_params(**rpar)
    rad_oracle.MomentPrim2Con(rp, p, b)
    rad_oracle.Initialize(rp, p, b)
    rad_oracle.MomentCalculateOpacities(rp, p, b)
    dt = rad_oracle.EstimateTimestepBlock(rp, p, b)
    sl = b.isl()
    buf = np.zeros_like(b["rcons"])
    for _ in range(2):
        rad_oracle.rk2_step(rp, p, b, buf, dt)
    R = b["rprim"]
    assert (R[abi.RFAIL][sl] == 1.0).all()
    assert np.isfinite(b["rcons"][(slice(None),) + sl]).all() and (R[abi.RJ][sl] > 0).all()
    # without absorption and with the fluid at rest (scattering off moving
    # matter exchanges lab-frame energy with it, dE = -tauH v.H) the periodic
    # transport conserves the total E up to round-off
    b2, par2, rpar2 = radiation.radiation_pulse_3d(n=16, kappa_a=0.0, v=(0.0, 0.0, 0.0))
    p2, rp2 = abi.default_params(**par2), abi.default_rad_params(**rpar2)
    rad_oracle.MomentPrim2Con(rp2, p2, b2)
    rad_oracle.Initialize(rp2, p2, b2)
    E0 = b2["rcons"][abi.RE][sl].sum()
    buf2 = np.zeros_like(b2["rcons"])
    rad_oracle.MomentCalculateOpacities(rp2, p2, b2)
    dt2 = rad_oracle.EstimateTimestepBlock(rp2, p2, b2)
    for _ in range(2):
        rad_oracle.rk2_step(rp2, p2, b2, buf2, dt2)
    E1 = b2["rcons"][abi.RE][sl].sum()
    assert abs(E1 - E0) / E0 < 1e-12


def closure_unit_block():
    """tst/unit/radiation/test_closure.cpp's grid as a 1D block: phi_v = 0,
    |v| in [0, 0.6) step 0.01, xi in [1e-10, 1] step 0.01; J = 1 and
    tilde H_1 = xi J / sqrt(gamma^11 - v_1^2) (the reference's loop bounds and
    accumulation, restated)."""
    from phoebus_gb300.block import Block
    from phoebus_gb300.radiation import alloc_rad

    pts = []
    vmag = 0.0
    while vmag < 0.6:
        xi = 1.0e-10
        while xi <= 1.0:
            pts.append((vmag, xi))
            xi += 1.0e-2
        vmag += 1.0e-2
    n = len(pts)
    b = Block((n, 1, 1), ng=4, ndim=1, xmin=(0.0, 0.0, 0.0), dx=(1.0 / n, 1.0, 1.0), backend="numpy")
    b.alloc(["prim", "cons", "flux", "face_sig", "cell_sig", "fail", "src", "emf", "dudt"])
    alloc_rad(b)
    sl = b.isl()
    v = np.array([q[0] for q in pts])
    x = np.array([q[1] for q in pts])
    W = 1 / np.sqrt(1 - v * v)
    P, R = b["prim"], b["rprim"]
    P[abi.PRHO][sl] = 1.0
    P[abi.PTMP][sl] = 1.0
    P[abi.PVEL][sl] = W * v
    R[abi.RJ][sl] = 1.0
    R[abi.RH][sl] = x * 1.0 / np.sqrt(1.0 - v * v)  # H_1 / J
    return b, v, x


def test_closure_unit_known_answer(rad_oracle):
    """tst/unit/radiation/test_closure.cpp ("M1 Closure"): prim2con, the M1
    guesses from the Eddington inversion, the closure solve and con2prim
    recover J and tilde H_1 within 1e-5 at every one of the 6000 points
    (REQUIRE(n_wrong == 0))."""
    b, v, x = closure_unit_block()
    rp, p = abi.default_rad_params(method="moment_m1"), abi.default_params()
    rad_oracle.MomentPrim2Con(rp, p, b)
    sl = b.isl()
    E = b["rcons"][abi.RE][sl].ravel()
    F = np.stack([b["rcons"][abi.RF + d][sl].ravel() for d in range(3)])
    con_v = np.stack([v, 0 * v, 0 * v])
    xig, phig = rad_oracle.M1GuessesFromEddington(E, F, con_v)
    b["rprim"][abi.RXI][sl] = xig
    b["rprim"][abi.RPHI][sl] = phig / 1.0001  # MomentCon2Prim scales the stored phi by 1.0001
    rad_oracle.MomentCon2Prim(rp, p, b, *b.interior())
    J_out = b["rprim"][abi.RJ][sl].ravel()
    H_out = b["rprim"][abi.RH][sl].ravel() * J_out
    H_in = x / np.sqrt(1.0 - v * v)
    wrong = ~((np.abs(1.0 - J_out) / 1.0 < 1.0e-5) & (np.abs(H_in - H_out) / 1.0 < 1.0e-5))
    assert len(x) == 6000 and wrong.sum() == 0, f"{wrong.sum()} of {len(x)} points wrong"


# ---- coupled fluid update (MomentFluidSource with update_fluid = true)
def equilibration_run(o, fo=None, steps=120, dt=0.01, kappa=5.0, nx1=4, b=None):
    """The radiation_equilibration problem (gas at T = 1, radiation at
    T = 0.01, gray absorption kappa) through any object with the RadOracle /
    RadiationContext task names: fo (an Oracle or a FluidContext) initialises
    the fluid, o the moments; fixed dt.  Returns (block, par, radiation par,
    total energy tau + E per interior zone at the start)."""
    hb, par, rpar, _ = radiation.radiation_equilibration(nx1=nx1, kappa=kappa)
    b = hb if b is None else b(hb)
    p, rp = abi.default_params(**par), abi.default_rad_params(**rpar)
    fo.PrimitiveToConserved(p, b, *b.entire())
    o.MomentPrim2Con(rp, p, b, *b.entire())
    fo.FillGhostsPeriodic(b, b["cons"], 5)
    o.FillGhostsPeriodic(b)
    fo.ConservedToPrimitive(p, b)
    o.MomentCon2Prim(rp, p, b)
    ks, js, is_ = b.isl()
    e0 = b["cons"][abi.CENG][ks, js, is_] + b["rcons"][abi.RE][ks, js, is_]
    fbuf = b["cons"] * 0
    rbuf = b["rcons"] * 0
    for _ in range(steps):
        o.rk2_fluid_step(rp, p, b, fbuf, rbuf, dt)
    return b, p, rp, e0


def test_equilibration_conserves_energy_and_equilibrates(rad_oracle):
    """Gas and radiation at rest exchange energy only through the source:
    tau + E per zone stays at its initial value to rounding, the gas cools
    monotonically towards the temperature T_eq with Cv T_eq + JBB(T_eq) =
    the initial total, and J approaches JBB(T_eq)."""
    from oracle.oracle import Oracle

    fo = Oracle()
    b, p, rp, e0 = equilibration_run(rad_oracle, fo, steps=1)
    T1 = b["prim"][abi.PTMP][b.isl()].copy()
    assert np.all(T1 < 1.0) and np.all(T1 > 0.9)
    b, p, rp, e0 = equilibration_run(rad_oracle, fo, steps=200)
    ks, js, is_ = b.isl()
    tot = b["cons"][abi.CENG][ks, js, is_] + b["rcons"][abi.RE][ks, js, is_]
    assert np.max(np.abs(tot - e0) / e0) < 1e-13
    T = b["prim"][abi.PTMP][ks, js, is_]
    J = b["rprim"][abi.RJ][ks, js, is_]
    e = float(e0.ravel()[0])
    # T_eq from Cv T + T^4 = e (Cv = jbb = 1) by Newton
    Teq = 0.7
    for _ in range(50):
        Teq -= (Teq + Teq ** 4 - e) / (1 + 4 * Teq ** 3)
    assert np.allclose(T, Teq, rtol=1e-9, atol=0), (T.ravel(), Teq)
    assert np.allclose(J, Teq ** 4, rtol=1e-8, atol=0)
    assert np.all(b["fail"][0][ks, js, is_] == 1.0) and np.all(b["rprim"][abi.RFAIL][ks, js, is_] == 1.0)
    assert np.all(b["prim"][abi.PVEL:abi.PVEL + 3][:, ks, js, is_] == 0.0)


@pytest.mark.parametrize("method", ["moment_eddington", "moment_m1"])
def test_fourd_equilibration(rad_oracle, method, monkeypatch):
    """The fourd source solver (moments_source.cpp:489-786) on the
    radiation_equilibration problem: at rest the 4-D Newton iteration over
    (u, W v^i) solves the same backward-Euler energy exchange as the oned
    temperature root find (T and J agree to 1e-10 after 20 steps); it
    conserves tau + E per zone to rounding and reaches T_eq and
    J = JBB(T_eq) with every zone converged."""
    from oracle.oracle import Oracle

    orig = radiation.radiation_equilibration

    def run(solver, steps):
        def patched(*a, **k):
            hb, par, rpar, t = orig(*a, **k)
            return hb, par, dict(rpar, src_solver=solver, method=method), t

        monkeypatch.setattr(radiation, "radiation_equilibration", patched)
        return equilibration_run(rad_oracle, Oracle(), steps=steps)

    b1, _, _, _ = run("oned", 20)
    b4, _, _, _ = run("fourd", 20)
    ks, js, is_ = b1.isl()
    for name, v in (("prim", abi.PTMP), ("rprim", abi.RJ)):
        a, c = b1[name][v][ks, js, is_], b4[name][v][ks, js, is_]
        assert np.max(np.abs(a - c) / np.abs(a)) < 1e-10
    b, p, rp, e0 = run("fourd", 200)
    tot = b["cons"][abi.CENG][ks, js, is_] + b["rcons"][abi.RE][ks, js, is_]
    assert np.max(np.abs(tot - e0) / e0) < 1e-13
    e = float(e0.ravel()[0])
    Teq = 0.7
    for _ in range(50):
        Teq -= (Teq + Teq ** 4 - e) / (1 + 4 * Teq ** 3)
    assert np.allclose(b["prim"][abi.PTMP][ks, js, is_], Teq, rtol=1e-9, atol=0)
    assert np.allclose(b["rprim"][abi.RJ][ks, js, is_], Teq ** 4, rtol=1e-8, atol=0)
    assert np.all(b["fail"][0][ks, js, is_] == 1.0) and np.all(b["rprim"][abi.RFAIL][ks, js, is_] == 1.0)


def test_update_fluid_failure_state(rad_oracle):
    """A zone whose fluid cannot be inverted (NaN conserved density) leaves
    MomentFluidSource with the reference's failure state: the fluid at
    rho = u = 10 SMALL at rest with P = (Gamma - 1) rho u / rho,
    T = (u / rho) / Cv, the bulk modulus Gamma (Gamma - 1) rho Cv T in the
    gamma1 slot and D, S, tau from prim2con; the radiation at J = SMALL,
    H = 0.  Other zones keep tau + E."""
    from oracle.oracle import Oracle

    fo = Oracle()
    hb = random_rad_block((12, 1, 1), 1, seed=41, vmax=0.2)
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.0)
    rp = abi.default_rad_params(method="moment_m1", kappa_a=3.0, kappa_s=5.0, jbb_coeff=0.5, update_fluid=1)
    P = hb["prim"]
    P[abi.PPRS] = p.gm1 * P[abi.PENG]
    P[abi.PGM1] = p.gm1 + 1.0
    fo.PrimitiveToConserved(p, hb, *hb.entire())
    rad_oracle.MomentPrim2Con(rp, p, hb, *hb.entire())
    rad_oracle.MomentCon2Prim(rp, p, hb)
    rad_oracle.MomentCalculateOpacities(rp, p, hb)
    bad = hb.ng + 5
    hb["cons"][abi.CRHO][0, 0, bad] = np.nan
    ks, js, is_ = hb.isl()
    e0 = hb["cons"][abi.CENG][ks, js, is_] + hb["rcons"][abi.RE][ks, js, is_]
    rad_oracle.MomentFluidSource(rp, p, hb, 0.05)
    small = 10 * np.finfo(np.float64).tiny
    z = (slice(None), 0, 0, bad)
    Pz, Uz, Rz = hb["prim"][z], hb["cons"][z], hb["rprim"][z]
    assert Pz[abi.PRHO] == 10 * small and Pz[abi.PENG] == 10 * small
    assert np.all(Pz[abi.PVEL:abi.PVEL + 3] == 0.0)
    sie = (10 * small) / (10 * small + small)
    assert Pz[abi.PPRS] == p.gm1 * (10 * small) * sie
    assert Pz[abi.PTMP] == sie / p.Cv
    assert Pz[abi.PGM1] == (p.gm1 + 1) * p.gm1 * (10 * small) * p.Cv * Pz[abi.PTMP]
    assert Uz[abi.CRHO] == Pz[abi.PRHO] and np.all(Uz[abi.CMOM:abi.CMOM + 3] == 0.0)
    assert Rz[abi.RJ] == small and np.all(Rz[abi.RH:abi.RH + 3] == 0.0)
    tot = hb["cons"][abi.CENG][ks, js, is_] + hb["rcons"][abi.RE][ks, js, is_]
    keep = np.ones(tot.shape, bool)
    keep[..., bad - hb.ng] = False
    assert np.max(np.abs(tot - e0)[keep] / np.abs(e0)[keep]) < 1e-12


# ---- curved geometry (FMKS tables)
@pytest.mark.parametrize("method", ["moment_m1", "moment_eddington"])
def test_fmks_closure_round_trip(rad_oracle, method):
    """On an FMKS block, MomentPrim2Con then MomentCon2Prim returns J and
    H_i / J (LocalThreeGeometry with gamma^ij from matrixInverse3x3, the
    tables' sqrt(gamma)) where the reference's closure solve is exact: the
    Eddington closure for a moving fluid (a linear inversion), M1 for a fluid
    at rest (the rest-frame flux then lies along the basis vector g the solve
    holds it to); the second prim2con returns E and F_i."""
    from tests.util import random_rad_block_fmks

    m1 = method == "moment_m1"
    hb = random_rad_block_fmks((12, 10, 1), 2, seed=31, vmax=0.0 if m1 else 0.3)
    rp = abi.default_rad_params(method=method)
    p = abi.default_params()
    J0, H0 = hb["rprim"][abi.RJ].copy(), hb["rprim"][abi.RH:abi.RH + 3].copy()
    rad_oracle.MomentPrim2Con(rp, p, hb, *hb.entire())
    E0 = hb["rcons"].copy()
    rad_oracle.MomentCon2Prim(rp, p, hb)
    tol = 1e-8 if m1 else 1e-12
    assert np.all(hb["rprim"][abi.RFAIL] == 1.0)
    assert np.max(np.abs(hb["rprim"][abi.RJ] - J0) / J0) < tol
    assert np.max(np.abs(hb["rprim"][abi.RH:abi.RH + 3] - H0) / np.abs(H0).max()) < tol
    rad_oracle.MomentPrim2Con(rp, p, hb, *hb.entire())
    assert np.max(np.abs(hb["rcons"] - E0) / np.abs(E0[0])) < tol


def test_fmks_geometric_source_equals_fluid_source(rad_oracle):
    """Isotropic radiation at rest (Eddington closure, H = 0, v = 0) has
    T^{mu nu} = (4/3) J u^mu u^nu + (1/3) J g^{mu nu}: the stress tensor of a
    perfect fluid with u = J, P = J / 3, rho = 0.  Its geometric source
    (moments.cpp:764-885) therefore equals the fluid's
    (CalculateFluidSourceTerms, fluid.cpp:566-657) on the same FMKS tables, to
    rounding of the two operation orders."""
    from oracle.oracle import Oracle
    from tests.util import random_rad_block_fmks

    hb = random_rad_block_fmks((10, 8, 1), 2, seed=5, vmax=0.0, hmax=0.0)
    rp = abi.default_rad_params(method="moment_eddington")
    p = abi.default_params(Gamma=4.0 / 3.0)
    J = hb["rprim"][abi.RJ]
    hb["rprim"][abi.RH:abi.RH + 3] = 0.0
    hb["prim"][abi.PVEL:abi.PVEL + 3] = 0.0
    rad_oracle.MomentPrim2Con(rp, p, hb, *hb.entire())
    src_r = rad_oracle.GeometricSource(rp, hb)
    P = hb["prim"]
    P[abi.PRHO] = 0.0
    P[abi.PENG] = J
    P[abi.PPRS] = J / 3.0
    P[abi.PB:abi.PB + 3] = 0.0
    Oracle().CalculateFluidSourceTerms(p, hb)
    src_f = hb["src"]  # S_1..3, tau
    ks, js, is_ = hb.isl()
    big = np.max(np.abs(src_f[:4][:, ks, js, is_]))
    for m_r, m_f, name in ((0, 3, "E / tau"), (1, 0, "F_1"), (2, 1, "F_2")):
        a, b = src_r[m_r][ks, js, is_], src_f[m_f][ks, js, is_]
        err = np.max(np.abs(a - b) / (np.abs(b) + 1e-14 * big))
        print(f"geometric source {name}: max rel {err:.2e}")
        assert err < 1e-10, name
    # d/dphi is a Killing vector of the axisymmetric metric: both F_3 sources
    # vanish, each to the rounding of its own sum
    a, b = src_r[3][ks, js, is_], src_f[2][ks, js, is_]
    print(f"geometric source F_3: max |rad| {np.abs(a).max():.2e}, max |fluid| {np.abs(b).max():.2e} of {big:.2e}")
    assert np.abs(a).max() <= 1e-12 * big and np.abs(b).max() <= 1e-12 * big


# ---- radiation parts of the fixups and floors
def _rad_state(rad_oracle, method, seed=13):
    hb = random_rad_block((16, 12, 1), 2, seed=seed, vmax=0.3)
    p = abi.default_params(Gamma=5.0 / 3.0, Cv=1.0)
    P = hb["prim"]
    P[abi.PPRS] = p.gm1 * P[abi.PENG]
    P[abi.PGM1] = p.gm1 + 1.0
    rp = abi.default_rad_params(method=method)
    rad_oracle.MomentPrim2Con(rp, p, hb, *hb.entire())
    rad_oracle.MomentCon2Prim(rp, p, hb)
    return hb, p, rp


@pytest.mark.parametrize("method", ["moment_m1", "moment_eddington"])
def test_rad_c2p_fixup(rad_oracle, method):
    """RadConservedToPrimitiveFixup (fixup_radc2p.cpp:45-225): a zone marked
    failed takes the mean of its valid face neighbours' J and H / J, and its
    E, F_i become prim2con of those; with no valid neighbour (or the floors
    strategy) J = 10 SMALL, H = 0; valid zones are untouched."""
    hb, p, rp = _rad_state(rad_oracle, method)
    p.enable_c2p_fixup = 1
    R = hb["rprim"]
    k, j0 = 0, hb.ng + 3
    i0 = hb.ng + 4
    R[abi.RFAIL][k, j0, i0] = 0.0             # isolated failure
    R[abi.RFAIL][k, j0 + 5, i0:i0 + 2] = 0.0  # two adjacent failures
    before = {n: hb[n].copy() for n in ("rprim", "rcons")}
    nbrs = [(k, j0, i0 - 1), (k, j0, i0 + 1), (k, j0 - 1, i0), (k, j0 + 1, i0)]
    want_J = np.mean([R[abi.RJ][z] for z in nbrs])
    want_H = [np.mean([R[abi.RH + a][z] for z in nbrs]) for a in range(3)]
    rad_oracle.RadConservedToPrimitiveFixup(rp, p, hb)
    assert hb["rprim"][abi.RJ][k, j0, i0] == pytest.approx(want_J, rel=1e-14)
    for a in range(3):
        assert hb["rprim"][abi.RH + a][k, j0, i0] == pytest.approx(want_H[a], rel=1e-12, abs=1e-15)
    # the pair: each sees three valid neighbours and one failed (contributing nothing)
    z = (k, j0 + 5, i0)
    n3 = [(k, j0 + 5, i0 - 1), (k, j0 + 4, i0), (k, j0 + 6, i0)]
    assert hb["rprim"][abi.RJ][z] == pytest.approx(np.mean([before["rprim"][abi.RJ][q] for q in n3]), rel=1e-14)
    changed = np.any(hb["rprim"] != before["rprim"], axis=0) | np.any(hb["rcons"] != before["rcons"], axis=0)
    assert set(map(tuple, np.argwhere(changed))) <= {(k, j0, i0), (k, j0 + 5, i0), (k, j0 + 5, i0 + 1)}
    # E, F from the fixed primitives
    fresh = hb.to_host()
    rad_oracle.MomentPrim2Con(rp, p, fresh, *fresh.entire())
    np.testing.assert_array_equal(hb["rcons"][:, k, j0, i0], fresh["rcons"][:, k, j0, i0])
    # floors strategy
    hb, p, rp = _rad_state(rad_oracle, method)
    p.enable_c2p_fixup, rp.rad_c2p_failure_floors = 1, 1
    hb["rprim"][abi.RFAIL][k, j0, i0] = 0.0
    rad_oracle.RadConservedToPrimitiveFixup(rp, p, hb)
    assert hb["rprim"][abi.RJ][k, j0, i0] == 10 * 10 * np.finfo(np.float64).tiny
    assert np.all(hb["rprim"][abi.RH:abi.RH + 3, k, j0, i0] == 0.0)


def test_rad_floors_and_ceiling(rad_oracle):
    """The radiation part of ApplyFloors (fixup.cpp:542-678): after it every
    zone has J at or above the J floor (an isotropic normal-observer field
    of the missing J added to E), xi = |H| / J at or below the xi ceiling,
    and zones the floors do not touch keep their state."""
    hb, p, rp = _rad_state(rad_oracle, "moment_m1", seed=17)
    p.enable_floors = 1
    p.rho0_floor, p.sie0_floor = 1e-12, 1e-12  # the fluid floors stay inactive
    J = hb["rprim"][abi.RJ]
    rp.enable_rad_floors, rp.J0_floor = 1, float(np.quantile(J, 0.3))
    rp.enable_rad_ceilings, rp.xi0_ceiling = 1, 0.5
    before = {n: hb[n].copy() for n in ("rprim", "rcons")}
    rad_oracle.ApplyFloors(rp, p, hb)
    R = hb["rprim"]
    assert np.all(R[abi.RJ] >= rp.J0_floor * (1 - 1e-9))
    raised = before["rprim"][abi.RJ] < rp.J0_floor
    assert raised.sum() > 10
    Hr = R[abi.RH:abi.RH + 3]
    P = hb["prim"]
    W = np.sqrt(1 + (P[abi.PVEL:abi.PVEL + 3] ** 2).sum(0))
    v = P[abi.PVEL:abi.PVEL + 3] / W
    xi = np.sqrt((Hr * Hr).sum(0) - (v * Hr).sum(0) ** 2)
    assert np.all(xi <= 0.5 * (1 + 1e-9))
    xb = before["rprim"][abi.RH:abi.RH + 3]
    xi0 = np.sqrt((xb * xb).sum(0) - (v * xb).sum(0) ** 2)
    keep = ~raised & (xi0 <= 0.5)
    np.testing.assert_array_equal(hb["rcons"][:, keep], before["rcons"][:, keep])
