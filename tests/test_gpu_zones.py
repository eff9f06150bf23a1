"""Independent zones in FMKS Kerr-Schild geometry (spin 0.9375): point
metric, prim2con and con2prim over a zone list, GPU against the oracle.

The exact build reproduces the oracle bit for bit on identical inputs
(geometry uploaded from the oracle); the production build is compared to
tolerance."""
import numpy as np
import pytest

from phoebus_gb300 import abi, learned, states
from tests.util import assert_bitwise, assert_close, host

pytestmark = pytest.mark.gpu
N = 40000


def params(tol=1e-10):
    p = abi.default_params(gm1=1.0 / 3.0)
    p.c2p_tol = tol
    p.c2p_max_iter = 100
    return p


@pytest.fixture(scope="module")
def zones(oracle):
    """Host zones: numpy draws, oracle metric, oracle prim2con."""
    g = learned.kerr_geometry()
    z = states.kerr_zones(N, seed=states.SEED + 41)
    geom = oracle.fmks_points(g, z["x1"], z["x2"])
    prim = np.ascontiguousarray(states.kerr_zone_prims(z, geom))
    cons = oracle.PrimitiveToConservedZones(params(), prim, geom)
    return dict(z=z, geom=geom, prim=prim, cons=cons, g=g)


def dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_fmks_points(ctx_fast, oracle, zones):
    z = zones["z"]
    got = host(ctx_fast.GeometryFMKSPoints(zones["g"], dev(z["x1"]), dev(z["x2"])))
    # CUDA and glibc transcendental functions differ by ulps; each quantity
    # is compared on its own scale.  Near a pole an ulp of theta is a
    # relative change ulp / theta of sin(theta), squared in the 1 / sin^2
    # components: that amplification is allowed for.
    x2 = z["x2"]
    th = np.pi * x2 + 0.5 * (1.0 - 0.3) * np.sin(2.0 * np.pi * x2)
    amp = 4.0 * np.finfo(float).eps / np.minimum(th, np.pi - th) ** 2
    for v in range(abi.GEOM_NLOC):
        ref = zones["geom"][v]
        lim = 1e-12 * (np.abs(ref) + np.abs(ref).max()) + amp * np.abs(ref)
        bad = ~(np.abs(got[v] - ref) <= lim)
        assert not bad.any(), (v, np.argwhere(bad)[:3].ravel(), got[v][bad][:3], ref[bad][:3])


@pytest.mark.parametrize("exact", [True, False])
def test_prim_to_con_zones(request, oracle, zones, exact):
    ctx = request.getfixturevalue("ctx_exact" if exact else "ctx_fast")
    sig = dev(np.zeros((3, N)))
    got = ctx.PrimitiveToConservedZones(params(), dev(zones["prim"]), dev(zones["geom"]), cell_sig=sig)
    ref_sig = np.zeros((3, N))
    ref = oracle.PrimitiveToConservedZones(params(), zones["prim"], zones["geom"], cell_sig=ref_sig)
    if exact:
        assert_bitwise(got, ref, "cons")
        assert_bitwise(sig, ref_sig, "cell_sig")
    else:
        got, sig = host(got), host(sig)
        for v in range(abi.NCONS):
            assert_close(got[v], ref[v], 1e-13, f"cons[{v}]")
        for d in range(3):
            assert_close(sig[d], ref_sig[d], 1e-13, f"cell_sig[{d}]")


def run_gpu(ctx, p, cons, geom, prim0, learned_start=False):
    import torch

    c, pr = dev(cons), dev(prim0)
    fail = torch.zeros(N, dtype=torch.float64, device="cuda")
    sig = torch.zeros((3, N), dtype=torch.float64, device="cuda")
    ctx.c2p_stats(reset=True)
    ctx.ConservedToPrimitiveZones(p, c, pr, dev(geom), fail=fail, cell_sig=sig, learned=learned_start)
    ctx.check()
    return host(c), host(pr), host(fail), host(sig), ctx.c2p_stats(reset=True)


def run_oracle(oracle, p, cons, geom, prim0, bracket=None):
    c, pr = cons.copy(), prim0.copy()
    fail, sig = np.zeros(N), np.zeros((3, N))
    it = np.zeros(N, dtype=np.int32)
    unbr = oracle.ConservedToPrimitiveZones(p, c, pr, geom, fail=fail, cell_sig=sig, iters=it, bracket=bracket)
    return c, pr, fail, sig, it, unbr


def test_con_to_prim_zones_exact(ctx_exact, oracle, zones):
    p = params()
    prim0 = zones["prim"].copy()
    prim0[abi.PMU] = 0.0
    c, pr, fail, sig, st = run_gpu(ctx_exact, p, zones["cons"], zones["geom"], prim0)
    rc, rpr, rfail, rsig, it, unbr = run_oracle(oracle, p, zones["cons"], zones["geom"], prim0)
    assert unbr == 0 and st["unbracketed"] == 0
    assert_bitwise(pr, rpr, "prim")
    assert_bitwise(c, rc, "cons")
    assert_bitwise(fail, rfail, "fail")
    assert_bitwise(sig, rsig, "cell_sig")
    assert st["zones"] == N
    assert st["iterations"] == int(it.sum())
    assert st["residual_evals"] == oracle.last_evals
    assert st["hist"][:64] == list(np.bincount(it, minlength=128)[:64])


def test_con_to_prim_zones_fast(ctx_fast, oracle, zones):
    """Production build: primitives agree with the oracle within the spread
    that the root-find tolerance itself allows (oracle at 1e-10 against
    the oracle at 1e-15), fail flags bitwise."""
    p = params()
    prim0 = zones["prim"].copy()
    prim0[abi.PMU] = 0.0
    _, pr, fail, _, st = run_gpu(ctx_fast, p, zones["cons"], zones["geom"], prim0)
    _, rpr, rfail, _, _, _ = run_oracle(oracle, p, zones["cons"], zones["geom"], prim0)
    _, tight, _, _, _, _ = run_oracle(oracle, params(1e-15), zones["cons"], zones["geom"], prim0)
    assert_bitwise(fail, rfail, "fail")
    for v in (abi.PRHO, abi.PVEL, abi.PVEL + 1, abi.PVEL + 2, abi.PENG, abi.PPRS):
        scale = np.abs(tight[v]) + 1e-300
        spread = np.max(np.abs(rpr[v] - tight[v]) / scale)
        err = np.max(np.abs(pr[v] - rpr[v]) / scale)
        assert err <= 2.5 * spread + 1e-13, (v, err, spread)
