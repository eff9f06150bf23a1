"""The learned con2prim start: GPU features, tensor-core inference,
training gradients and AdamW against the NumPy oracle; bit-exact parity of
the learned con2prim with the oracle's learned root find; and the gain of the
trained network over the plain start at the same 1e-10 tolerance."""
import numpy as np
import pytest

import oracle.mlp_oracle as M
from phoebus_gb300 import abi, learned, states
from tests.util import assert_bitwise, host

pytestmark = pytest.mark.gpu
N = 40000


def params(tol=1e-10):
    p = abi.default_params(gm1=1.0 / 3.0)
    p.c2p_tol = tol
    p.c2p_max_iter = 100
    return p


def dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def zones(oracle):
    g = learned.kerr_geometry()
    z = states.kerr_zones(N, seed=states.SEED + 42)
    geom = oracle.fmks_points(g, z["x1"], z["x2"])
    prim = np.ascontiguousarray(states.kerr_zone_prims(z, geom))
    cons = oracle.PrimitiveToConservedZones(params(), prim, geom)
    return dict(geom=geom, prim=prim, cons=cons)


@pytest.fixture(scope="module")
def trained_exact(ctx_exact):
    """A network trained on the GPU (exact build) on 2e6 pairs; returns the
    per-epoch losses."""
    losses = learned.train(ctx_exact, params(), n=2_000_000, opts=abi.default_train_opts(epochs=6))
    return losses


def test_features_match_oracle(ctx_exact, oracle, zones):
    got = host(ctx_exact.MLPFeaturesZones(params(), dev(zones["cons"]), dev(zones["geom"])))
    ref = oracle.C2PFeaturesZones(params(), zones["cons"], zones["geom"])
    # FP64 setup is bitwise; the FP32 log10 of CUDA and glibc differ by ulps
    assert np.abs(got - ref).max() <= 1e-6


def test_forward_matches_numpy(ctx_fast, oracle, zones):
    theta = learned.init_weights(11)
    theta[M.offsets()["b4"][0]:] = [-1.0, -2.0]
    ctx_fast.mlp_set_weights(theta)
    x = oracle.C2PFeaturesZones(params(), zones["cons"], zones["geom"])
    got = host(ctx_fast.MLPForward(dev(x)))
    ref = M.forward(theta, x, infer=True)
    d = np.abs(got - ref)
    # BF16 operands, FP32 accumulation in a different order, tanh.approx:
    # an activation may round to the neighbouring BF16 value
    assert np.median(d) < 2e-3 and d.max() < 3e-2, (np.median(d), d.max())


def test_gradient_matches_numpy(ctx_fast):
    rng = np.random.default_rng(5)
    n = 3000
    x = rng.uniform(-1, 1, (6, n)).astype(np.float32)
    y = rng.uniform(-4, 0, n).astype(np.float32)
    theta = learned.init_weights(3)
    ctx_fast.mlp_set_weights(theta)
    loss, grad = ctx_fast.MLPLossGrad(dev(x), dev(y))
    rl, rg = M.loss_and_grad(theta, x, y)
    assert abs(float(loss.item()) - rl) <= 1e-5 * abs(rl) + 1e-6
    g = host(grad)
    for name, (o, shp) in M.offsets().items():
        size = int(np.prod(shp))
        a, b = g[o:o + size], rg[o:o + size]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b) + 1e-9, name


def test_adamw_step_matches_numpy(ctx_fast):
    rng = np.random.default_rng(6)
    n = 4096
    x = rng.uniform(-1, 1, (6, n)).astype(np.float32)
    y = rng.uniform(-4, 0, n).astype(np.float32)
    theta = learned.init_weights(4)
    ctx_fast.mlp_set_weights(theta)
    opts = abi.default_train_opts(batch=n, epochs=1, lr=1e-3)
    losses = ctx_fast.MLPTrain(dev(x), dev(y), opts)
    got = ctx_fast.mlp_get_weights()
    rl, rg = M.loss_and_grad(theta, x, y)
    ref = theta.copy()
    m, v = np.zeros_like(ref), np.zeros_like(ref)
    M.adamw(ref, rg, m, v, 1, 1e-3, wd=1e-4)
    assert abs(losses[0] - rl) <= 1e-5 * abs(rl) + 1e-6
    # first Adam step: lr * g / (|g| + eps): sign-dominated, compare absolutely
    assert np.abs(got - ref).max() <= 2e-6


def test_training_reduces_loss(trained_exact):
    assert trained_exact[-1] < trained_exact[0] - 0.5, trained_exact


def test_learned_con2prim_matches_oracle(ctx_exact, oracle, zones, trained_exact):
    """Exact build: the learned con2prim on the GPU equals the oracle's
    learned root find started from the GPU network's brackets, bit for bit,
    with the same accepted count and iteration total."""
    import torch

    p = params()
    prim0 = zones["prim"].copy()
    prim0[abi.PMU] = 0.0
    br = host(ctx_exact.MLPBracketZones(p, dev(zones["cons"]), dev(zones["geom"])))
    c, pr = dev(zones["cons"]), dev(prim0)
    fail = torch.zeros(N, dtype=torch.float64, device="cuda")
    sig = torch.zeros((3, N), dtype=torch.float64, device="cuda")
    ctx_exact.c2p_stats(reset=True)
    ctx_exact.ConservedToPrimitiveZones(p, c, pr, dev(zones["geom"]), fail=fail, cell_sig=sig, learned=True)
    ctx_exact.check()
    st = ctx_exact.c2p_stats(reset=True)
    rc, rpr = zones["cons"].copy(), prim0.copy()
    rfail, rsig = np.zeros(N), np.zeros((3, N))
    it = np.zeros(N, dtype=np.int32)
    unbr = oracle.ConservedToPrimitiveZones(p, rc, rpr, zones["geom"], fail=rfail, cell_sig=rsig, iters=it,
                                            bracket=np.ascontiguousarray(br))
    assert unbr == 0
    assert_bitwise(pr, rpr, "prim")
    assert_bitwise(c, rc, "cons")
    assert_bitwise(fail, rfail, "fail")
    assert_bitwise(sig, rsig, "cell_sig")
    assert st["learned_accepted"] == oracle.last_accepted
    assert st["iterations"] == int(it.sum())
    assert st["residual_evals"] == oracle.last_evals
    assert oracle.last_accepted > 0.9 * N


def test_learned_gain(ctx_exact, oracle, zones, trained_exact):
    """The trained start needs fewer FP64 residual evaluations than the
    reference's start at the same tolerance, and gives primitives of the
    same accuracy (against the sampled state)."""
    p = params()
    prim0 = zones["prim"].copy()
    prim0[abi.PMU] = 0.0
    br = host(ctx_exact.MLPBracketZones(p, dev(zones["cons"]), dev(zones["geom"])))
    res = {}
    for name, b in (("plain", None), ("learned", np.ascontiguousarray(br))):
        c, pr = zones["cons"].copy(), prim0.copy()
        fail = np.zeros(N)
        it = np.zeros(N, dtype=np.int32)
        oracle.ConservedToPrimitiveZones(p, c, pr, zones["geom"], fail=fail, iters=it, bracket=b)
        res[name] = dict(evals=oracle.last_evals / N, iters=it.mean(), prim=pr, fail=fail)
    assert res["learned"]["evals"] < 0.8 * res["plain"]["evals"], (res["learned"]["evals"], res["plain"]["evals"])
    assert_bitwise(res["learned"]["fail"], res["plain"]["fail"], "fail")
    # same convergence criterion: both end within the tolerance of the root
    # mu* = 1 / (h W) of the sampled state
    truth = zones["prim"]
    h = 1.0 + (truth[abi.PENG] + truth[abi.PPRS]) / truth[abi.PRHO]
    g = zones["geom"]
    wsq = sum(g[abi.G_GCOV + states._flat2(m + 1, k + 1)] * truth[1 + m] * truth[1 + k]
              for m in range(3) for k in range(3))
    mu = 1.0 / (h * np.sqrt(1.0 + wsq))
    for name in ("plain", "learned"):
        assert np.abs(res[name]["prim"][abi.PMU] - mu).max() <= 2.0 * p.c2p_tol, name
    # and primitives of the same statistical accuracy (the largest errors sit
    # in the few zones whose primitives are ill-conditioned in mu)
    for v in (abi.PRHO, abi.PENG, abi.PVEL):
        e_pl = np.abs(res["plain"]["prim"][v] - truth[v]) / (np.abs(truth[v]) + 1e-300)
        e_le = np.abs(res["learned"]["prim"][v] - truth[v]) / (np.abs(truth[v]) + 1e-300)
        assert np.quantile(e_le, 0.999) <= 2.0 * np.quantile(e_pl, 0.999) + 1e-12, v
        assert np.median(e_le) <= 2.0 * np.median(e_pl) + 1e-14, v
