"""CPU checks of the learned-start checkers: the NumPy network's analytic
gradient against finite differences, its BF16 rounding, the oracle's
zone-list con2prim round trip on Kerr-Schild zones, and the oracle's
learned root find (a good bracket saves evaluations, a bad one falls back to
the reference's start with the same root)."""
import numpy as np
import pytest

import oracle.mlp_oracle as M
from phoebus_gb300 import abi, learned, states

N = 4000


def params(tol=1e-10):
    p = abi.default_params(gm1=1.0 / 3.0)
    p.c2p_tol = tol
    p.c2p_max_iter = 100
    return p


def test_bf16_round_known_values():
    # BF16 keeps 7 fraction bits: the spacing at 1 is 2^-7
    x = np.array([1.0, 1.0 + 2.0 ** -7, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, 1.0 + 3 * 2.0 ** -8, -2.5, 0.0,
                  3.0e38], dtype=np.float32)
    r = M.bf16_round(x)
    # ties go to the even neighbour: 1 + 2^-8 -> 1, 1 + 3 * 2^-8 -> 1 + 2^-6
    assert list(r[:7]) == [1.0, 1.0 + 2.0 ** -7, 1.0, 1.0 + 2.0 ** -7, 1.0 + 2.0 ** -6, -2.5, 0.0]
    assert np.isfinite(r[7])


def test_gradient_finite_differences(monkeypatch):
    monkeypatch.setattr(M, "ROUND_BF16", False)
    rng = np.random.default_rng(0)
    th = M.init(3).astype(np.float64)
    x = rng.standard_normal((6, 17))
    y = rng.uniform(-4, 0, 17)
    _, g = M.loss_and_grad(th, x, y)
    for i in rng.choice(M.NPARAM, 40, replace=False):
        h = 1e-6
        tp, tm = th.copy(), th.copy()
        tp[i] += h
        tm[i] -= h
        fd = (M.loss_and_grad(tp, x, y)[0] - M.loss_and_grad(tm, x, y)[0]) / (2 * h)
        assert abs(g[i] - fd) <= 1e-5 * max(abs(fd), 1e-3), (i, g[i], fd)


def test_init_weights_layout():
    th = learned.init_weights(7)
    assert th.shape == (abi.MLP_NPARAM,) and M.NPARAM == abi.MLP_NPARAM
    P = M.unpack(th)
    assert np.abs(P["W2"]).max() <= 1.0 / 8.0 and np.all(P["b2"] == 0.0)


@pytest.fixture(scope="module")
def zones(oracle):
    g = learned.kerr_geometry()
    z = states.kerr_zones(N, seed=states.SEED + 43)
    geom = oracle.fmks_points(g, z["x1"], z["x2"])
    prim = np.ascontiguousarray(states.kerr_zone_prims(z, geom))
    cons = oracle.PrimitiveToConservedZones(params(), prim, geom)
    h = 1.0 + (prim[abi.PENG] + prim[abi.PPRS]) / prim[abi.PRHO]
    wsq = sum(geom[abi.G_GCOV + states._flat2(m + 1, k + 1)] * prim[1 + m] * prim[1 + k]
              for m in range(3) for k in range(3))
    mu = 1.0 / (h * np.sqrt(1.0 + wsq))
    return dict(geom=geom, prim=prim, cons=cons, mu=mu)


def solve(oracle, zones, bracket=None, tol=1e-10):
    pr = zones["prim"].copy()
    pr[abi.PMU] = 0.0
    fail = np.zeros(N)
    it = np.zeros(N, dtype=np.int32)
    unbr = oracle.ConservedToPrimitiveZones(params(tol), zones["cons"].copy(), pr, zones["geom"], fail=fail,
                                            iters=it, bracket=bracket)
    return pr, fail, unbr, oracle.last_evals / N, oracle.last_accepted


def test_round_trip(oracle, zones):
    pr, fail, unbr, evals, _ = solve(oracle, zones)
    assert unbr == 0 and fail.min() == 1.0
    assert np.abs(pr[abi.PMU] - zones["mu"]).max() <= 2e-10  # |mu - root| <= tol at exit
    rel = np.abs(pr[abi.PRHO] - zones["prim"][abi.PRHO]) / zones["prim"][abi.PRHO]
    assert np.median(rel) < 1e-12 and rel.max() < 1e-5
    assert 8.0 < evals < 16.0


def test_learned_root_find_good_and_bad_brackets(oracle, zones):
    mu = zones["mu"]
    _, _, _, plain_evals, _ = solve(oracle, zones)
    good = np.ascontiguousarray(np.stack([mu, mu * np.exp(-1e-3), np.minimum(mu * np.exp(1e-3), 1.0)]))
    pr, fail, unbr, evals, acc = solve(oracle, zones, good)
    assert acc == N and unbr == 0 and fail.min() == 1.0
    assert evals < 0.7 * plain_evals
    assert np.abs(pr[abi.PMU] - mu).max() <= 2e-10
    # a bracket that misses the root is rejected: the reference start decides
    bad = np.ascontiguousarray(np.stack([mu * 0.5, mu * 0.4, mu * 0.6]))
    pr2, fail2, unbr2, evals2, acc2 = solve(oracle, zones, bad)
    ref, _, _, _, _ = solve(oracle, zones)
    assert acc2 == 0 and unbr2 == 0
    assert np.array_equal(pr2, ref)
    assert evals2 == pytest.approx(plain_evals + 2.0)
    # NaN brackets are not tried at all
    nan = np.full((3, N), np.nan)
    pr3, _, _, evals3, acc3 = solve(oracle, zones, nan)
    assert acc3 == 0 and evals3 == pytest.approx(plain_evals) and np.array_equal(pr3, ref)


def test_learned_start_only_for_cold_zones(oracle, zones):
    """A zone with a previous solution (guess > 0) keeps the reference's
    warm start even when a learned bracket is given."""
    mu = zones["mu"]
    good = np.ascontiguousarray(np.stack([mu, mu * np.exp(-1e-3), np.minimum(mu * np.exp(1e-3), 1.0)]))
    guess = np.ascontiguousarray(mu * (1.0 + 1e-6))
    pr = zones["prim"].copy()
    fail = np.zeros(N)
    oracle.ConservedToPrimitiveZones(params(), zones["cons"].copy(), pr, zones["geom"], fail=fail, guess=guess,
                                     bracket=good)
    assert oracle.last_accepted == 0
    pr2 = zones["prim"].copy()
    oracle.ConservedToPrimitiveZones(params(), zones["cons"].copy(), pr2, zones["geom"], fail=fail, guess=guess)
    assert np.array_equal(pr, pr2)
