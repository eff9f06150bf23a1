"""The library's written-out exp, log, sin, cos and pow (phoebus_gb300/csrc/
phx_math.h) against the C library, on the CPU through the oracle (which
compiles the same header).  The GPU evaluates the same operations; the GPU
side is tests/test_gpu_math.py.

Bounds (ulp of the C library's result, which is itself within about half an
ulp of the exact value): exp within 1, log, sin, cos within 2; pow within 1
for integer exponents and within 2 |y ln x| + 2 otherwise (exp of the
rounded y ln x).  Special values follow
C: NaN in, NaN out; exp overflow to inf and underflow to 0; log of 0, of a
negative number and of inf; pow(x, 0) = 1.
"""
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def orc(built):
    from oracle.oracle import Oracle

    return Oracle()


def _ulps(got, ref):
    got, ref = np.asarray(got), np.asarray(ref)
    sp = np.spacing(np.abs(ref))
    return np.abs(got - ref) / np.where(sp > 0, sp, 5e-324)


def _libm(fn, x, y=None):
    f = {"exp": math.exp, "log": math.log, "sin": math.sin, "cos": math.cos}
    if fn == "pow":
        return np.array([math.pow(a, b) for a, b in zip(x, y)])
    out = []
    for a in x:
        try:
            out.append(f[fn](a))
        except OverflowError:
            out.append(math.inf)
    return np.array(out)


def test_exp(orc):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.uniform(-700, 700, 20000), rng.uniform(-1, 1, 20000), rng.uniform(-30, 30, 20000),
                        [0.0, -0.0, 1e-300, -1e-300, 0.5 * math.log(2), -0.5 * math.log(2), 709.7, -708.0]])
    got = orc.math_eval("exp", x)
    e = _ulps(got, _libm("exp", x))
    print(f"exp: max {e.max():.2f} ulp")
    assert e.max() <= 1.0
    sp = orc.math_eval("exp", np.array([800.0, -800.0, np.nan, np.inf, -np.inf, -740.0]))
    assert sp[0] == np.inf and sp[1] == 0.0 and np.isnan(sp[2]) and sp[3] == np.inf and sp[4] == 0.0
    assert 0 < sp[5] < 1e-320  # subnormal range


def test_log(orc):
    rng = np.random.default_rng(2)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 20000), rng.uniform(0.5, 2.0, 20000),
                        rng.uniform(1 - 1e-6, 1 + 1e-6, 5000), [1.0, 2.0, 0.5, math.sqrt(2), 5e-324, 1e-310]])
    got = orc.math_eval("log", x)
    ref = _libm("log", x)
    # log near 1 is near 0: measure there in ulps of the argument's distance
    e = _ulps(got, ref)
    near1 = np.abs(ref) < 1e-3
    print(f"log: max {e[~near1].max():.2f} ulp (away from 1), {e[near1].max():.2f} ulp (near 1)")
    assert e[~near1].max() <= 2.0
    assert e[near1].max() <= 2.0
    sp = orc.math_eval("log", np.array([0.0, -1.0, np.inf, np.nan]))
    assert sp[0] == -np.inf and np.isnan(sp[1]) and sp[2] == np.inf and np.isnan(sp[3])


@pytest.mark.parametrize("fn", ["sin", "cos"])
def test_sin_cos(orc, fn):
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-10, 10, 40000), rng.uniform(-1e5, 1e5, 20000), rng.uniform(-1e-8, 1e-8, 2000),
                        np.pi * np.arange(-8, 9) / 4, np.pi * rng.uniform(0, 1, 2000),
                        2 * np.pi * rng.uniform(-0.1, 1.1, 2000)])
    got = orc.math_eval(fn, x)
    ref = _libm(fn, x)
    # near a zero of the function the result is tiny: measure the error
    # against the spacing of 1 (the argument's scale) there
    small = np.abs(ref) < 1e-3
    e = _ulps(got, ref)
    ea = np.abs(got - ref)[small] / np.spacing(1.0)
    print(f"{fn}: max {e[~small].max():.2f} ulp, near zeros {ea.max() if ea.size else 0:.2f} ulp of 1")
    assert e[~small].max() <= 2.0
    assert ea.size == 0 or ea.max() <= 2.0
    assert np.isnan(orc.math_eval(fn, np.array([np.nan, np.inf]))).all()


def test_pow(orc):
    rng = np.random.default_rng(4)
    x = np.concatenate([rng.uniform(-1.3, 1.3, 10000), rng.uniform(0, 50, 10000), [2.0, -2.0, 0.0, 1.5]])
    yint = np.concatenate([np.full(10000, 14.0), rng.integers(-8, 9, 10000).astype(float), [64.0, 3.0, 4.0, 0.0]])
    got = orc.math_eval("pow", x, yint)
    e = _ulps(got, _libm("pow", x, yint))
    print(f"pow (integer exponents): max {e.max():.2f} ulp")
    assert e.max() <= 1.0
    xp = rng.uniform(1e-3, 300, 20000)
    yp = rng.uniform(-3, 3, 20000)
    got = orc.math_eval("pow", xp, yp)
    e = _ulps(got, _libm("pow", xp, yp))
    bound = 2.0 * np.abs(yp * np.log(xp)) + 2.0
    print(f"pow (real exponents): max {e.max():.2f} ulp, max / bound {np.max(e / bound):.3f}")
    assert np.all(e <= bound)
    # the FMKS finite-difference step scale eps^(1/3) and the thJ power
    assert orc.math_eval("pow", np.array([2.220446049250313e-16]), np.array([1.0 / 3.0]))[0] == pytest.approx(
        2.220446049250313e-16 ** (1.0 / 3.0), rel=4e-16)
    sp = orc.math_eval("pow", np.array([-2.0, 0.0, 0.0, np.nan, 3.0]), np.array([0.5, 2.5, -1.5, 1.0, 0.0]))
    assert np.isnan(sp[0]) and sp[1] == 0.0 and sp[2] == np.inf and np.isnan(sp[3]) and sp[4] == 1.0
