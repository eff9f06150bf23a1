"""NumPy restatement of the learned con2prim start network.

TEST INFRASTRUCTURE ONLY (the checker of the GPU training and inference
kernels): imported by tests/ and bench.py's CPU-baseline leg, never by the
product.  The network has no reference counterpart; it supplies the starting
bracket of the reference's unchanged regula-falsi root find
(root_find.hpp:110-167) through its guess argument
(con2prim_robust.hpp:375).

Network: 6 -> 64 -> 64 -> 64 -> 2, GELU (tanh form) after each hidden layer.
Parameters are one FP32 vector in the order W1[64][6], b1[64], W2[64][64],
b2[64], W3[64][64], b3[64], W4[2][64], b4[2] (weights [out][in]).  The
forward pass of training uses BF16-rounded weights and inputs (what the
tensor-core inference multiplies), FP32 everything else.

Outputs: o0 = predicted ln(mu), o1 = ln(sigma) of its error.  Loss: the
Gaussian negative log-likelihood 0.5 (y - o0)^2 exp(-2 o1) + o1 averaged over
the batch, y = ln(mu*) with mu* = 1 / (h W) of the primitive state.
Optimiser: AdamW with decoupled weight decay on the weights only.
"""
from __future__ import annotations

import numpy as np

IN, HID, OUT = 6, 64, 2
SHAPES = [("W1", (HID, IN)), ("b1", (HID,)), ("W2", (HID, HID)), ("b2", (HID,)), ("W3", (HID, HID)),
          ("b3", (HID,)), ("W4", (OUT, HID)), ("b4", (OUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)
GELU_C = np.float32(0.7978845608028654)  # sqrt(2 / pi)
GELU_A = np.float32(0.044715)


def offsets():
    off, o = {}, 0
    for name, shp in SHAPES:
        off[name] = (o, shp)
        o += int(np.prod(shp))
    return off


def unpack(theta: np.ndarray) -> dict:
    return {k: theta[o:o + int(np.prod(s))].reshape(s) for k, (o, s) in offsets().items()}


ROUND_BF16 = True  # False only to check the analytic gradient by finite differences


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round FP32 to the nearest BF16 (ties to even), returned as FP32."""
    if not ROUND_BF16:
        return a
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (u >> np.uint64(16)) & np.uint64(1)
    r = ((u + np.uint64(0x7FFF) + lsb) & np.uint64(0xFFFF0000)).astype(np.uint32)
    nan = np.isnan(a)
    out = r.view(np.float32).copy()
    out[nan] = np.nan
    return out


def init(seed: int = 7) -> np.ndarray:
    """Uniform fan-in initialisation (+-1/sqrt(fan_in)), zero biases."""
    rng = np.random.default_rng(seed)
    th = np.zeros(NPARAM, dtype=np.float32)
    P = unpack(th)
    for k in ("W1", "W2", "W3", "W4"):
        fan = P[k].shape[1]
        P[k][...] = rng.uniform(-1.0, 1.0, P[k].shape).astype(np.float32) / np.float32(np.sqrt(fan))
    return th


def gelu(z):
    t = np.tanh(GELU_C * (z + GELU_A * z * z * z))
    return np.float32(0.5) * z * (np.float32(1.0) + t), t


def gelu_grad(z, t):
    return np.float32(0.5) * (np.float32(1.0) + t) + np.float32(0.5) * z * (np.float32(1.0) - t * t) * GELU_C * (
        np.float32(1.0) + np.float32(3.0) * GELU_A * z * z)


def forward(theta: np.ndarray, x: np.ndarray, keep: bool = False, infer: bool = False):
    """x: [6][n] FP32 -> outputs [2][n] (and the activations when keep).
    infer: also round each hidden activation to BF16, as the tensor-core
    inference does (its A operands are BF16)."""
    P = unpack(theta)
    a0 = bf16_round(x.astype(np.float32))
    acts = [a0]
    zs, ts = [], []
    a = a0
    for l in (1, 2, 3):
        W = bf16_round(P[f"W{l}"])
        z = W @ a + P[f"b{l}"][:, None]
        a, t = gelu(z)
        if infer:
            a = bf16_round(a)
        zs.append(z)
        ts.append(t)
        acts.append(a)
    W4 = bf16_round(P["W4"])
    o = W4 @ a + P["b4"][:, None]
    if keep:
        return o, (acts, zs, ts)
    return o


def loss_and_grad(theta: np.ndarray, x: np.ndarray, y: np.ndarray):
    """Mean NLL over the batch and its gradient (straight through the BF16
    weight rounding)."""
    n = x.shape[1]
    o, (acts, zs, ts) = forward(theta, x, keep=True)
    e = y.astype(np.float32) - o[0]
    s2 = np.exp(np.float32(-2.0) * o[1])
    loss = float(np.mean(np.float32(0.5) * e * e * s2 + o[1]))
    inv_n = np.float32(1.0 / n)
    d = np.stack([-e * s2, np.float32(1.0) - e * e * s2]) * inv_n  # dL/do [2][n]
    P = unpack(theta)
    g = np.zeros_like(theta)
    G = unpack(g)
    G["W4"][...] = d @ acts[3].T
    G["b4"][...] = d.sum(axis=1)
    da = bf16_round(P["W4"]).T @ d
    for l in (3, 2, 1):
        dz = da * gelu_grad(zs[l - 1], ts[l - 1])
        G[f"W{l}"][...] = dz @ acts[l - 1].T
        G[f"b{l}"][...] = dz.sum(axis=1)
        if l > 1:
            da = bf16_round(P[f"W{l}"]).T @ dz
    return loss, g


def weight_mask() -> np.ndarray:
    m = np.zeros(NPARAM, dtype=bool)
    for k, (o, s) in offsets().items():
        if k.startswith("W"):
            m[o:o + int(np.prod(s))] = True
    return m


def adamw(theta, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8, wd=1e-4):
    """One AdamW update in place (step counts from 1)."""
    m[...] = b1 * m + (1 - b1) * g
    v[...] = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    decay = np.where(weight_mask(), wd, 0.0).astype(np.float32)
    theta[...] = theta - lr * (mh / (np.sqrt(vh) + eps) + decay * theta)


def bracket(o: np.ndarray, k: float = 3.0) -> np.ndarray:
    """(m, lo, hi) from the outputs: m = exp(o0) clipped to [0, 1], half-width
    k sigma in ln(mu)."""
    w = k * np.exp(o[1].astype(np.float64))
    c = o[0].astype(np.float64)
    m = np.minimum(np.exp(c), 1.0)
    lo = np.minimum(np.exp(c - w), 1.0)
    hi = np.minimum(np.exp(c + w), 1.0)
    return np.stack([m, lo, hi])
