"""The learned con2prim start: training pairs and training, all on the GPU.

Pairs come from the project's own prim2con (phx_prim_to_con_zones) on seeded
Kerr-Schild zones (states.kerr_zones): the network input is the 6 invariants
of the conserved state (phx_mlp_features_zones), the target ln(mu*) with
mu* = 1 / (h W) of the primitive state that produced it -- the root the
reference's con2prim looks for (con2prim_robust.hpp:46-180).  Training is the
library's own forward/backward and AdamW kernels (phx_mlp_train).  The
network has no reference counterpart; it only chooses where the unchanged
FP64 root find starts.
"""
from __future__ import annotations

import numpy as np

from . import abi, states

TRAIN_SEED = states.SEED + 100  # training pairs: a stream separate from every benchmark state


def init_weights(seed: int = 7) -> np.ndarray:
    """Uniform fan-in initialisation (+-1/sqrt(fan_in)) from the SplitMix64
    stream, zero biases."""
    theta = np.zeros(abi.MLP_NPARAM, dtype=np.float32)
    shapes = [(abi.MLP_HID, abi.MLP_IN), (abi.MLP_HID,), (abi.MLP_HID, abi.MLP_HID), (abi.MLP_HID,),
              (abi.MLP_HID, abi.MLP_HID), (abi.MLP_HID,), (abi.MLP_OUT, abi.MLP_HID), (abi.MLP_OUT,)]
    off = 0
    for k, shp in enumerate(shapes):
        size = int(np.prod(shp))
        if len(shp) == 2:
            u = states.uniform(seed, 500 + k, size)
            theta[off:off + size] = ((2.0 * u - 1.0) / np.sqrt(shp[1])).astype(np.float32)
        off += size
    return theta


def kerr_geometry() -> abi.Geometry:
    """FMKS Kerr-Schild with spin 0.9375 and no pole derefinement."""
    return abi.default_geometry(abi.GEOM_FMKS, a=states.KERR_SPIN, derefine_poles=0)


def log_mu(prim, geom):
    """ln(1 / (h W)) of primitives prim[12][n] in metric geom[21][n] (torch):
    h = 1 + u / rho + P / rho, W^2 = 1 + gamma_ij (W v^i)(W v^j)."""
    wsq = 0.0
    for m in range(3):
        for k in range(3):
            wsq = wsq + geom[abi.G_GCOV + states._flat2(m + 1, k + 1)] * prim[1 + m] * prim[1 + k]
    W = (1.0 + wsq) ** 0.5
    h = 1.0 + (prim[abi.PENG] + prim[abi.PPRS]) / prim[abi.PRHO]
    return (-(h * W).log()).to(dtype=prim.dtype)


def kerr_zone_set(ctx, p: abi.Params, n: int, seed: int, device, start: int = 0):
    """n seeded Kerr-Schild zones on the GPU: (prim, cons, geom), cons from
    the library's prim2con."""
    g = kerr_geometry()
    z = states.kerr_zones(n, seed=seed, device=device, start=start, Gamma=p.gm1 + 1.0)
    geom = ctx.GeometryFMKSPoints(g, z["x1"].contiguous(), z["x2"].contiguous())
    prim = states.kerr_zone_prims(z, geom).contiguous()
    cons = ctx.PrimitiveToConservedZones(p, prim, geom)
    return prim, cons, geom


def training_pairs(ctx, p: abi.Params, n: int, seed: int = TRAIN_SEED, device="cuda", chunk: int = 2_000_000):
    """(x [6][n] float32, y [n] float32) on the device, built in chunks."""
    import torch

    x = torch.empty((abi.MLP_IN, n), dtype=torch.float32, device=device)
    y = torch.empty(n, dtype=torch.float32, device=device)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        prim, cons, geom = kerr_zone_set(ctx, p, m, seed, device, start=s)
        x[:, s:s + m] = ctx.MLPFeaturesZones(p, cons, geom)
        y[s:s + m] = log_mu(prim, geom).float()
    return x, y


def train(ctx, p: abi.Params, n: int = 10_000_000, opts: abi.MlpTrainOpts | None = None, seed: int = 7,
          device="cuda"):
    """Initialise, generate n pairs and train; the weights stay loaded in
    ctx.  Returns the per-epoch mean losses."""
    ctx.mlp_set_weights(init_weights(seed))
    x, y = training_pairs(ctx, p, n, device=device)
    return ctx.MLPTrain(x, y, opts)
