"""Host API of the GB300 fluid hot path, mirroring the reference's tasks.

The functions keep the names and argument meaning of the phoebus fluid
package tasks (fluid.hpp:27-69) and forward to the C ABI of phx_fluid.h:

    PrimitiveToConserved(Region)   fluid.cpp:359-449
    ConservedToPrimitive(Region)   fluid.cpp:451-517 (robust solver)
    CalculateFluxes                fluid.cpp:659-773
    FluxCT                         fluid.cpp:775-841
    CalculateFluidSourceTerms      fluid.cpp:566-657
    EstimateTimestepBlock          fluid.cpp:899-944
plus the RK stage glue of PhoebusDriver::RungeKuttaStage.  Errors follow the
reference: invalid configuration raises (PARTHENON_THROW), an unbracketed
con2prim root raises on the next check (PARTHENON_FAIL aborts the run).
All work runs on the GPU; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

from . import abi
from .block import Block


def _stream(stream):
    if stream is None:
        import torch

        return torch.cuda.current_stream().cuda_stream
    return getattr(stream, "cuda_stream", stream)


def _tp(t):
    """Device pointer of a contiguous float64 CUDA tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous() or t.dtype.itemsize != 8:
        raise ValueError("expected a contiguous 8-byte CUDA tensor")
    return t.data_ptr()


def _tp4(t):
    """Device pointer of a contiguous float32 CUDA tensor."""
    if not t.is_cuda or not t.is_contiguous() or t.dtype.itemsize != 4:
        raise ValueError("expected a contiguous 4-byte CUDA tensor")
    return t.data_ptr()


def _rng(r):
    return abi.Range(int(r[0]), int(r[1]))


class FluidContext:
    """A phx_ctx on one device, plus the calls that use it."""

    def __init__(self, device: int = 0, exact: bool = False):
        self.lib = abi.load(exact)
        self.exact = exact
        h = C.c_void_p()
        abi.check(self.lib, self.lib.phx_ctx_create(device, C.byref(h)))
        self.h = h
        self.device = device

    def close(self):
        if self.h:
            self.lib.phx_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, st):
        abi.check(self.lib, st)

    # ---- context
    def check(self):
        """Synchronise; raise on a sticky device error (e.g. an unbracketed root)."""
        self._ok(self.lib.phx_ctx_check(self.h))

    def c2p_stats(self, reset: bool = False) -> dict:
        s = abi.C2PStats()
        self._ok(self.lib.phx_ctx_c2p_stats(self.h, C.byref(s), int(reset)))
        return {"zones": s.zones, "iterations": s.iterations, "residual_evals": s.residual_evals,
                "failures": s.failures, "unbracketed": s.unbracketed, "learned_accepted": s.learned_accepted,
                "hist": list(s.hist)}

    # ---- tasks
    def PrimitiveToConserved(self, p: abi.Params, b: Block, ib=None, jb=None, kb=None, stream=None):
        e = b.entire()
        ib, jb, kb = ib or e[0], jb or e[1], kb or e[2]
        s = b.struct()
        self._ok(self.lib.phx_prim_to_con(self.h, C.byref(p), C.byref(s), _rng(ib), _rng(jb), _rng(kb),
                                          _stream(stream)))

    def ConservedToPrimitive(self, p: abi.Params, b: Block, ib=None, jb=None, kb=None, learned=False,
                             stream=None):
        e = b.entire()
        ib, jb, kb = ib or e[0], jb or e[1], kb or e[2]
        s = b.struct()
        fn = self.lib.phx_con_to_prim_learned if learned else self.lib.phx_con_to_prim
        self._ok(fn(self.h, C.byref(p), C.byref(s), _rng(ib), _rng(jb), _rng(kb), _stream(stream)))

    # ---- independent zones: torch CUDA float64 tensors [var][n]
    def PrimitiveToConservedZones(self, p: abi.Params, prim, geom=None, cons=None, cell_sig=None, stream=None):
        import torch

        n = prim.shape[1]
        if cons is None:
            cons = torch.zeros((abi.NCONS, n), dtype=torch.float64, device=prim.device)
        self._ok(self.lib.phx_prim_to_con_zones(self.h, C.byref(p), n, _tp(prim), _tp(geom), _tp(cons),
                                                _tp(cell_sig), _stream(stream)))
        return cons

    def ConservedToPrimitiveZones(self, p: abi.Params, cons, prim, geom=None, fail=None, cell_sig=None,
                                  coords=None, learned=False, stream=None):
        import torch

        n = cons.shape[1]
        if fail is None:
            fail = torch.zeros(n, dtype=torch.float64, device=cons.device)
        self._ok(self.lib.phx_con_to_prim_zones(self.h, C.byref(p), n, _tp(cons), _tp(prim), _tp(geom), _tp(fail),
                                                _tp(cell_sig), _tp(coords), int(learned), _stream(stream)))
        return fail

    # ---- learned con2prim start
    def mlp_set_weights(self, theta):
        import numpy as np

        t = np.ascontiguousarray(theta, dtype=np.float32)
        assert t.size == abi.MLP_NPARAM
        self._ok(self.lib.phx_mlp_set_weights(self.h, t.ctypes.data_as(C.POINTER(C.c_float))))

    def mlp_get_weights(self):
        import numpy as np

        t = np.zeros(abi.MLP_NPARAM, dtype=np.float32)
        self._ok(self.lib.phx_mlp_get_weights(self.h, t.ctypes.data_as(C.POINTER(C.c_float))))
        return t

    def mlp_input_box(self):
        """(lo[6], hi[6]) of the learned start's input box."""
        import numpy as np

        lo, hi = (C.c_float * abi.MLP_IN)(), (C.c_float * abi.MLP_IN)()
        self._ok(self.lib.phx_mlp_get_input_box(self.h, lo, hi))
        return np.array(lo[:], dtype=np.float32), np.array(hi[:], dtype=np.float32)

    def mlp_set_input_box(self, lo=None, hi=None):
        """Set the box (None: that side unbounded)."""
        f = lambda a: None if a is None else (C.c_float * abi.MLP_IN)(*[float(x) for x in a])  # noqa: E731
        self._ok(self.lib.phx_mlp_set_input_box(self.h, f(lo), f(hi)))

    def MLPFeaturesZones(self, p: abi.Params, cons, geom=None, coords=None, x=None, stream=None):
        import torch

        n = cons.shape[1]
        if x is None:
            x = torch.empty((abi.MLP_IN, n), dtype=torch.float32, device=cons.device)
        self._ok(self.lib.phx_mlp_features_zones(self.h, C.byref(p), n, _tp(cons), _tp(geom), _tp(coords),
                                                 _tp4(x), _stream(stream)))
        return x

    def MLPForward(self, x, out=None, stream=None):
        import torch

        n = x.shape[1]
        if out is None:
            out = torch.empty((abi.MLP_OUT, n), dtype=torch.float32, device=x.device)
        self._ok(self.lib.phx_mlp_forward(self.h, n, _tp4(x), _tp4(out), _stream(stream)))
        return out

    def MLPBracketZones(self, p: abi.Params, cons, geom=None, coords=None, out=None, stream=None):
        import torch

        n = cons.shape[1]
        if out is None:
            out = torch.empty((3, n), dtype=torch.float64, device=cons.device)
        self._ok(self.lib.phx_mlp_bracket_zones(self.h, C.byref(p), n, _tp(cons), _tp(geom), _tp(coords),
                                                _tp(out), _stream(stream)))
        return out

    def MLPLossGrad(self, x, y, stream=None):
        import torch

        grad = torch.empty(abi.MLP_NPARAM, dtype=torch.float32, device=x.device)
        loss = torch.empty(1, dtype=torch.float32, device=x.device)
        self._ok(self.lib.phx_mlp_loss_grad(self.h, x.shape[1], _tp4(x), _tp4(y), _tp4(grad), _tp4(loss),
                                            _stream(stream)))
        return loss, grad

    def MLPTrain(self, x, y, opts: abi.MlpTrainOpts | None = None, stream=None):
        """Returns the mean training loss of each epoch."""
        opts = opts or abi.default_train_opts()
        out = (C.c_float * opts.epochs)()
        self._ok(self.lib.phx_mlp_train(self.h, x.shape[1], _tp4(x), _tp4(y), C.byref(opts), out, _stream(stream)))
        return list(out)

    def GeometryFMKSPoints(self, g: abi.Geometry, x1, x2, geom=None, stream=None):
        import torch

        n = x1.shape[0]
        if geom is None:
            geom = torch.empty((abi.GEOM_NLOC, n), dtype=torch.float64, device=x1.device)
        self._ok(self.lib.phx_geometry_fmks_points(self.h, C.byref(g), n, _tp(x1), _tp(x2), _tp(geom),
                                                   _stream(stream)))
        return geom

    def CalculateFluxes(self, p: abi.Params, b: Block, stream=None):
        s = b.struct()
        self._ok(self.lib.phx_calculate_fluxes(self.h, C.byref(p), C.byref(s), _stream(stream)))

    def FluxCT(self, p: abi.Params, b: Block, stream=None):
        s = b.struct()
        self._ok(self.lib.phx_flux_ct(self.h, C.byref(p), C.byref(s), _stream(stream)))

    def CalculateFluidSourceTerms(self, p: abi.Params, blocks, stream=None):
        blocks = blocks if isinstance(blocks, (list, tuple)) else [blocks]
        arr = (abi.BlockS * len(blocks))(*[b.struct() for b in blocks])
        self._ok(self.lib.phx_calculate_fluid_source_terms(self.h, C.byref(p), arr, len(blocks), _stream(stream)))

    def UpdateStage(self, b: Block, cons_base, cons_out, beta: float, dt: float, stream=None):
        from .block import _ptr

        s = b.struct()
        self._ok(self.lib.phx_update_stage(self.h, C.byref(s), _ptr(cons_base), _ptr(cons_out), beta, dt,
                                           _stream(stream)))

    def FillGhostsPeriodic(self, b: Block, field, nvar: int, stream=None):
        from .block import _ptr

        s = b.struct()
        self._ok(self.lib.phx_fill_ghosts_periodic(self.h, C.byref(s), _ptr(field), nvar, _stream(stream)))

    def EstimateTimestepBlock(self, p: abi.Params, b: Block, use_face_speeds: bool, out=None, stream=None):
        """Returns cfl * min dt (a 1-element device tensor; no host sync)."""
        import torch

        if out is None:
            out = torch.zeros(1, dtype=torch.float64, device=f"cuda:{self.device}")
        s = b.struct()
        self._ok(self.lib.phx_estimate_timestep(self.h, C.byref(p), C.byref(s), int(use_face_speeds),
                                                out.data_ptr(), _stream(stream)))
        return out

    def ConservedToPrimitiveFixup(self, p: abi.Params, b: Block, stream=None):
        s = b.struct()
        self._ok(self.lib.phx_c2p_fixup(self.h, C.byref(p), C.byref(s), _stream(stream)))

    def ApplyFloors(self, p: abi.Params, b: Block, ib=None, jb=None, kb=None, stream=None):
        e = b.entire()
        ib, jb, kb = ib or e[0], jb or e[1], kb or e[2]
        s = b.struct()
        self._ok(self.lib.phx_apply_floors(self.h, C.byref(p), C.byref(s), _rng(ib), _rng(jb), _rng(kb),
                                           _stream(stream)))

    def TorusInit(self, p: abi.Params, tp: abi.TorusParams, blocks, stream=None) -> float:
        """The torus problem generator on every block and the field
        normalisation (phx_torus_init); returns the field factor."""
        arr = (abi.BlockS * len(blocks))(*[b.struct() for b in blocks])
        fac = C.c_double()
        self._ok(self.lib.phx_torus_init(self.h, C.byref(p), C.byref(tp), arr, len(blocks), C.byref(fac),
                                         _stream(stream)))
        return fac.value

    def GeometryFillFMKS(self, b: Block, stream=None):
        assert b.geom is not None
        g = b.geom.struct()
        s = b.struct()
        self._ok(self.lib.phx_geometry_fill_fmks(self.h, C.byref(g), C.byref(s), _stream(stream)))

    def Stage(self, p: abi.Params, b: Block, cons_base, cons_out, beta: float, dt: float, learned=False,
              stream=None):
        from .block import _ptr

        s = b.struct()
        self._ok(self.lib.phx_stage(self.h, C.byref(p), C.byref(s), _ptr(cons_base), _ptr(cons_out), beta, dt,
                                    int(learned), _stream(stream)))

    def StageBatched(self, p: abi.Params, blocks, cons_base, cons_out, beta: float, dt: float, learned=False,
                     stream=None):
        """One RK stage over many independent blocks (phx_stage_batched):
        blocks[n]['cons'] is block n's stage input, cons_base[n] / cons_out[n]
        its step-start state and stage output."""
        from .block import _ptr

        n = len(blocks)
        arr = (abi.BlockS * n)(*[b.struct() for b in blocks])
        base = (C.c_void_p * n)(*[_ptr(x) for x in cons_base])
        out = (C.c_void_p * n)(*[_ptr(x) for x in cons_out])
        self._ok(self.lib.phx_stage_batched(self.h, C.byref(p), arr, n, base, out, beta, dt, int(learned),
                                            _stream(stream)))

    def StageMesh(self, p: abi.Params, mesh, blocks, cons_base, cons_out, beta: float, dt: float, learned=False,
                  batched=True, stream=None):
        """One RK stage over a tiled mesh (phx_stage_mesh); mesh: a
        phoebus_gb300.mesh.TiledMesh, blocks in its block order."""
        from .block import _ptr

        n = len(blocks)
        arr = (abi.BlockS * n)(*[b.struct() for b in blocks])
        base = (C.c_void_p * n)(*[_ptr(x) for x in cons_base])
        out = (C.c_void_p * n)(*[_ptr(x) for x in cons_out])
        m = mesh.struct()
        self._ok(self.lib.phx_stage_mesh(self.h, C.byref(p), C.byref(m), arr, n, base, out, beta, dt, int(learned),
                                         int(batched), _stream(stream)))

    def MeshExchange(self, p: abi.Params, mesh, blocks, stream=None):
        """The boundary exchange of a tiled mesh (phx_mesh_exchange)."""
        n = len(blocks)
        arr = (abi.BlockS * n)(*[b.struct() for b in blocks])
        m = mesh.struct()
        self._ok(self.lib.phx_mesh_exchange(self.h, C.byref(p), C.byref(m), arr, n, _stream(stream)))

    def FixFluxes(self, p: abi.Params, mesh, blocks, stream=None):
        """fixup::FixFluxes on the blocks' flux arrays at the mesh's physical
        boundaries (phx_fix_fluxes; a no-op unless p.enable_flux_fixup)."""
        n = len(blocks)
        arr = (abi.BlockS * n)(*[b.struct() for b in blocks])
        m = mesh.struct()
        self._ok(self.lib.phx_fix_fluxes(self.h, C.byref(p), C.byref(m), arr, n, _stream(stream)))

    def FixFluxesBlock(self, p: abi.Params, b: Block, bc_lo, bc_hi, stream=None):
        """fixup::FixFluxes(MeshBlockData*) (phx_fix_fluxes_block): bc_lo /
        bc_hi the boundary kind of each face, abi.BC_PERIODIC where the block
        has a neighbour."""
        lo, hi = (C.c_int * 3)(*bc_lo), (C.c_int * 3)(*bc_hi)
        s = b.struct()
        self._ok(self.lib.phx_fix_fluxes_block(self.h, C.byref(p), C.byref(s), lo, hi, _stream(stream)))

    def batch_info(self) -> dict:
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self._ok(self.lib.phx_batch_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"x1_cells": a.value, "sweep_seg": b.value, "graph_nodes": c.value}

    def probe_fp64_peak(self) -> float:
        v = C.c_double()
        self._ok(self.lib.phx_probe_fp64_peak(self.h, C.byref(v)))
        return v.value

    # ---- composite helpers
    def Initialize(self, p: abi.Params, b: Block, stream=None):
        """Mesh initialisation after a problem generator wrote the prims:
        PrimitiveToConserved (entire), periodic ghost exchange of the
        conserved variables, FillDerived (con2prim, entire)."""
        self.PrimitiveToConserved(p, b, stream=stream)
        self.FillGhostsPeriodic(b, b["cons"], abi.NCONS if p.mhd else 5, stream=stream)
        self.ConservedToPrimitive(p, b, stream=stream)


def rk2_step(ctx: FluidContext, p: abi.Params, b: Block, cons_stage, dt: float, learned=False, stream=None):
    """One Heun RK2 step (rk2 LowStorageIntegrator: beta = 1, 1/2).  b['cons']
    holds U^n on entry and U^{n+1} on exit; cons_stage is the second buffer."""
    base = b["cons"]
    ctx.Stage(p, b, base, cons_stage, 1.0, dt, learned, stream)
    b2 = Block(b.nx, b.ng, b.ndim, b.xmin, b.dx, backend=b.backend, device=b.device, arrays=dict(b.arrays),
               geom=b.geom)
    b2.arrays["cons"] = cons_stage
    ctx.Stage(p, b2, base, base, 0.5, dt, learned, stream)


class MeshRK2:
    """Heun RK2 steps of a tiled mesh through phx_stage_mesh (the rk2
    LowStorageIntegrator: beta = 1, 1/2).  The blocks' 'cons' hold U^n on
    entry and U^{n+1} on exit; the second-stage buffers are allocated once,
    so every step replays the same two cached stage plans."""

    def __init__(self, ctx: FluidContext, p: abi.Params, mesh, blocks):
        import torch

        self.ctx, self.p, self.mesh, self.blocks = ctx, p, mesh, blocks
        self.bases = [b["cons"] for b in blocks]
        self.seconds = [torch.zeros_like(b["cons"]) for b in blocks]
        self.stage2 = []
        for b, s2 in zip(blocks, self.seconds):
            c = Block(b.nx, b.ng, b.ndim, b.xmin, b.dx, backend=b.backend, device=b.device, arrays=dict(b.arrays),
                      geom=b.geom)
            c.arrays["cons"] = s2
            self.stage2.append(c)

    def step(self, dt: float, learned=False, batched=True, stream=None):
        self.ctx.StageMesh(self.p, self.mesh, self.blocks, self.bases, self.seconds, 1.0, dt, learned, batched,
                           stream)
        self.ctx.StageMesh(self.p, self.mesh, self.stage2, self.bases, self.bases, 0.5, dt, learned, batched, stream)

    def initialize(self, stream=None):
        """After a problem generator wrote the primitives (entire blocks):
        PrimitiveToConserved, the mesh's boundary exchange, FillDerived."""
        for b in self.blocks:
            self.ctx.PrimitiveToConserved(self.p, b, stream=stream)
        self.ctx.MeshExchange(self.p, self.mesh, self.blocks, stream)
        for b in self.blocks:
            self.ctx.ConservedToPrimitive(self.p, b, stream=stream)

    def estimate_dt(self, use_face_speeds: bool) -> float:
        return min(self.ctx.EstimateTimestepBlock(self.p, b, use_face_speeds).item() for b in self.blocks)
