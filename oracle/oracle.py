"""ctypes wrapper of the CPU oracle (oracle/phx_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker.  The product never loads it.

The task functions mirror phoebus_gb300.fluid.FluidContext on host (numpy)
Blocks, so a parity test runs the same sequence on both sides.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
import sys  # noqa: E402

if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
from phoebus_gb300 import abi  # noqa: E402  (struct layouts only)
from phoebus_gb300.block import Block  # noqa: E402

LIB = ROOT / "oracle" / "_build" / "libphx_oracle.so"
SRC = ROOT / "oracle" / "phx_oracle.cpp"


LIB_TUNED = ROOT / "oracle" / "_build" / "libphx_oracle_tuned.so"


def build(force: bool = False) -> Path:
    """Both oracle builds (phoebus_gb300/build.py: the parity build with
    contraction off, and the -O3 timing build)."""
    from phoebus_gb300.build import build_oracle

    return build_oracle(force)


_libs = {}


def lib(tuned: bool = False) -> C.CDLL:
    """The parity build, or with tuned the timing build (CPU baseline only:
    its contracted arithmetic rounds differently)."""
    if tuned not in _libs:
        build()
        L = C.CDLL(str(LIB_TUNED if tuned else LIB))
        P, B, R = C.POINTER(abi.Params), C.POINTER(abi.BlockS), abi.Range
        L.orc_prim_to_con.argtypes = [P, B, R, R, R]
        L.orc_prim_to_con.restype = None
        L.orc_con_to_prim.argtypes = [P, B, R, R, R, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_con_to_prim.restype = C.c_longlong
        L.orc_calculate_fluxes.argtypes = [P, B]
        L.orc_calculate_fluxes.restype = None
        L.orc_flux_ct.argtypes = [B]
        L.orc_flux_ct.restype = None
        L.orc_sources.argtypes = [P, B]
        L.orc_sources.restype = None
        L.orc_flux_divergence.argtypes = [P, B]
        L.orc_flux_divergence.restype = None
        L.orc_update.argtypes = [P, B, C.c_void_p, C.c_void_p, C.c_double, C.c_double]
        L.orc_update.restype = None
        L.orc_fill_ghosts_periodic.argtypes = [B, C.c_void_p, C.c_int]
        L.orc_fill_ghosts_periodic.restype = None
        L.orc_estimate_timestep.argtypes = [P, B, C.c_int]
        L.orc_estimate_timestep.restype = C.c_double
        L.orc_geometry_fill_fmks.argtypes = [C.POINTER(abi.Geometry), B]
        L.orc_geometry_fill_fmks.restype = None
        L.orc_fmks_point.argtypes = [C.POINTER(abi.Geometry), C.c_double, C.c_double, C.c_double, C.c_void_p]
        L.orc_fmks_point.restype = None
        L.orc_c2p_fixup.argtypes = [P, B]
        L.orc_c2p_fixup.restype = None
        L.orc_apply_floors.argtypes = [P, B, R, R, R]
        L.orc_apply_floors.restype = C.c_longlong
        L.orc_prim_to_con_zones.argtypes = [P, C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_prim_to_con_zones.restype = None
        L.orc_con_to_prim_zones.argtypes = [P, C.c_longlong] + [C.c_void_p] * 11
        L.orc_con_to_prim_zones.restype = C.c_longlong
        L.orc_c2p_features_zones.argtypes = [P, C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_c2p_features_zones.restype = None
        L.orc_fmks_points.argtypes = [C.POINTER(abi.Geometry), C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_fmks_points.restype = None
        RP, PP, BS, RB = C.POINTER(abi.RadParams), C.POINTER(abi.Params), C.POINTER(abi.BlockS), C.POINTER(abi.RadBlockS)
        for name, args, res in [
            ("orc_rad_prim_to_con", [RP, PP, BS, RB, abi.Range, abi.Range, abi.Range], None),
            ("orc_rad_con_to_prim", [RP, PP, BS, RB, abi.Range, abi.Range, abi.Range], None),
            ("orc_rad_calculate_opacities", [RP, PP, BS, RB], None),
            ("orc_rad_calculate_fluxes", [RP, PP, BS, RB], None),
            ("orc_rad_update", [RP, BS, RB, C.c_void_p, C.c_void_p, C.c_double, C.c_double], None),
            ("orc_rad_geometric_source", [RP, BS, RB, C.c_void_p], None),
            ("orc_rad_c2p_fixup", [RP, PP, BS, RB], None),
            ("orc_rad_apply_floors", [RP, PP, BS, RB, abi.Range, abi.Range, abi.Range], None),
            ("orc_rad_fluid_source", [RP, PP, BS, RB, C.c_double], C.c_longlong),
            ("orc_rad_fill_ghosts_periodic", [BS, RB], None),
            ("orc_rad_estimate_timestep", [RP, PP, BS, RB], C.c_double),
            ("orc_rad_tanh", [C.c_double], C.c_double),
            ("orc_math_eval", [C.c_int, C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p], None),
            ("orc_con_to_prim_zones_at_mu", [PP, C.c_longlong] + [C.c_void_p] * 5, None),
            ("orc_torus_init", [PP, C.POINTER(abi.TorusParams), C.POINTER(abi.BlockS), C.c_int,
                                C.POINTER(C.c_double)], None),
            ("orc_rad_m1_guess", [C.c_void_p] * 3 + [C.c_longlong] + [C.c_void_p] * 2, None),
        ]:
            fn = getattr(L, name)
            fn.argtypes, fn.restype = args, res
        _libs[tuned] = L
    return _libs[tuned]


def _r(r):
    return abi.Range(int(r[0]), int(r[1]))


def set_threads(n: int | None):
    if n:
        os.environ["OMP_NUM_THREADS"] = str(n)


class Oracle:
    """The reference tasks on host Blocks (numpy arrays).  tuned selects the
    -O3 timing build (for the CPU baseline; the tests use the parity build)."""

    def __init__(self, tuned: bool = False):
        self.L = lib(tuned)

    def PrimitiveToConserved(self, p, b: Block, ib=None, jb=None, kb=None):
        e = b.entire()
        s = b.struct()
        self.L.orc_prim_to_con(C.byref(p), C.byref(s), _r(ib or e[0]), _r(jb or e[1]), _r(kb or e[2]))

    def ConservedToPrimitive(self, p, b: Block, ib=None, jb=None, kb=None, iters=None, guess=None):
        """Returns the number of unbracketed zones.  iters: optional int32
        array shaped like one field, receiving iteration counts."""
        e = b.entire()
        s = b.struct()
        it = iters.ctypes.data if iters is not None else None
        gs = guess.ctypes.data if guess is not None else None
        ev = C.c_longlong()
        n = self.L.orc_con_to_prim(C.byref(p), C.byref(s), _r(ib or e[0]), _r(jb or e[1]), _r(kb or e[2]), it, gs,
                                   C.byref(ev))
        self.last_evals = ev.value
        return n

    def CalculateFluxes(self, p, b: Block):
        s = b.struct()
        self.L.orc_calculate_fluxes(C.byref(p), C.byref(s))

    def FluxCT(self, p, b: Block):
        if not p.mhd or b.ndim == 1:
            return
        s = b.struct()
        self.L.orc_flux_ct(C.byref(s))

    def CalculateFluidSourceTerms(self, p, b: Block):
        s = b.struct()
        self.L.orc_sources(C.byref(p), C.byref(s))

    def FluxDivergence(self, p, b: Block):
        s = b.struct()
        self.L.orc_flux_divergence(C.byref(p), C.byref(s))

    def Update(self, p, b: Block, base, out, beta, dt):
        s = b.struct()
        self.L.orc_update(C.byref(p), C.byref(s), base.ctypes.data, out.ctypes.data, beta, dt)

    def FillGhostsPeriodic(self, b: Block, field, nvar):
        s = b.struct()
        self.L.orc_fill_ghosts_periodic(C.byref(s), field.ctypes.data, nvar)

    def EstimateTimestepBlock(self, p, b: Block, use_face_speeds: bool) -> float:
        s = b.struct()
        return self.L.orc_estimate_timestep(C.byref(p), C.byref(s), int(use_face_speeds))

    def ConservedToPrimitiveFixup(self, p, b: Block):
        s = b.struct()
        self.L.orc_c2p_fixup(C.byref(p), C.byref(s))

    def ApplyFloors(self, p, b: Block, ib=None, jb=None, kb=None):
        e = b.entire()
        s = b.struct()
        return self.L.orc_apply_floors(C.byref(p), C.byref(s), _r(ib or e[0]), _r(jb or e[1]), _r(kb or e[2]))

    def GeometryFillFMKS(self, b: Block):
        g = b.geom.struct()
        s = b.struct()
        self.L.orc_geometry_fill_fmks(C.byref(g), C.byref(s))

    def fmks_point(self, g, X1, X2, X3=0.0):
        out = np.zeros(abi.GEOM_NLOC)
        self.L.orc_fmks_point(C.byref(g), X1, X2, X3, out.ctypes.data)
        return out

    # ---- independent zones (arrays [var][n], C-contiguous float64)
    @staticmethod
    def _p(a):
        if a is None:
            return None
        assert a.dtype == np.float64 and a.flags.c_contiguous
        return a.ctypes.data

    def PrimitiveToConservedZones(self, p, prim, geom=None, cons=None, cell_sig=None):
        n = prim.shape[1]
        if cons is None:
            cons = np.zeros((abi.NCONS, n))
        self.L.orc_prim_to_con_zones(C.byref(p), n, self._p(prim), self._p(geom), self._p(cons), self._p(cell_sig))
        return cons

    def ConservedToPrimitiveZones(self, p, cons, prim, geom=None, fail=None, cell_sig=None, coords=None,
                                  iters=None, guess=None, bracket=None):
        """In place on prim (and cons where bounds applied).  Returns the
        number of unbracketed zones; self.last_evals = residual evaluations,
        self.last_accepted = learned brackets accepted.  bracket: optional
        [3][n] learned starts (m, lo, hi)."""
        n = cons.shape[1]
        if fail is None:
            fail = np.zeros(n)
        ev, acc = C.c_longlong(), C.c_longlong()
        it = iters.ctypes.data if iters is not None else None
        r = self.L.orc_con_to_prim_zones(C.byref(p), n, self._p(cons), self._p(prim), self._p(geom), self._p(fail),
                                         self._p(cell_sig), self._p(coords), it, self._p(guess), self._p(bracket),
                                         C.byref(ev), C.byref(acc))
        self.last_evals = ev.value
        self.last_accepted = acc.value
        return r

    def ConservedToPrimitiveZonesAtMu(self, p, cons, prim, mu, geom=None):
        """The reference's con2prim finish at the given roots (no root find),
        in place on prim (and cons where bounds applied); returns the fail
        flags."""
        n = cons.shape[1]
        fail = np.zeros(n)
        self.L.orc_con_to_prim_zones_at_mu(C.byref(p), n, self._p(cons), self._p(prim), self._p(geom),
                                           self._p(np.ascontiguousarray(mu, dtype=np.float64)), fail.ctypes.data)
        return fail

    def C2PFeaturesZones(self, p, cons, geom=None, coords=None):
        """The learned start's FP32 inputs [6][n]."""
        n = cons.shape[1]
        x = np.zeros((abi.MLP_IN, n), dtype=np.float32)
        self.L.orc_c2p_features_zones(C.byref(p), n, self._p(cons), self._p(geom), self._p(coords), x.ctypes.data)
        return x

    def math_eval(self, fn: str, x, y=None):
        """phx_math.h's exp / log / sin / cos / pow over a float64 array."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        yy = None if y is None else np.ascontiguousarray(y, dtype=np.float64)
        out = np.empty_like(x)
        self.L.orc_math_eval(abi.MATH[fn], x.size, x.ctypes.data, None if yy is None else yy.ctypes.data,
                             out.ctypes.data)
        return out

    def TorusInit(self, p, tp, blocks) -> float:
        """pgen/torus.cpp's ProblemGenerator on every block and the field
        normalisation of PostInitializationModifier; returns the factor."""
        arr = (abi.BlockS * len(blocks))(*[b.struct() for b in blocks])
        # the structs point at each block's geometry struct: keep them alive
        keep = [b._gstruct for b in blocks]
        fac = C.c_double()
        self.L.orc_torus_init(C.byref(p), C.byref(tp), arr, len(blocks), C.byref(fac))
        del keep
        return fac.value

    def fmks_points(self, g, x1, x2):
        n = x1.shape[0]
        out = np.zeros((abi.GEOM_NLOC, n))
        self.L.orc_fmks_points(C.byref(g), n, self._p(np.ascontiguousarray(x1)), self._p(np.ascontiguousarray(x2)),
                               out.ctypes.data)
        return out

    # ---- composite sequences (same order as the GPU host API)
    def _exchange(self, p, b: Block, exchange):
        if exchange is None:
            self.FillGhostsPeriodic(b, b["cons"], abi.NCONS if p.mhd else 5)
        else:
            exchange(b)

    def Initialize(self, p, b: Block, exchange=None):
        """exchange(b): the ghost exchange of b's current arrays; None = the
        periodic exchange of the conserved variables."""
        self.PrimitiveToConserved(p, b)
        self._exchange(p, b, exchange)
        return self.ConservedToPrimitive(p, b)

    def Stage(self, p, b: Block, base, out, beta, dt, exchange=None):
        """PhoebusDriver::RungeKuttaStage for one block: sources, fluxes,
        FluxCT, divergence + update, con2prim (entire), ghost exchange,
        con2prim (entire).  b['cons'] is the stage input."""
        self.CalculateFluidSourceTerms(p, b)
        self.CalculateFluxes(p, b)
        self.FluxCT(p, b)
        self.FluxDivergence(p, b)
        self.Update(p, b, base, out, beta, dt)
        cons_in = b.arrays["cons"]
        b.arrays["cons"] = out
        unbr = self.ConservedToPrimitive(p, b)
        self.ConservedToPrimitiveFixup(p, b)
        self.ApplyFloors(p, b)
        self._exchange(p, b, exchange)
        unbr += self.ConservedToPrimitive(p, b)
        self.ConservedToPrimitiveFixup(p, b)
        self.ApplyFloors(p, b)
        b.arrays["cons"] = cons_in
        return unbr

    def rk2_step(self, p, b: Block, cons_stage, dt, exchange=None):
        base = b.arrays["cons"]
        self.Stage(p, b, base, cons_stage, 1.0, dt, exchange)
        b.arrays["cons"] = cons_stage
        self.Stage(p, b, base, base, 0.5, dt, exchange)
        b.arrays["cons"] = base


class RadOracle:
    """The reference's radiation moment tasks on host Blocks (numpy arrays
    "prim" ... and "rcons", "rprim", "rflux", "rdudt"), in the order of
    phoebus_gb300.radiation.RadiationContext."""

    def __init__(self, tuned: bool = False):
        self.L = lib(tuned)

    @staticmethod
    def _s(b: Block, cons=None):
        from phoebus_gb300.radiation import rad_struct

        return b.struct(), rad_struct(b, cons)

    def MomentPrim2Con(self, rp, p, b: Block, ib=None, jb=None, kb=None):
        e = b.interior()
        s, r = self._s(b)
        self.L.orc_rad_prim_to_con(C.byref(rp), C.byref(p), C.byref(s), C.byref(r), _r(ib or e[0]), _r(jb or e[1]),
                                   _r(kb or e[2]))

    def MomentCon2Prim(self, rp, p, b: Block, ib=None, jb=None, kb=None):
        e = b.entire()
        s, r = self._s(b)
        self.L.orc_rad_con_to_prim(C.byref(rp), C.byref(p), C.byref(s), C.byref(r), _r(ib or e[0]), _r(jb or e[1]),
                                   _r(kb or e[2]))

    def MomentCalculateOpacities(self, rp, p, b: Block):
        s, r = self._s(b)
        self.L.orc_rad_calculate_opacities(C.byref(rp), C.byref(p), C.byref(s), C.byref(r))

    def CalculateFluxes(self, rp, p, b: Block):
        s, r = self._s(b)
        self.L.orc_rad_calculate_fluxes(C.byref(rp), C.byref(p), C.byref(s), C.byref(r))

    def Update(self, rp, b: Block, base, out, beta, dt):
        s, r = self._s(b)
        self.L.orc_rad_update(C.byref(rp), C.byref(s), C.byref(r), base.ctypes.data, out.ctypes.data, beta, dt)

    def GeometricSource(self, rp, b: Block):
        """CalculateGeometricSource over the interior: [4][k][j][i] (zero on
        Minkowski blocks)."""
        s, r = self._s(b)
        out = np.zeros((abi.RNCONS,) + b.shape)
        self.L.orc_rad_geometric_source(C.byref(rp), C.byref(s), C.byref(r), out.ctypes.data)
        return out

    def RadConservedToPrimitiveFixup(self, rp, p, b: Block):
        s, r = self._s(b)
        self.L.orc_rad_c2p_fixup(C.byref(rp), C.byref(p), C.byref(s), C.byref(r))

    def ApplyFloors(self, rp, p, b: Block, ib=None, jb=None, kb=None):
        """fixup::ApplyFloors with radiation active: the fluid part, then
        (rp.enable_rad_floors) the radiation part."""
        e = b.entire()
        s, r = self._s(b)
        self.L.orc_rad_apply_floors(C.byref(rp), C.byref(p), C.byref(s), C.byref(r), _r(ib or e[0]), _r(jb or e[1]),
                                    _r(kb or e[2]))

    def MomentFluidSource(self, rp, p, b: Block, dt) -> int:
        s, r = self._s(b)
        return self.L.orc_rad_fluid_source(C.byref(rp), C.byref(p), C.byref(s), C.byref(r), dt)

    def FillGhostsPeriodic(self, b: Block):
        s, r = self._s(b)
        self.L.orc_rad_fill_ghosts_periodic(C.byref(s), C.byref(r))

    def EstimateTimestepBlock(self, rp, p, b: Block) -> float:
        s, r = self._s(b)
        return self.L.orc_rad_estimate_timestep(C.byref(rp), C.byref(p), C.byref(s), C.byref(r))

    def tanh(self, x: float) -> float:
        return self.L.orc_rad_tanh(x)

    def M1GuessesFromEddington(self, E, F, v):
        """ClosureM1::GetM1GuessesFromEddington for arrays E [n], F [3][n],
        coordinate velocity v [3][n]; returns (xi [n], phi [n])."""
        E, F, v = (np.ascontiguousarray(a, dtype=np.float64) for a in (E, F, v))
        n = E.shape[0]
        xi, phi = np.zeros(n), np.zeros(n)
        self.L.orc_rad_m1_guess(E.ctypes.data, F.ctypes.data, v.ctypes.data, n, xi.ctypes.data, phi.ctypes.data)
        return xi, phi

    def Initialize(self, rp, p, b: Block):
        self.FillGhostsPeriodic(b)
        self.MomentCon2Prim(rp, p, b)

    def Stage(self, rp, p, b: Block, base, out, beta, dt):
        """PhoebusDriver::RungeKuttaStage with the fluid not evolved
        (phoebus_driver.cpp:349-362, 547-620, 640-668): opacities, fluxes,
        update into out, con2prim, RadConservedToPrimitiveFixup, ApplyFloors,
        the implicit source over beta dt, ApplyFloors, ghost exchange,
        con2prim, fixup and floors again (each fixup and floor as p / rp
        enable it).  b['rcons'] is the stage input."""
        self.MomentCalculateOpacities(rp, p, b)
        self.CalculateFluxes(rp, p, b)
        self.Update(rp, b, base, out, beta, dt)
        cons_in = b.arrays["rcons"]
        b.arrays["rcons"] = out

        def derived(first):  # FillDerived (hydro off: the moments alone), the fixup, the floors
            if first and not p.enable_c2p_fixup:  # the ghosts' inversion is overwritten unread
                self.MomentCon2Prim(rp, p, b, *b.interior())
            else:
                self.MomentCon2Prim(rp, p, b)
            self.RadConservedToPrimitiveFixup(rp, p, b)
            self.ApplyFloors(rp, p, b)

        derived(True)
        self.MomentFluidSource(rp, p, b, beta * dt)
        self.ApplyFloors(rp, p, b)
        self.FillGhostsPeriodic(b)
        derived(False)
        b.arrays["rcons"] = cons_in

    def rk2_step(self, rp, p, b: Block, stage_buf, dt):
        base = b.arrays["rcons"]
        self.Stage(rp, p, b, base, stage_buf, 1.0, dt)
        b.arrays["rcons"] = stage_buf
        self.Stage(rp, p, b, base, base, 0.5, dt)
        b.arrays["rcons"] = base

    def FluidStage(self, rp, p, b: Block, fbase, fout, rbase, rout, beta, dt):
        """PhoebusDriver::RungeKuttaStage with the fluid and the moments
        active on one periodic block (phoebus_driver.cpp:318-362, 547-620,
        640-680): fluid source terms, fluxes, FluxCT, opacities, moment
        fluxes; both updates; FillDerived (fluid con2prim over the entire
        block, then MomentCon2Prim), the fluid and radiation c2p fixups,
        ApplyFloors; MomentFluidSource(update_fluid = true) over beta dt;
        ApplyFloors; the periodic exchange of the fluid's conserved variables
        and the radiation fields; FillDerived, fixups and floors again.
        b['cons'] and b['rcons'] are the stage inputs."""
        import copy

        orc = Oracle()
        orc.L = self.L
        orc.CalculateFluidSourceTerms(p, b)
        orc.CalculateFluxes(p, b)
        orc.FluxCT(p, b)
        self.MomentCalculateOpacities(rp, p, b)
        self.CalculateFluxes(rp, p, b)
        orc.FluxDivergence(p, b)
        orc.Update(p, b, fbase, fout, beta, dt)
        self.Update(rp, b, rbase, rout, beta, dt)
        fin, rin = b.arrays["cons"], b.arrays["rcons"]
        b.arrays["cons"], b.arrays["rcons"] = fout, rout

        def derived():  # FillDerived, ConservedToPrimitiveFixup, RadConservedToPrimitiveFixup, ApplyFloors
            orc.ConservedToPrimitive(p, b)
            self.MomentCon2Prim(rp, p, b)
            orc.ConservedToPrimitiveFixup(p, b)
            self.RadConservedToPrimitiveFixup(rp, p, b)
            self.ApplyFloors(rp, p, b)

        derived()
        rpu = copy.copy(rp)
        rpu.update_fluid = 1
        self.MomentFluidSource(rpu, p, b, beta * dt)
        self.ApplyFloors(rp, p, b)
        orc.FillGhostsPeriodic(b, b["cons"], abi.NCONS if p.mhd else 5)
        self.FillGhostsPeriodic(b)
        derived()
        b.arrays["cons"], b.arrays["rcons"] = fin, rin

    def rk2_fluid_step(self, rp, p, b: Block, fluid_buf, rad_buf, dt):
        fb, rb = b.arrays["cons"], b.arrays["rcons"]
        self.FluidStage(rp, p, b, fb, fluid_buf, rb, rad_buf, 1.0, dt)
        b.arrays["cons"], b.arrays["rcons"] = fluid_buf, rad_buf
        self.FluidStage(rp, p, b, fb, fb, rb, rb, 0.5, dt)
        b.arrays["cons"], b.arrays["rcons"] = fb, rb
