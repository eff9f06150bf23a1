"""ctypes mirror of include/phx_fluid.h and include/phx_radiation.h, and
loader of the sm_103a libraries.

The structures here are byte-for-byte the C structs of the header; the same
definitions describe host arrays (numpy) and device arrays (torch CUDA
tensors), since the ABI only sees pointers.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIBDIR = PKG / "_lib"

# ---- constants (phx_fluid.h)
PRHO, PVEL, PENG, PB, PPRS, PGM1, PTMP, PMU = 0, 1, 4, 5, 8, 9, 10, 11
NPRIM, NRECON = 12, 10
CRHO, CMOM, CENG, CB = 0, 1, 4, 5
NCONS = 8
RECON = {"constant": 0, "linear": 1, "weno5": 2, "weno5z": 2, "mp5": 3}
RIEMANN = {"llf": 0, "hll": 1}
GEOM_MINKOWSKI, GEOM_FMKS = 0, 1
FLOOR = {"ConstantRhoSie": 0, "ExpX1RhoSie": 1, "ExpX1RhoU": 2, "X1RhoSie": 3, "RRhoSie": 4}
G_ALPHA, G_BETA, G_GCOV, G_GAMCON, G_DETGAM, GEOM_NLOC = 0, 1, 4, 14, 20, 21
GD_DALPHA, GD_DG, GEOM_NDER = 0, 3, 33
C2P_HIST = 128
MLP_IN, MLP_HID, MLP_OUT = 6, 64, 2
C2P_CHUNK = 1 << 21  # zones per con2prim chunk inside the library (launch accounting only)
MLP_MAX_EPOCHS = 1024
MLP_NPARAM = MLP_IN * MLP_HID + MLP_HID + 2 * (MLP_HID * MLP_HID + MLP_HID) + MLP_HID * 2 + 2

# ---- constants (phx_radiation.h)
RE, RF, RNCONS = 0, 1, 4
RJ, RH, RXI, RPHI, RFAIL, RKAPPAJ, RKAPPAH, RJBB, RNPRIM = 0, 1, 4, 5, 6, 7, 8, 9, 10
RAD_METHOD = {"moment_m1": 0, "moment_eddington": 1}
RAD_ONED_FIXUP = {"none": 0, "ignore_dJ": 1, "ignore_all": 2}
RAD_SRC_SOLVER = {"oned": 0, "fourd": 1}  # radiation/src_solver (radiation.cpp:403-415)
RAD_FLOOR = {"ConstantJ": 0, "ExpX1J": 1}  # fixup/rad_floor_type (fixup.cpp:188-200)

MATH = {"exp": 0, "log": 1, "sin": 2, "cos": 3, "pow": 4, "rcp": 5, "rsqrt": 6}
PHX_OK, PHX_ERR_INVALID_ARG, PHX_ERR_UNBRACKETED, PHX_ERR_NAN_INPUT, PHX_ERR_TIMEOUT = 0, 1, 2, 3, 4
PHX_ERR_CUDA, PHX_ERR_NO_DEVICE, PHX_ERR_CAPACITY, PHX_ERR_UNSUPPORTED = 5, 6, 7, 8
STATUS = {0: "ok", 1: "invalid argument", 2: "con2prim root not bracketed", 3: "NaN input",
          4: "device wait timed out", 5: "CUDA error", 6: "no CUDA device",
          7: "request exceeds a fixed capacity", 8: "unsupported"}


class TorusParams(C.Structure):
    _fields_ = [("rin", C.c_double), ("rmax", C.c_double), ("kappa", C.c_double), ("u_jitter", C.c_double),
                ("target_beta", C.c_double), ("magnetized", C.c_int), ("seed", C.c_ulonglong)]


class Range(C.Structure):
    _fields_ = [("s", C.c_int), ("e", C.c_int)]


class Params(C.Structure):
    _fields_ = [
        ("gm1", C.c_double), ("Cv", C.c_double), ("rho_min_eos", C.c_double), ("sie_min_eos", C.c_double),
        ("c2p_tol", C.c_double), ("c2p_max_iter", C.c_int), ("c2p_floor_scale_fac", C.c_double),
        ("c2p_fail_on_floors", C.c_int), ("c2p_fail_on_ceilings", C.c_int),
        ("recon", C.c_int), ("riemann", C.c_int), ("cfl", C.c_double), ("mhd", C.c_int),
        ("enable_floors", C.c_int), ("enable_ceilings", C.c_int), ("enable_mhd_floors", C.c_int),
        ("enable_c2p_fixup", C.c_int), ("c2p_failure_strategy_floors", C.c_int), ("floor_type", C.c_int),
        ("rho0_floor", C.c_double), ("sie0_floor", C.c_double), ("rho_exp_floor", C.c_double),
        ("sie_exp_floor", C.c_double), ("gam0_ceiling", C.c_double), ("sie0_ceiling", C.c_double),
        ("bsqorho0_ceiling", C.c_double), ("bsqou0_ceiling", C.c_double),
        ("enable_flux_fixup", C.c_int), ("enable_ox1_fmks_inflow_check", C.c_int),
    ]


class Geometry(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("a", C.c_double), ("hslope", C.c_double), ("poly_xt", C.c_double),
        ("poly_alpha", C.c_double), ("x0", C.c_double), ("smooth", C.c_double), ("hexp_br", C.c_double),
        ("hexp_nsq", C.c_double), ("hexp_csq", C.c_double), ("derefine_poles", C.c_int),
        ("cent", C.c_void_p), ("face1", C.c_void_p), ("face2", C.c_void_p), ("deriv", C.c_void_p),
    ]


class BlockS(C.Structure):
    _fields_ = [
        ("nx1", C.c_int), ("nx2", C.c_int), ("nx3", C.c_int), ("ng", C.c_int), ("ndim", C.c_int),
        ("var_stride", C.c_longlong),
        ("x1min", C.c_double), ("x2min", C.c_double), ("x3min", C.c_double),
        ("dx1", C.c_double), ("dx2", C.c_double), ("dx3", C.c_double),
        ("prim", C.c_void_p), ("cons", C.c_void_p), ("flux", C.c_void_p), ("face_sig", C.c_void_p),
        ("cell_sig", C.c_void_p), ("fail", C.c_void_p), ("src", C.c_void_p), ("emf", C.c_void_p),
        ("dudt", C.c_void_p), ("geom", C.POINTER(Geometry)),
    ]


class C2PStats(C.Structure):
    _fields_ = [("zones", C.c_ulonglong), ("iterations", C.c_ulonglong), ("residual_evals", C.c_ulonglong),
                ("failures", C.c_ulonglong), ("unbracketed", C.c_ulonglong),
                ("learned_accepted", C.c_ulonglong), ("hist", C.c_ulonglong * C2P_HIST)]


class Mesh(C.Structure):
    _fields_ = [("n", C.c_int * 3), ("nseg", C.c_int * 3), ("seg_start", C.c_void_p * 3), ("bc_lo", C.c_int * 3),
                ("bc_hi", C.c_int * 3), ("bc_vars", C.c_int)]


BC_PERIODIC, BC_OUTFLOW, BC_REFLECT, BC_POLAR = 0, 1, 2, 3
BC_VARS_CONSERVED, BC_VARS_PRIMITIVE = 0, 1


class RadParams(C.Structure):
    _fields_ = [("method", C.c_int), ("recon", C.c_int), ("cfl", C.c_double), ("closure_frail", C.c_int),
                ("recon_fixup_bounds", C.c_int), ("src_rootfind_tol", C.c_double),
                ("src_rootfind_maxiter", C.c_int), ("oned_fixup_strategy", C.c_int), ("kappa_a", C.c_double),
                ("kappa_s", C.c_double), ("jbb_coeff", C.c_double), ("enable_rad_floors", C.c_int),
                ("J0_floor", C.c_double), ("enable_rad_ceilings", C.c_int), ("xi0_ceiling", C.c_double),
                ("tau0_ceiling", C.c_double), ("update_fluid", C.c_int), ("rad_c2p_failure_floors", C.c_int),
                ("src_solver", C.c_int), ("src_rootfind_eps", C.c_double), ("src_use_oned_backup", C.c_int),
                ("rad_floor_type", C.c_int), ("J_exp_floor", C.c_double)]


class RadBlockS(C.Structure):
    _fields_ = [("var_stride", C.c_longlong), ("cons", C.c_void_p), ("prim", C.c_void_p), ("flux", C.c_void_p),
                ("dudt", C.c_void_p)]


class MlpTrainOpts(C.Structure):
    _fields_ = [("batch", C.c_int), ("epochs", C.c_int), ("lr", C.c_float), ("lr_min", C.c_float),
                ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float), ("weight_decay", C.c_float)]


def default_train_opts(**over) -> MlpTrainOpts:
    # same defaults as phx_mlp_train_opts_default
    o = MlpTrainOpts(batch=4096, epochs=10, lr=3e-3, lr_min=0.0, beta1=0.9, beta2=0.999, eps=1e-8,
                     weight_decay=1e-4)
    for k, v in over.items():
        setattr(o, k, v)
    return o


class PhxError(RuntimeError):
    """Raised when an entry point returns a non-OK phx_status."""

    def __init__(self, status: int, detail: str):
        super().__init__(f"phx status {status} ({STATUS.get(status, '?')}): {detail}")
        self.status = status


_LIBS: dict[str, C.CDLL] = {}

_P = C.c_void_p
_SIGS = {
    "phx_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "phx_ctx_destroy": (C.c_int, [_P]),
    "phx_ctx_check": (C.c_int, [_P]),
    "phx_ctx_c2p_stats": (C.c_int, [_P, C.POINTER(C2PStats), C.c_int]),
    "phx_status_string": (C.c_char_p, [C.c_int]),
    "phx_last_error": (C.c_char_p, []),
    "phx_abi_version": (C.c_int, []),
    "phx_build_exact": (C.c_int, []),
    "phx_params_default": (None, [C.POINTER(Params)]),
    "phx_geometry_default": (None, [C.POINTER(Geometry), C.c_int]),
    "phx_prim_to_con": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), Range, Range, Range, _P]),
    "phx_con_to_prim": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), Range, Range, Range, _P]),
    "phx_con_to_prim_learned": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), Range, Range, Range, _P]),
    "phx_mlp_features_zones": (C.c_int, [_P, C.POINTER(Params), C.c_longlong, _P, _P, _P, _P, _P]),
    "phx_mlp_forward": (C.c_int, [_P, C.c_longlong, _P, _P, _P]),
    "phx_mlp_bracket_zones": (C.c_int, [_P, C.POINTER(Params), C.c_longlong, _P, _P, _P, _P, _P]),
    "phx_mlp_loss_grad": (C.c_int, [_P, C.c_longlong, _P, _P, _P, _P, _P]),
    "phx_mlp_train_opts_default": (None, [C.POINTER(MlpTrainOpts)]),
    "phx_mlp_train": (C.c_int, [_P, C.c_longlong, _P, _P, C.POINTER(MlpTrainOpts), _P, _P]),
    "phx_prim_to_con_zones": (C.c_int, [_P, C.POINTER(Params), C.c_longlong, _P, _P, _P, _P, _P]),
    "phx_con_to_prim_zones": (C.c_int, [_P, C.POINTER(Params), C.c_longlong, _P, _P, _P, _P, _P, _P, C.c_int, _P]),
    "phx_geometry_fmks_points": (C.c_int, [_P, C.POINTER(Geometry), C.c_longlong, _P, _P, _P, _P]),
    "phx_calculate_fluxes": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), _P]),
    "phx_flux_ct": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), _P]),
    "phx_calculate_fluid_source_terms": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), C.c_int, _P]),
    "phx_update_stage": (C.c_int, [_P, C.POINTER(BlockS), _P, _P, C.c_double, C.c_double, _P]),
    "phx_fill_ghosts_periodic": (C.c_int, [_P, C.POINTER(BlockS), _P, C.c_int, _P]),
    "phx_estimate_timestep": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), C.c_int, _P, _P]),
    "phx_estimate_timestep_static": (C.c_int, [C.POINTER(Params), C.POINTER(BlockS), C.c_int, _P, _P]),
    "phx_c2p_fixup": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), _P]),
    "phx_apply_floors": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), Range, Range, Range, _P]),
    "phx_geometry_fill_fmks": (C.c_int, [_P, C.POINTER(Geometry), C.POINTER(BlockS), _P]),
    "phx_stage": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), _P, _P, C.c_double, C.c_double,
                            C.c_int, _P]),
    "phx_stage_batched": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), C.c_int, _P, _P, C.c_double,
                                    C.c_double, C.c_int, _P]),
    "phx_stage_mesh": (C.c_int, [_P, C.POINTER(Params), C.POINTER(Mesh), C.POINTER(BlockS), C.c_int, _P, _P,
                                 C.c_double, C.c_double, C.c_int, C.c_int, _P]),
    "phx_mesh_exchange": (C.c_int, [_P, C.POINTER(Params), C.POINTER(Mesh), C.POINTER(BlockS), C.c_int, _P]),
    "phx_fix_fluxes": (C.c_int, [_P, C.POINTER(Params), C.POINTER(Mesh), C.POINTER(BlockS), C.c_int, _P]),
    "phx_fix_fluxes_block": (C.c_int, [_P, C.POINTER(Params), C.POINTER(BlockS), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), _P]),
    "phx_rad_params_default": (None, [C.POINTER(RadParams)]),
    "phx_rad_prim_to_con": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), Range, Range, Range, _P]),
    "phx_rad_con_to_prim": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), Range, Range, Range, _P]),
    "phx_rad_calculate_opacities": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), _P]),
    "phx_rad_calculate_fluxes": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), _P]),
    "phx_rad_update": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(BlockS), C.POINTER(RadBlockS), _P, _P, C.c_double, C.c_double, _P]),
    "phx_rad_fluid_source": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), C.c_double, _P]),
    "phx_rad_fill_ghosts_periodic": (C.c_int, [_P, C.POINTER(BlockS), C.POINTER(RadBlockS), _P]),
    "phx_rad_fix_fluxes": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(Mesh),
                                     C.POINTER(BlockS), C.POINTER(RadBlockS), C.c_int, _P]),
    "phx_rad_mesh_exchange": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(Mesh),
                                        C.POINTER(BlockS), C.POINTER(RadBlockS), C.c_int, _P]),
    "phx_rad_estimate_timestep": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), _P, _P]),
    "phx_rad_stage": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), _P, _P, C.c_double, C.c_double, _P]),
    "phx_rad_fluid_stage": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), _P, _P, _P, _P, C.c_double, C.c_double, _P]),
    "phx_rad_c2p_fixup": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), _P]),
    "phx_rad_apply_floors": (C.c_int, [_P, C.POINTER(RadParams), C.POINTER(Params), C.POINTER(BlockS), C.POINTER(RadBlockS), Range, Range, Range, _P]),
    "phx_batch_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "phx_mlp_set_weights": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "phx_mlp_get_weights": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "phx_mlp_set_input_box": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "phx_mlp_get_input_box": (C.c_int, [_P, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "phx_math_eval": (C.c_int, [C.c_int, C.c_longlong, _P, _P, _P, _P]),
    "phx_torus_params_default": (None, [C.POINTER(TorusParams)]),
    "phx_torus_init": (C.c_int, [_P, C.POINTER(Params), C.POINTER(TorusParams), C.POINTER(BlockS), C.c_int,
                                 C.POINTER(C.c_double), _P]),
    "phx_probe_fp64_peak": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "phx_probe_bounded_wait": (C.c_int, [_P, C.c_longlong, _P]),
}


def exported_symbols() -> list[str]:
    """Every entry point include/phx_fluid.h and include/phx_radiation.h
    declare (kept in sync by a test)."""
    return sorted(_SIGS)


def lib_path(exact: bool = False) -> Path:
    return LIBDIR / ("libphx_fluid_exact.so" if exact else "libphx_fluid.so")


def load(exact: bool = False) -> C.CDLL:
    """Load the CUDA library.  Fails loudly if it was not built: there is no
    CPU fallback for the hot path."""
    key = "exact" if exact else "fast"
    if key in _LIBS:
        return _LIBS[key]
    path = lib_path(exact)
    if not path.exists():
        raise RuntimeError(f"{path} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                           "(the fluid hot path has no CPU fallback)")
    lib = C.CDLL(str(path))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIBS[key] = lib
    return lib


def check(lib: C.CDLL, status: int) -> None:
    if status != 0:
        raise PhxError(status, lib.phx_last_error().decode())


def default_params(lib: C.CDLL | None = None, **over) -> Params:
    p = Params()
    # same defaults as phx_params_default (fluid.cpp:53-136, fixup.cpp:48-280)
    p.gm1, p.Cv = 4.0 / 3.0 - 1.0, 1.0
    p.c2p_tol, p.c2p_max_iter, p.c2p_floor_scale_fac = 1.0e-8, 20, 1.0
    p.recon, p.riemann, p.cfl, p.mhd = RECON["linear"], RIEMANN["hll"], 0.8, 1
    p.floor_type, p.rho_exp_floor, p.sie_exp_floor = 0, -2.0, -1.0
    p.gam0_ceiling, p.sie0_ceiling, p.bsqorho0_ceiling, p.bsqou0_ceiling = 1000.0, 100.0, 50.0, 2500.0
    for k, v in over.items():
        if k == "recon" and isinstance(v, str):
            v = RECON[v]
        if k == "riemann" and isinstance(v, str):
            v = RIEMANN[v]
        if k == "floor_type" and isinstance(v, str):
            v = FLOOR[v]
        if k == "Gamma":
            k, v = "gm1", v - 1.0
        setattr(p, k, v)
    return p


def default_geometry(kind: int, **over) -> Geometry:
    g = Geometry()
    g.kind = kind
    g.a, g.hslope, g.poly_xt, g.poly_alpha, g.x0, g.smooth = 0.0, 0.3, 0.82, 14.0, 0.0, 0.5
    g.hexp_br, g.hexp_nsq, g.hexp_csq, g.derefine_poles = 1.0e30, 4.0, 4.0, 1
    for k, v in over.items():
        setattr(g, k, v)
    return g


def default_torus_params(**over) -> TorusParams:
    """phx_torus_params_default (torus.cpp:174-181, 525-530 defaults), then
    overrides."""
    t = TorusParams()
    t.rin, t.rmax, t.kappa, t.u_jitter, t.target_beta, t.magnetized, t.seed = 6.0, 12.0, 1e-2, 1e-2, 100.0, 1, 0
    for k, v in over.items():
        setattr(t, k, v)
    return t


def default_rad_params(**over) -> RadParams:
    """phx_rad_params_default (radiation.cpp:340-450, fixup.cpp:75-76,
    188-215 defaults), then overrides; method / oned_fixup_strategy / recon
    accept the input-deck strings."""
    r = RadParams()
    r.method, r.recon, r.cfl = RAD_METHOD["moment_m1"], RECON["linear"], 0.8
    r.closure_frail, r.recon_fixup_bounds = 0, 1
    r.src_rootfind_tol, r.src_rootfind_maxiter, r.oned_fixup_strategy = 1.0e-12, 100, 0
    r.kappa_a, r.kappa_s, r.jbb_coeff = 0.0, 0.0, 0.0
    r.enable_rad_floors, r.J0_floor = 0, 0.0
    r.enable_rad_ceilings, r.xi0_ceiling, r.tau0_ceiling = 0, 0.99, 1.0e3
    r.update_fluid, r.rad_c2p_failure_floors = 0, 0
    r.src_solver, r.src_rootfind_eps, r.src_use_oned_backup = RAD_SRC_SOLVER["oned"], 1.0e-8, 0
    r.rad_floor_type, r.J_exp_floor = RAD_FLOOR["ConstantJ"], -2.0
    for k, v in over.items():
        if k == "method" and isinstance(v, str):
            v = RAD_METHOD[v]
        if k == "recon" and isinstance(v, str):
            v = RECON[v]
        if k == "oned_fixup_strategy" and isinstance(v, str):
            v = RAD_ONED_FIXUP[v]
        if k == "src_solver" and isinstance(v, str):
            v = RAD_SRC_SOLVER[v]
        if k == "rad_floor_type" and isinstance(v, str):
            v = RAD_FLOOR[v]
        if not hasattr(r, k):
            raise KeyError(k)
        setattr(r, k, v)
    return r
