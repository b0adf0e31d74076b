"""ctypes binding of libhermes_gb300.so (include/hermes_gb300.h).

The library is the only compute path: there is no CPU fallback.  Loading
fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

from .config import Config

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libhermes_gb300.so")

HERMES_OK = 0
ABI_VERSION = 8          # HERMES_ABI_VERSION of include/hermes_gb300.h
STATUS = {0: "HERMES_OK", 1: "HERMES_ERR_CONFIG", 2: "HERMES_ERR_SHAPE", 3: "HERMES_ERR_DTYPE",
          4: "HERMES_ERR_NONFINITE", 5: "HERMES_ERR_TIMEOUT", 6: "HERMES_ERR_CUDA", 7: "HERMES_ERR_ALLOC",
          8: "HERMES_ERR_ARG"}

# every function include/hermes_gb300.h declares
EXPORTS = ("hermes_abi_version", "hermes_config_size", "hermes_sizes", "hermes_create", "hermes_ensemble_create", "hermes_box_offsets",
           "hermes_destroy", "hermes_last_error", "hermes_stream", "hermes_get_min_dt", "hermes_limiter",
           "hermes_rhs", "hermes_euler_stage", "hermes_step", "hermes_advance", "hermes_advance_host",
           "hermes_enqueue_steps", "hermes_profile_enable", "hermes_profile_read",
           "hermes_box_times", "hermes_set_time", "hermes_set_noise_step", "hermes_set_noise_stage", "hermes_check", "hermes_rhs_noalloc",
           "hermes_rhs_vjp", "hermes_stage_vjp", "hermes_limiter_vjp", "hermes_set_launch", "hermes_get_launch",
           "hermes_checkpoint_write", "hermes_checkpoint_read", "hermes_derived",
           "hermes_init_state", "hermes_conserved")


class HermesLaunch(C.Structure):
    """hermes_launch of include/hermes_gb300.h."""
    _fields_ = [("face_tpb", C.c_int32), ("dt_tpb", C.c_int32), ("steps_per_graph", C.c_int32),
                ("noise_inline", C.c_int32), ("face_traces", C.c_int32), ("split_update", C.c_int32),
                ("tile_stage", C.c_int32), ("pdl", C.c_int32),
                ("faces_merged", C.c_int32), ("update_tpb", C.c_int32), ("cell_concurrent", C.c_int32)]


class HermesOutputUnits(C.Structure):
    """hermes_output_units of include/hermes_gb300.h."""
    _fields_ = [("n0", C.c_double), ("v0", C.c_double), ("t0", C.c_double), ("te0", C.c_double),
                ("eV_per_K", C.c_double)]


class HermesError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class NonFiniteError(HermesError, FloatingPointError):
    pass


class HermesConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("nbasis", C.c_int32), ("iquad", C.c_int32), ("iorder", C.c_int32),
        ("ivis", C.c_int32), ("ieos", C.c_int32), ("ihllc", C.c_int32),
        ("bc", C.c_int32 * 6),
        ("precision", C.c_int32), ("llns", C.c_int32),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("aindex", C.c_double), ("rh_floor", C.c_double), ("T_floor", C.c_double), ("rh_mult", C.c_double),
        ("coll", C.c_double), ("colvis", C.c_double), ("cflm", C.c_double),
        ("P_1", C.c_double), ("P_base", C.c_double),
        ("eta_sd", C.c_double), ("zeta_sd", C.c_double),
        ("seed", C.c_uint64),
        ("body_force", C.c_double),
        ("inflow_u", C.c_double), ("inflow_rho", C.c_double), ("inflow_p", C.c_double),
    ]


def to_c(cfg: Config) -> HermesConfig:
    c = HermesConfig()
    c.nx, c.ny, c.nz = cfg.nx, cfg.ny, cfg.nz
    c.nbasis, c.iquad, c.iorder = cfg.nbasis, cfg.iquad, cfg.iorder
    c.ivis, c.ieos, c.ihllc = cfg.ivis, cfg.ieos, int(cfg.ihllc)
    for i, b in enumerate(cfg.bc):
        c.bc[i] = b
    c.precision = 64 if cfg.precision == "fp64" else 32
    c.llns = int(bool(cfg.llns))
    c.lx, c.ly, c.lz = cfg.lx, cfg.ly, cfg.lz
    c.aindex, c.rh_floor, c.T_floor, c.rh_mult = cfg.aindex, cfg.rh_floor, cfg.T_floor, cfg.rh_mult
    c.coll, c.colvis, c.cflm = cfg.coll, cfg.colvis, cfg.cflm
    c.P_1, c.P_base = cfg.P_1, cfg.P_base
    c.eta_sd, c.zeta_sd = cfg.eta_sd, cfg.zeta_sd
    c.seed = cfg.seed & ((1 << 64) - 1)
    c.body_force = cfg.body_force
    c.inflow_u, c.inflow_rho, c.inflow_p = cfg.inflow_u, cfg.inflow_rho, cfg.inflow_pressure
    return c


_lib = None


def lib() -> C.CDLL:
    """Load libhermes_gb300.so; raise if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built: run `python -m hermeshd_gb300.build` "
                           "(or __graft_entry__.build()); there is no CPU fallback")
    L = C.CDLL(LIB_PATH)
    vp, dp, i32, cfgp = C.c_void_p, C.POINTER(C.c_double), C.c_int, C.POINTER(HermesConfig)
    ctxpp = C.POINTER(C.c_void_p)
    sig = {
        "hermes_abi_version": (i32, []),
        "hermes_config_size": (i32, []),
        "hermes_sizes": (i32, [cfgp, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
        "hermes_create": (i32, [cfgp, vp, ctxpp]),
        "hermes_ensemble_create": (i32, [cfgp, i32, C.POINTER(C.c_int32), dp, C.POINTER(C.c_uint64), vp, ctxpp]),
        "hermes_box_offsets": (i32, [vp, C.POINTER(C.c_int64)]),
        "hermes_destroy": (i32, [vp]),
        "hermes_last_error": (C.c_char_p, [vp]),
        "hermes_stream": (vp, [vp]),
        "hermes_get_min_dt": (i32, [vp, vp, dp]),
        "hermes_limiter": (i32, [vp, vp]),
        "hermes_rhs": (i32, [vp, vp, vp, i32]),
        "hermes_euler_stage": (i32, [vp, vp, vp, C.c_double]),
        "hermes_step": (i32, [vp, vp, vp, vp, dp, dp]),
        "hermes_advance": (i32, [vp, vp, vp, vp, i32, dp, dp]),
        "hermes_advance_host": (i32, [vp, vp, i32, dp, dp]),
        "hermes_enqueue_steps": (i32, [vp, vp, vp, i32]),
        "hermes_profile_enable": (i32, [vp, i32]),
        "hermes_profile_read": (i32, [vp, dp, C.POINTER(C.c_int64)]),
        "hermes_box_times": (i32, [vp, dp, dp]),
        "hermes_set_time": (i32, [vp, C.c_double]),
        "hermes_set_noise_step": (i32, [vp, C.c_uint64]),
        "hermes_set_noise_stage": (i32, [vp, C.c_int32]),
        "hermes_check": (i32, [vp]),
        "hermes_rhs_noalloc": (i32, [cfgp, vp, vp, i32, vp, C.c_char_p, C.c_size_t]),
        "hermes_rhs_vjp": (i32, [vp, vp, vp, vp]),
        "hermes_limiter_vjp": (i32, [vp, vp, vp, vp]),
        "hermes_stage_vjp": (i32, [vp, vp, vp, vp, vp, C.c_double, dp]),
        "hermes_set_launch": (i32, [vp, C.POINTER(HermesLaunch)]),
        "hermes_get_launch": (i32, [vp, C.POINTER(HermesLaunch)]),
        "hermes_checkpoint_write": (i32, [C.c_char_p, vp, i32, i32, i32, i32, C.c_double, C.c_double, i32,
                                          C.POINTER(C.c_int32), C.c_char_p, C.c_size_t]),
        "hermes_init_state": (i32, [vp, vp, i32, C.c_uint64]),
        "hermes_conserved": (i32, [vp, vp, dp]),
        "hermes_derived": (i32, [vp, vp, vp, i32, C.c_uint32, C.POINTER(HermesOutputUnits)]),
        "hermes_checkpoint_read": (i32, [C.c_char_p, vp, i32, i32, i32, i32, dp, dp, C.POINTER(C.c_int32),
                                         C.POINTER(C.c_int32), C.c_char_p, C.c_size_t]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc: int, ctx=None) -> None:
    if rc == HERMES_OK:
        return
    msg = lib().hermes_last_error(ctx).decode() if ctx else ""
    if rc == 4:
        raise NonFiniteError(rc, msg)
    raise HermesError(rc, msg)
