"""ctypes binding of libgvs.so (the C ABI in include/gvs.h).

The library is loaded from this package directory only (in-tree build).  If
it is missing, importing the engine raises: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgvs.so")
# The bounds-checked build (same ABI); a process that sets GVS_CHECKED=1 before the
# first load uses it.
CHECKED_LIB_PATH = os.path.join(HERE, "libgvs_checked.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "gvs.h")

OK, ERR_INVALID_ARG, ERR_OOM, ERR_LAUNCH, ERR_DEVICE, ERR_TIMEOUT, ERR_INJECTED, ERR_NO_DEVICE, ERR_STATE = range(9)
STATUS_NAMES = ["OK", "INVALID_ARG", "OOM", "LAUNCH", "DEVICE", "TIMEOUT", "INJECTED", "NO_DEVICE", "STATE"]
PREC_FP64_EXACT, PREC_FP64, PREC_FP32, PREC_MIXED = 0, 1, 2, 3
ALGO_NONE, ALGO_DIRECT, ALGO_BH = 0, 1, 2


class GvsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"gvs status {name}: {msg}")
        self.status = status


class Diag(C.Structure):
    _fields_ = [("kinetic_energy", C.c_double), ("potential_energy", C.c_double),
                ("thermal_energy", C.c_double), ("total_energy", C.c_double),
                ("momentum", C.c_double * 3), ("angular_momentum", C.c_double * 3),
                ("center_of_mass", C.c_double * 3), ("center_of_mass_velocity", C.c_double * 3),
                ("virial_ratio", C.c_double)]


class SphParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("gamma", "eta", "cfl_factor", "force_factor", "h_max", "beta_visc",
                                          "alpha_min", "alpha_max", "alpha_cond", "sigma_visc")] + \
               [("precision", C.c_int)]


class Profile(C.Structure):
    _fields_ = [("force_ms", C.c_double), ("force_launches", C.c_longlong), ("launches", C.c_longlong),
                ("force_flops", C.c_double), ("force_bytes", C.c_double), ("tile_visits", C.c_double),
                ("near_tile_visits", C.c_double), ("vjp_ms", C.c_double), ("vjp_launches", C.c_longlong),
                ("sph_f64_redo", C.c_longlong), ("bh_groups", C.c_longlong),
                ("bh_group_fallbacks", C.c_longlong), ("bh_group_iterations", C.c_longlong),
                ("bh_group_interactions", C.c_longlong), ("bh_walk_terms", C.c_longlong)]


_P = C.c_void_p  # every array argument is passed as a raw address
_d, _sz, _i, _u64, _ll = C.c_double, C.c_size_t, C.c_int, C.c_uint64, C.c_longlong
_ST = C.c_int

SIGNATURES = {
    "gvs_version": (C.c_char_p, []),
    "gvs_create": (_ST, [C.POINTER(C.c_void_p), _i]),
    "gvs_destroy": (_ST, [_P]),
    "gvs_last_error": (_ST, [_P, C.c_char_p, _sz]),
    "gvs_set_fault": (_ST, [_P, C.c_char_p]),
    "gvs_sync": (_ST, [_P]),
    "gvs_device_errors": (_ST, [_P, C.POINTER(C.c_uint)]),
    "gvs_set_state": (_ST, [_P, _sz] + [_P] * 11),
    "gvs_get_state": (_ST, [_P] + [_P] * 9),
    "gvs_set_accelerations": (_ST, [_P, _P, _P, _P]),
    "gvs_get_gas": (_ST, [_P] + [_P] * 7),
    "gvs_count": (_sz, [_P]),
    "gvs_set_gas": (_ST, [_P] + [_P] * 7),
    "gvs_gravity_direct": (_ST, [_P, _sz, _P, _P, _P, _P, _d, _i, _P, _P, _P]),
    "gvs_gravity_bh": (_ST, [_P, _sz, _P, _P, _P, _P, _d, _d, _i, _P, _P, _P]),
    "gvs_tree_export": (_ST, [_P, _sz, C.POINTER(_sz)] + [_P] * 8),
    "gvs_compute_forces": (_ST, [_P, _i, _i, _d, _d]),
    "gvs_ensemble_setup": (_ST, [_P, _i, _P, _d]),
    "gvs_ensemble_forces": (_ST, [_P]),
    "gvs_ensemble_kdk_steps": (_ST, [_P, _d, _ll, _i]),
    "gvs_adjoint_forward": (_ST, [_P, _i, _d, _d, _ll, _ll]),
    "gvs_adjoint_backward": (_ST, [_P] + [_P] * 13),
    "gvs_adjoint_checkpoints": (_ST, [_P, _ll, _P, _P]),
    "gvs_ic_plummer_device": (_ST, [_P, _sz, _u64, _d, _d]),
    "gvs_ic_collision_device": (_ST, [_P, _sz, _u64, _d]),
    "gvs_adjoint_checkpoint_read": (_ST, [_P, _ll] + [_P] * 6),
    "gvs_adjoint_prepare": (_ST, [_P, _i, _d, _d, _ll, _ll]),
    "gvs_adjoint_checkpoint_write": (_ST, [_P, _ll] + [_P] * 6),
    "gvs_sph_params_default": (_ST, [C.POINTER(SphParams)]),
    "gvs_sph_compute": (_ST, [_P, C.POINTER(SphParams), _P, _P, _P, _P]),
    "gvs_sph_timestep": (_ST, [_P, C.POINTER(SphParams), C.POINTER(_d)]),
    "gvs_sph_step": (_ST, [_P, C.POINTER(SphParams), _i, _i, _d, _d, _d, C.POINTER(_d)]),
    "gvs_sph_neighbors": (_ST, [_P, _sz, C.POINTER(_sz), _P, _P, _P]),
    "gvs_kdk_steps": (_ST, [_P, _i, _i, _d, _d, _d, _ll]),
    "gvs_kdk_step_host": (_ST, [_P, _sz] + [_P] * 10 + [_i, _i, _d, _d, _d]),
    "gvs_diagnostics": (_ST, [_P, _d, _i, C.POINTER(Diag)]),
    "gvs_diagnostics_noalloc": (_ST, [_i, _P, _sz] + [_P] * 9 + [_d, _i, C.POINTER(Diag)]),
    "gvs_direct_subset": (_ST, [_P, _i, _d, _P, _sz, _P, _P, _P]),
    "gvs_ic_plummer": (_ST, [_sz, _u64, _d, _d] + [_P] * 7),
    "gvs_ic_two_body": (_ST, [_d, _d, _d] + [_P] * 7),
    "gvs_ic_evrard": (_ST, [_sz, _u64, _d, _d, _d] + [_P] * 6),
    "gvs_ic_cold_collapse": (_ST, [_sz, _u64, _d, _d, _i] + [_P] * 9),
    "gvs_ic_collision": (_ST, [_sz, _u64, _d] + [_P] * 7),
    "gvs_ic_gas_sphere_1r": (_ST, [_sz, _d, _d, _d, _d] + [_P] * 6),
    "gvs_ic_ensemble_sizes": (_ST, [_sz, _u64, _d, _d, _P]),
    "gvs_autotune_direct": (_ST, [_P, _i, _d, C.POINTER(_i), C.POINTER(_i), C.POINTER(_d)]),
    "gvs_set_direct_shape": (_ST, [_P, _i, _i, _i, _i]),
    "gvs_set_bh_walk": (_ST, [_P, _i, _i]),
    "gvs_autotune_report": (_ST, [_P, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "gvs_profile_enable": (_ST, [_P, _i]),
    "gvs_profile_read": (_ST, [_P, C.POINTER(Profile)]),
    "gvs_event_record": (_ST, [_P, _i]),
    "gvs_event_elapsed": (_ST, [_P, _i, _i, C.POINTER(C.c_float)]),
    "gvs_l2_flush": (_ST, [_P]),
    "gvs_stream": (_ST, [_P, C.POINTER(C.c_void_p)]),
    "gvs_check_bounded_wait": (_ST, [_P, C.c_uint]),
    "gvs_measure_fp32_peak": (_ST, [_P, C.POINTER(C.c_double)]),
    "gvs_fp32_peak_variants": (_ST, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]),
}

_lib = None


def header_symbols() -> list[str]:
    """Every function declared in include/gvs.h."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gvs_[a-z0-9_]+)\s*\(", src)))


def load(path: str | None = None):
    """Loads libgvs.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or (CHECKED_LIB_PATH if os.environ.get("GVS_CHECKED") == "1" else LIB_PATH)
    if not os.path.exists(p):
        raise ImportError(f"{p} not found: build it with `python -m gravis_gb300.build` "
                          "(the engine has no CPU fallback)")
    L = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error(ctx=None) -> str:
    buf = C.create_string_buffer(512)
    load().gvs_last_error(ctx, buf, 512)
    return buf.value.decode(errors="replace")


def check(status: int, ctx=None):
    if status != OK:
        raise GvsError(status, last_error(ctx))
