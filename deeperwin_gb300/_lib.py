"""ctypes binding of libdwgb.so (the C ABI declared in include/dwgb.h).

The library is built in-tree by ``deeperwin_gb300.build``. Loading fails loudly when it is
missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "csrc" / "libdwgb.so"

DW_PRECISION = {"fp32": 0, "plain": 0, "mixed": 1, "bf16": 2, "fp64": 3, "fp32_det64": 4, "mixed_det64": 5}


class DwArch(ctypes.Structure):
    _fields_ = [("n_el", ctypes.c_int32), ("n_up", ctypes.c_int32), ("n_ions", ctypes.c_int32),
                ("n_dets", ctypes.c_int32), ("z_min", ctypes.c_int32), ("z_max", ctypes.c_int32),
                ("width_one", ctypes.c_int32), ("width_two", ctypes.c_int32), ("width_ion", ctypes.c_int32),
                ("jastrow0", ctypes.c_int32), ("jastrow1", ctypes.c_int32)]


class DwMcmcScalars(ctypes.Structure):
    _fields_ = [("acc_rate", ctypes.c_double), ("last_acc", ctypes.c_double), ("stepsize", ctypes.c_float),
                ("step_nr", ctypes.c_int32), ("ticket", ctypes.c_uint32), ("error", ctypes.c_int32)]


class DwMcmcConfig(ctypes.Structure):
    _fields_ = [("n_steps", ctypes.c_int32), ("max_age", ctypes.c_int32),
                ("stepsize_update_interval", ctypes.c_int32), ("target_acceptance_rate", ctypes.c_float),
                ("min_stepsize", ctypes.c_float), ("max_stepsize", ctypes.c_float), ("seed", ctypes.c_uint64),
                ("reevaluate", ctypes.c_int32), ("proposal", ctypes.c_int32), ("r_min", ctypes.c_float),
                ("r_max", ctypes.c_float), ("langevin_scale", ctypes.c_float), ("p_spin_swap", ctypes.c_float),
                ("p_spin_flip", ctypes.c_float)]


DW_PROPOSAL = {"normal": 0, "cauchy": 1, "langevin": 2, "local": 3, "normal_one_el": 4, "local_one_el": 5}


SCALARS_BYTES = ctypes.sizeof(DwMcmcScalars)

_P = ctypes.c_void_p
_SIGS = {
    "dw_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "dw_version": (ctypes.c_char_p, []),
    "dw_param_count": (ctypes.c_int64, [ctypes.POINTER(DwArch)]),
    "dw_param_layout": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64), ctypes.c_int]),
    "dw_prepared_bytes": (ctypes.c_size_t, [ctypes.POINTER(DwArch), ctypes.c_int]),
    "dw_prepare_params": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, ctypes.c_size_t, _P]),
    "dw_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(DwArch), ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "dw_log_psi_sqr": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P, _P, _P,
                                      _P, ctypes.c_size_t, _P]),
    "dw_local_energy": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P, _P,
                                       _P, _P, _P, ctypes.c_size_t, _P]),
    "dw_potential_energy": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_int, _P, _P]),
    "dw_mcmc_steps": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P, _P, _P,
                                     _P, ctypes.POINTER(DwMcmcConfig), _P, ctypes.c_size_t, _P]),
    "dw_log_psi_sqr_packed": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P,
                                             ctypes.c_int, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "dw_local_energy_packed": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P,
                                              ctypes.c_int, _P, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "dw_mcmc_steps_packed": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P,
                                            ctypes.c_int, _P, _P, _P, _P, _P, _P, ctypes.POINTER(DwMcmcConfig), _P,
                                            ctypes.c_size_t, _P]),
    "dw_energy_stats": (ctypes.c_int, [_P, ctypes.c_int, _P, _P]),
    "dw_forces_workspace_bytes": (ctypes.c_size_t, [ctypes.POINTER(DwArch), ctypes.c_int, ctypes.c_int]),
    "dw_forces": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P, _P,
                                 ctypes.c_float, ctypes.c_float, ctypes.c_int, _P, _P, _P, ctypes.c_size_t, _P]),
    "dw_clip_energies": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, _P, _P,
                                        _P]),
    "dw_log_psi_sqr_backward": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P,
                                               _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "dw_last_launch_count": (ctypes.c_int64, []),
    "dw_log_psi_sqr_noalloc": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P, _P,
                                              _P, _P, _P]),
    "dw_noalloc_scratch_bytes": (ctypes.c_size_t, []),
    "dw_debug_gemm_bf16": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, _P]),
    "dw_debug_tc_error_flag": (ctypes.c_int, []),
    "dw_debug_set_gemm_bk": (ctypes.c_int, [ctypes.c_int]),
    "dw_debug_set_guard_form": (ctypes.c_int, [ctypes.c_int]),
    "dw_debug_set_det_tangents_kernel": (ctypes.c_int, [ctypes.c_int]),
    "dw_guard_tier_stats": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int64),
                                           ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64), ctypes.c_int]),
    "dw_debug_slogdet_small": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                              _P, _P, _P, _P]),
    "dw_debug_local_energy_scales": (ctypes.c_int, [ctypes.POINTER(DwArch), ctypes.c_int, _P, _P, _P, ctypes.c_int, _P,
                                                    _P, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "dw_guard_stats": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_int64), ctypes.c_int]),
    "dw_timer_enable": (ctypes.c_int, [ctypes.c_int]),
    "dw_timer_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64),
                                     ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
}

_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m deeperwin_gb300.build` "
                               "(there is no CPU fallback)")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


# Launch count standing in for the library's own when one host-level call issued several library
# calls (run_mcmc_steps with the steps split across ranks); any later checked call clears it.
launch_override = None


def check(status: int, what: str = "") -> None:
    global launch_override
    launch_override = None
    if status != 0:
        msg = lib().dw_status_string(status).decode()
        raise RuntimeError(f"{what}: dwgb status {status} ({msg})")


def make_arch(a) -> DwArch:
    return DwArch(a.n_el, a.n_up, a.n_ions, a.n_dets, a.z_min, a.z_max, a.width_one, a.width_two, a.width_ion,
                  a.jastrow[0], a.jastrow[1])
