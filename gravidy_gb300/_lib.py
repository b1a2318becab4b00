"""ctypes binding of libgravidy_gb300.so (include/gravidy_gb300.h).

The library is built in-tree (gravidy_gb300/build.py).  There is no CPU
fallback: if the library cannot be loaded, or no CUDA device is present,
every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .build import LIB, build_library

H4_OK = 0
H4_FORCE_FP64 = 0
H4_FORCE_EXACT = 1
H4_FORCE_MIXED = 2
MODES = {"fp64": H4_FORCE_FP64, "exact": H4_FORCE_EXACT, "mixed": H4_FORCE_MIXED}

# Every symbol of include/gravidy_gb300.h with its ctypes signature.
_vp, _d, _f, _u, _i = C.c_void_p, C.c_double, C.c_float, C.c_uint, C.c_int
_pd, _pu = C.POINTER(C.c_double), C.POINTER(C.c_uint)
SIGNATURES = {
    "h4_last_error": (C.c_char_p, []),
    "h4_status_string": (C.c_char_p, [_i]),
    "h4_abi_version": (_i, []),
    "h4_build_flags": (_i, []),
    "h4_create": (_i, [C.POINTER(_vp), _u, _d, _f, _vp, _vp, _i]),
    "h4_destroy": (_i, [_vp]),
    "h4_set_stream": (_i, [_vp, _vp]),
    "h4_set_dt_limits": (_i, [_vp, _d, _d]),
    "h4_set_force_mode": (_i, [_vp, _i]),
    "h4_set_mixed_threshold": (_i, [_vp, _u]),
    "h4_init_acc_jrk": (_i, [_vp]),
    "h4_init_dt": (_i, [_vp, _pd, _f, _d]),
    "h4_find_particles_to_move": (_i, [_vp, _d, _pu]),
    "h4_save_old_acc_jrk": (_i, [_vp, _u]),
    "h4_predicted_pos_vel": (_i, [_vp, _d]),
    "h4_update_acc_jrk": (_i, [_vp, _u]),
    "h4_correction_pos_vel": (_i, [_vp, _d, _u]),
    "h4_next_integration_time": (_i, [_vp, _pd]),
    "h4_get_energy": (_i, [_vp, _pd, _pd, _pd]),
    "h4_step": (_i, [_vp, _pd, _pd, _pu]),
    "h4_advance": (_i, [_vp, _d, _d, _pd, _pd, _pd]),
    "h4_download": (_i, [_vp] + [_vp] * 9),
    "h4_upload": (_i, [_vp] + [_vp] * 6),
    "h4_download_predicted": (_i, [_vp, _vp, _vp]),
    "h4_restore": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _d]),
    "h4_forces_for": (_i, [_vp, _vp, _vp, _u, _vp, _vp]),
    "h4_last_timings": (_i, [_vp, C.POINTER(_f), C.POINTER(_f)]),
    "h4_kernel_launches": (_i, [_vp, C.POINTER(C.c_ulonglong)]),
    "h4_nact_histogram": (_i, [_vp, _vp]),
    "h4_phase_times": (_i, [_vp, _vp, _vp]),
    "h4_phase_name": (C.c_char_p, [_i]),
    "h4_probe_peaks": (_i, [_pd, _pd]),
    "h4_selftest_bounded_wait": (_i, [_d, C.POINTER(_i)]),
    "h4_forces_noalloc": (_i, [_u, _d, _vp, _vp, _u, _vp, _vp, _vp]),
    "h4_center_of_density": (_i, [_vp, _vp]),
    "h4_mass_radii": (_i, [_vp, _vp, _f, _pd, _pd, _vp]),
    "h4_diag_last_error": (C.c_char_p, []),
    "h4_ens_last_error": (C.c_char_p, []),
    "h4_ens_create": (_i, [C.POINTER(_vp), _u, _vp, _vp, _vp, _vp, _vp, _i]),
    "h4_ens_destroy": (_i, [_vp]),
    "h4_ens_set_stream": (_i, [_vp, _vp]),
    "h4_ens_set_tuning": (_i, [_vp, _vp, _vp, _vp]),
    "h4_ens_set_dt_limits": (_i, [_vp, _d, _d]),
    "h4_ens_init": (_i, [_vp]),
    "h4_ens_advance": (_i, [_vp, _vp, _pd]),
    "h4_ens_energy": (_i, [_vp, _vp, _vp]),
    "h4_ens_download": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "h4_ens_system_stats": (_i, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "h4_ens_tune_force": (_i, [_vp, _u, _u, _u, _u, C.POINTER(_f)]),
    "h4_ens_bucket_stats": (_i, [_vp, _vp, _vp]),
    "h4_ens_timings": (_i, [_vp, C.POINTER(_f), C.POINTER(C.c_ulonglong)]),
    "h4_ens_phase_times": (_i, [_vp, _vp]),
    "h4_forces_noalloc_error": (C.c_char_p, []),
}


class H4Error(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


_lib = None


def library_path() -> str:
    """The library to load: GRAVIDY_GB300_LIB if set (e.g. the bounds-checked
    build), else the in-tree build."""
    return os.environ.get("GRAVIDY_GB300_LIB") or LIB


def load(build_if_missing: bool = True):
    """Load the native library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if path != LIB or not build_if_missing:
            raise OSError(f"{path} not built; run python -m gravidy_gb300.build")
        build_library()
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != H4_OK:
        L = load()
        raise H4Error(status, L.h4_last_error().decode() or L.h4_status_string(status).decode())


def check_ens(status: int) -> None:
    if status != H4_OK:
        L = load()
        raise H4Error(status, L.h4_ens_last_error().decode() or L.h4_status_string(status).decode())


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


def probe_peaks():
    """(fp64 flop/s, fp32 flop/s) measured on the current GPU."""
    a, b = C.c_double(), C.c_double()
    check(load().h4_probe_peaks(C.byref(a), C.byref(b)))
    return a.value, b.value
