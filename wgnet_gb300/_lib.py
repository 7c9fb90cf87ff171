"""ctypes binding of `libwgnet_gb300.so` (the C ABI declared in include/wgnet_gb300.h).

There is no fallback: if the library is missing or cannot be loaded, every entry point raises.
Build it with `python -m wgnet_gb300.build` (or `__graft_entry__.build()`).
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_native" / "libwgnet_gb300.so"

WG_OK = 0
WG_ERR_ARG = 1
WG_ERR_CUDA = 2
WG_ERR_NONFINITE = 3
WG_ERR_ENERGY = 4
WG_ERR_UNSUPPORTED = 5
WG_ERR_CFL = 6
WG_ERR_OOM = 7


class WgConfig(ctypes.Structure):
    _fields_ = [
        ("shots", ctypes.c_int), ("nt", ctypes.c_int), ("dt", ctypes.c_float), ("peak_hz", ctypes.c_float),
        ("pml", ctypes.c_int), ("vmin", ctypes.c_float), ("vmax", ctypes.c_float), ("nx_vis", ctypes.c_int),
        ("nz_vis", ctypes.c_int), ("h", ctypes.c_float), ("nrec", ctypes.c_int),
    ]


_P = ctypes.c_void_p
_I = ctypes.c_int
_F = ctypes.c_float

# name -> (restype, argtypes); the exported symbols of include/wgnet_gb300.h.
SIGNATURES: dict[str, tuple] = {
    "wg_engine_create": (_I, [ctypes.POINTER(WgConfig), ctypes.POINTER(_P)]),
    "wg_engine_destroy": (None, [_P]),
    "wg_engine_dims": (_I, [_P] + [ctypes.POINTER(_I)] * 7),
    "wg_get_sources": (_I, [_P, _P, _I]),
    "wg_set_sources": (_I, [_P, _P, _I]),
    "wg_get_wavelet": (_I, [_P, _P, _I]),
    "wg_set_wavelet": (_I, [_P, _P, _I]),
    "wg_simulate": (_I, [_P, _P, _I, _P]),
    "wg_simulate_dev": (_I, [_P, _P, _I, _P, _P]),
    "wg_evaluate_adjoint": (_I, [_P, _P, _P, _I, _P, _P]),
    "wg_evaluate_adjoint_dev": (_I, [_P, _P, _P, _I, _P, _P, _P]),
    "wg_engine_status": (_I, [_P, _P]),
    "wg_selftest_wait_timeout": (_I, [_P, ctypes.c_longlong, _P]),
    "wg_set_checkpoint_interval": (_I, [_P, _I]),
    "wg_get_checkpoint_interval": (_I, [_P]),
    "wg_set_option": (_I, [_P, ctypes.c_char_p, _I]),
    "wg_get_option": (_I, [_P, ctypes.c_char_p, ctypes.POINTER(_I)]),
    "wg_set_launch_shape": (_I, [_P, _I, _I, _I, _I]),
    "wg_get_launch_shape": (_I, [_P, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "wg_shape_candidates": (_I, [_P, _I, _P, _I]),
    "wg_simulate_shot": (_I, [_P, _I, _I, _F, _F, _I, _I, _F, _F, _F, _F, _F, _P]),
    "wg_ricker_wavelet": (_I, [_I, _F, _F, _P]),
    "wg_cpml_profiles": (_I, [_I, _F, _F, _I, _F, _F, _P, _P, _P]),
    "wg_bandlimit_dev": (_I, [_P, _P, _I, _I, _I, _I, _P, _P]),
    "wg_lowpass_decimate_f16_dev": (_I, [_P, _P, _I, _I, _I, _I, _I, _I, _P, _P]),
    "wg_gen_plan_create": (_I, [_P, _P, _I, _P, _P, _I, _P, _I, _F, ctypes.c_size_t, ctypes.POINTER(_P)]),
    "wg_gen_plan_launch": (_I, [_P, _P]),
    "wg_gen_plan_info": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(ctypes.c_size_t), _P, _I, ctypes.POINTER(_I)]),
    "wg_gen_plan_destroy": (None, [_P]),
    "wg_lowpass_taps": (_I, [ctypes.c_double, ctypes.c_double, _P, _I]),
    "wg_gemm_bf16_dev": (_I, [_P, _P, _P, _I, _I, _I, _I, _P, _P]),
    "wg_lbfgs_direction_dev": (_I, [_P, _P, _P, _P, _P, _I, _I, ctypes.c_long, _P, _P]),
    "wg_dot_f64_dev": (_I, [_P, _P, _I, ctypes.c_long, _P, _P]),
    "wg_misfit_dev": (_I, [_P, _P, _I, ctypes.c_long, _P, _P]),
    "wg_pc_im2col": (_I, [_P, _I, _I, _I, _I, _I, _I, _P, _P]),
    "wg_pc_col2im": (_I, [_P, _I, _I, _I, _I, _I, _I, _P, _I, _P]),
    "wg_pc_transpose_bf16": (_I, [_P, ctypes.c_long, _I, _P, _P]),
    "wg_pc_cast_bf16": (_I, [_P, ctypes.c_long, _I, _I, _I, _P, _P]),
    "wg_pc_add": (_I, [_P, _P, ctypes.c_long, _P, _P, _P]),
    "wg_pc_relu_grad": (_I, [_P, _P, ctypes.c_long, _P, _P]),
    "wg_pc_features": (_I, [_P, _P, _P, _I, _I, _I, _P, _P, _P]),
    "wg_pc_mse": (_I, [_P, _I, _P, _F, ctypes.c_long, _P, _P, _P]),
    "wg_pc_adam": (_I, [_P, _I, _I, _I, _P, _P, _P, _F, _F, _F, _F, _I, _P, _P, _P]),
    "wg_render_fwd_dev": (_I, [_P, _I, _P, _P]),
    "wg_render_bwd_dev": (_I, [_P, _P, _I, _P, _P]),
    "wg_profile": (_I, [_P, _I]),
    "wg_profile_read": (_I, [_P, _P, _P, _I]),
    "wg_evaluate_adjoint_noalloc": (_I, [_P, _P, _P, _I, _P, _P, _P]),
    "wg_last_error": (ctypes.c_char_p, []),
    "wg_launch_count": (ctypes.c_longlong, [_I]),
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


def load() -> ctypes.CDLL:
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA extension with "
                                   "`python -m wgnet_gb300.build` (there is no CPU fallback)")
            lib = ctypes.CDLL(str(LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def last_error() -> str:
    msg = load().wg_last_error()
    return msg.decode() if msg else ""


def check(rc: int, what: str = "") -> None:
    """Map a C-ABI status to the reference's Python exceptions (ValueError for bad input)."""
    if rc == WG_OK:
        return
    msg = last_error() or f"status {rc}"
    if what:
        msg = f"{what}: {msg}"
    if rc in (WG_ERR_ARG, WG_ERR_NONFINITE, WG_ERR_CFL):
        raise ValueError(msg)
    if rc == WG_ERR_ENERGY:
        raise RuntimeError(msg)
    if rc == WG_ERR_OOM:
        raise MemoryError(msg)
    raise RuntimeError(msg)


def ptr(a) -> int | None:
    """Address of a numpy array or a torch tensor (None for None)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def launch_count(reset: bool = False) -> int:
    return int(load().wg_launch_count(1 if reset else 0))
