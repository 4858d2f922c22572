"""ctypes binding of libmsc_gpu.so (the C ABI declared in include/msc_gpu.h).

The library is built in-tree by :mod:`msceer_gb300.build`.  There is no CPU
fallback: if the shared object is missing or a call fails, this module raises.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libmsc_gpu.so"
_lock = threading.Lock()
_lib = None

MSC_OK = 0
ERRORS = {
    -1: "MSC_ERR_BAD_DIMS", -2: "MSC_ERR_NULL_POINTER", -3: "MSC_ERR_CUDA", -4: "MSC_ERR_OOM",
    -5: "MSC_ERR_NAN_INPUT", -6: "MSC_ERR_ITER_LIMIT", -7: "MSC_ERR_QUEUE_OVERFLOW", -8: "MSC_ERR_TOO_LARGE",
}

# every symbol include/msc_gpu.h declares: (restype, argtypes)
_I64P = ctypes.POINTER(ctypes.c_int64)
_VP = ctypes.c_void_p
SIGNATURES = {
    "msc_version": (ctypes.c_int, []),
    "msc_last_error_string": (ctypes.c_char_p, []),
    "msc_last_ldir_passes": (ctypes.c_int, []),
    "msc_num_cells_3d": (ctypes.c_int64, [_I64P]),
    "msc_num_cells_2d": (ctypes.c_int64, [_I64P]),
    "msc_lower_star_grad_3d": (ctypes.c_int, [_VP, _I64P, _VP, _VP]),
    "msc_lower_star_grad_2d": (ctypes.c_int, [_VP, _I64P, _VP, _VP]),
    "msc_lower_star_pairs_3d": (ctypes.c_int, [_VP, _I64P, _VP, _VP]),
    "msc_lower_star_pairs_2d": (ctypes.c_int, [_VP, _I64P, _VP, _VP]),
    "msc_ascending_manifold_dims_3d": (ctypes.c_int, [_VP, _I64P, _VP, ctypes.POINTER(ctypes.c_int)]),
    "msc_ascending_manifold_dims_2d": (ctypes.c_int, [_VP, _I64P, _VP, ctypes.POINTER(ctypes.c_int)]),
    "msc_ascending_manifold_dims_3d_static": (ctypes.c_int, [_VP, _I64P, _VP, ctypes.POINTER(ctypes.c_int)]),
    "msc_central_diff_grad_3d": (ctypes.c_int, [_VP, _I64P, _VP, ctypes.c_int, _VP]),
    "msc_central_diff_grad_2d": (ctypes.c_int, [_VP, _I64P, _VP, ctypes.c_int, _VP]),
    "msc_central_diff_grad_3d_f64": (ctypes.c_int, [_VP, _I64P, _VP, _VP]),
    "msc_central_diff_grad_2d_f64": (ctypes.c_int, [_VP, _I64P, _VP, _VP]),
    "msc_integrated_labels_3d": (ctypes.c_int, [_VP, _VP, _I64P, _VP, _VP, _VP, _VP]),
    "msc_integrated_labels_3d_stages": (ctypes.c_int, [_VP, _VP, _I64P, _VP, _VP, _VP, _VP, _VP]),
    "msc_lower_star_grad_batch_3d": (ctypes.c_int, [ctypes.c_int, _VP, _I64P, _VP, _VP]),
    "msc_kernel_launches": (ctypes.c_int64, []),
    "msc_labels_last_error_string": (ctypes.c_char_p, []),
    "msc_clean_regions_3d": (ctypes.c_int, [_VP, _VP, _I64P, ctypes.c_int, _VP, _VP]),
    "msc_conforming_grad_3d": (ctypes.c_int, [_VP, _VP, _VP, _I64P, _VP, _VP, _I64P, _VP]),
    "msc_labels_last_stats": (None, [_I64P]),
    "msc_labels_last_iterations": (None, [_I64P]),
    "msc_trim_scratch": (None, []),
    "msc_triage_last_error_string": (ctypes.c_char_p, []),
    "msc_triage_features_3d": (ctypes.c_int, [_VP, _VP, _I64P, _VP, _VP, _VP, _VP]),  # f grad dims p feat tgt st
    "msc_triage_forward_3d": (ctypes.c_int, [_VP, _I64P, _VP, _VP, _VP, _VP, _VP]),
    "msc_triage_backward_3d": (ctypes.c_int, [_VP, _VP, _VP, _VP, _VP, _I64P, _VP, ctypes.c_float, _VP, _VP, _VP]),
    "msc_triage_adam_step": (ctypes.c_int, [_VP, _VP, _VP, _VP, ctypes.c_int, ctypes.c_float, _VP]),
    "msc_triage_labels_3d": (ctypes.c_int, [_VP, _VP, _I64P, _VP, _VP, _VP, _VP, _I64P, _VP]),
    "msc_ondemand_labels_host": (ctypes.c_int, [_VP, _I64P, _VP, _VP, _VP, _VP]),
    "msc_steepest_lstar_host": (ctypes.c_int, [_VP, _I64P, _VP]),
    "msc_lower_star_grad_2d_host": (ctypes.c_int, [_VP, _I64P, _VP]),
    # grad f dims build node_cap cell value dim boundary arc_cap lower upper persistence counts stream
    "msc_ms_graph_3d": (ctypes.c_int, [_VP, _VP, _I64P, _VP, ctypes.c_int64, _VP, _VP, _VP, _VP, ctypes.c_int64, _VP,
                                       _VP, _VP, _I64P, _VP]),
    # f grad zeroed dims which params cells stats stream
    "msc_saddle_lines_3d": (ctypes.c_int, [_VP, _VP, _VP, _I64P, ctypes.c_int, _VP, _VP, _I64P, _VP]),
}


class IntegParams(ctypes.Structure):
    """msc_integ_params (include/msc_gpu.h)."""
    _fields_ = [("error_threshold", ctypes.c_float), ("gradient_threshold", ctypes.c_float),
                ("iteration_limit", ctypes.c_int), ("max_step", ctypes.c_float),
                ("presimp_threshold", ctypes.c_float), ("precision", ctypes.c_int)]


class MscError(RuntimeError):
    def __init__(self, code: int, fn: str, msg: str):
        super().__init__(f"{fn} failed with {ERRORS.get(code, code)}: {msg}")
        self.code = code


def lib_path() -> Path:
    return _LIB_PATH


def load() -> ctypes.CDLL:
    """Load libmsc_gpu.so (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not _LIB_PATH.exists():
                raise RuntimeError(f"{_LIB_PATH} is missing: run `python -m msceer_gb300.build` "
                                   "(there is no CPU fallback)")
            lib = ctypes.CDLL(str(_LIB_PATH))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
        return _lib


def dims_arg(dims) -> ctypes.Array:
    return (ctypes.c_int64 * len(dims))(*[int(d) for d in dims])


def check(rc: int, fn: str) -> None:
    if rc != MSC_OK:
        lib = load()
        labels = "labels" in fn or "clean" in fn
        err = lib.msc_labels_last_error_string if labels else lib.msc_last_error_string
        raise MscError(rc, fn, err().decode(errors="replace"))
