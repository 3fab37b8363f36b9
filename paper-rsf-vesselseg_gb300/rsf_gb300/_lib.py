"""ctypes binding of librsf_gb300.so (the C ABI in include/rsf.h).

Loading fails loudly: there is no CPU fallback for the evolution.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

from . import build as _build

RSF_OK = 0
STATUS_NAMES = {
    0: "RSF_OK", 1: "RSF_ERR_INVALID_ARGUMENT", 2: "RSF_ERR_SHAPE", 3: "RSF_ERR_DTYPE",
    4: "RSF_ERR_UNSUPPORTED", 5: "RSF_ERR_NO_MEMORY", 6: "RSF_ERR_WORKSPACE_TOO_SMALL", 7: "RSF_ERR_CUDA",
    8: "RSF_ERR_NONFINITE", 9: "RSF_ERR_IO", 10: "RSF_ERR_NO_DEVICE",
}
RSF_U8, RSF_F32 = 0, 1
RSF_BOUNDARY_REFERENCE, RSF_BOUNDARY_CLAMP = 0, 1
RSF_ARITH_PORTABLE, RSF_ARITH_REFERENCE = 0, 1


class RsfParams(ctypes.Structure):
    _fields_ = [("sigma", ctypes.c_float), ("dt", ctypes.c_float), ("mu", ctypes.c_float),
                ("lambda1", ctypes.c_float), ("lambda2", ctypes.c_float), ("nu", ctypes.c_float),
                ("eps", ctypes.c_float), ("sigma2", ctypes.c_float), ("boundary", ctypes.c_int32),
                ("arith", ctypes.c_int32), ("data_term", ctypes.c_int32), ("reserved", ctypes.c_int32 * 5)]


class RsfSubvol(ctypes.Structure):
    _fields_ = [("phi", ctypes.c_void_p), ("image", ctypes.c_void_p), ("W", ctypes.c_int64),
                ("H", ctypes.c_int64), ("L", ctypes.c_int64)]


class RsfAdjointSubvol(ctypes.Structure):
    _fields_ = [("phi", ctypes.c_void_p), ("image", ctypes.c_void_p), ("phi_bar_in", ctypes.c_void_p),
                ("phi_bar_out", ctypes.c_void_p), ("W", ctypes.c_int64), ("H", ctypes.c_int64), ("L", ctypes.c_int64)]


class RsfTile(ctypes.Structure):
    _fields_ = [("phi", ctypes.c_void_p), ("x0", ctypes.c_int64), ("y0", ctypes.c_int64), ("z0", ctypes.c_int64),
                ("W", ctypes.c_int64), ("H", ctypes.c_int64), ("L", ctypes.c_int64)]


class RsfError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


# Every symbol include/rsf.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I32 = ctypes.c_int32
SIGNATURES = {
    "rsf_abi_version": (ctypes.c_int, []),
    "rsf_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "rsf_last_error": (ctypes.c_char_p, []),
    "rsf_params_default": (ctypes.c_int, [ctypes.POINTER(RsfParams)]),
    "rsf_gaussian_taps": (ctypes.c_int, [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int)]),
    "rsf_workspace_create": (ctypes.c_int, [_I64, _I32, ctypes.POINTER(ctypes.c_void_p)]),
    "rsf_workspace_destroy": (ctypes.c_int, [_P]),
    "rsf_workspace_bytes": (ctypes.c_size_t, [_P]),
    "rsf_workspace_bytes_for": (ctypes.c_size_t, [_I64, _I32]),
    "rsf_workspace_set_launch_shape": (ctypes.c_int, [_P, _I32, _I32, _I32]),
    "rsf_evolve": (ctypes.c_int, [_P, ctypes.POINTER(RsfParams), _P, ctypes.c_int, _P, _I64, _I64, _I64, _I32, _P]),
    "rsf_evolve_batched": (ctypes.c_int, [_P, ctypes.POINTER(RsfParams), ctypes.c_int, ctypes.POINTER(RsfSubvol),
                                          _I32, _I32, _P]),
    "rsf_evolve_host": (ctypes.c_int, [_P, ctypes.POINTER(RsfParams), _P, ctypes.c_int, _P, _I64, _I64, _I64, _I32]),
    "rsf_step_debug": (ctypes.c_int, [_P, ctypes.POINTER(RsfParams), _P, ctypes.c_int, _P, _P, _P, _I64, _I64, _I64,
                                      _P]),
    "rsf_workspace_check": (ctypes.c_int, [_P, _P]),
    "rsf_signed_distance": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_float, _P, _I64, _I64, _I64, _P]),
    "rsf_reassemble": (ctypes.c_int, [_P, _P, _I32, _I32, _I32, _P, _P, _P, _I32, _P, _I64, _I64, _I64, _P]),
    "rsf_copy_async": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P]),
    "rsf_step_adjoint": (ctypes.c_int, [_P, ctypes.POINTER(RsfParams), _P, ctypes.c_int, _P, _P, _P, _P, _I64, _I64,
                                        _I64, _P]),
    "rsf_step_adjoint_batched": (ctypes.c_int, [_P, ctypes.POINTER(RsfParams), ctypes.c_int,
                                                ctypes.POINTER(RsfAdjointSubvol), _I32, _P, _P]),
    "rsf_set_kernel_timing": (ctypes.c_int, [_P, ctypes.c_int]),
    "rsf_kernel_times": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64),
                                        ctypes.c_int]),
}

_lib = None


def lib_path() -> Path:
    return _build.LIB_PATH


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Returns the loaded library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build() "
                               "(python -c 'import __graft_entry__ as g; g.build()')")
        _build.build()
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != RSF_OK:
        lib = load()
        raise RsfError(status, lib.rsf_last_error().decode(errors="replace"))
