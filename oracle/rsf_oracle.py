"""ctypes loader and NumPy wrappers of the CPU oracle (rsf_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arm of bench.py, as the checker.  Arrays are NumPy
(L, H, W) C order, x fastest, like the reference's volumes.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "rsf_oracle.c"
LIB = HERE / "librsf_oracle.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    flags = ["-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")  # hardware fmaf; results are identical either way
    cmd = ["gcc", *flags, str(SRC), "-o", str(LIB), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    return LIB


class OracleParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in
                ("sigma", "dt", "mu", "lambda1", "lambda2", "nu", "eps", "sigma2")] + \
               [("boundary", ctypes.c_int32), ("mag_form", ctypes.c_int32), ("arith", ctypes.c_int32),
                ("data_term", ctypes.c_int32)]


_lib = None
_FP = ctypes.POINTER(ctypes.c_float)
_DP = ctypes.POINTER(ctypes.c_double)
_I64 = ctypes.c_int64


def lib():
    global _lib
    if _lib is None:
        build()
        l = ctypes.CDLL(str(LIB))
        l.oracle_taps.argtypes = [ctypes.c_float, _FP, ctypes.c_int]
        l.oracle_taps.restype = ctypes.c_int
        l.oracle_step_f32.argtypes = [_FP, _FP, _FP, _I64, _I64, _I64, ctypes.POINTER(OracleParams), _FP]
        l.oracle_step_f32.restype = ctypes.c_int
        l.oracle_evolve_f32.argtypes = [_FP, _FP, _I64, _I64, _I64, ctypes.POINTER(OracleParams), ctypes.c_int,
                                        ctypes.c_int]
        l.oracle_evolve_f32.restype = ctypes.c_int
        l.oracle_evolve_f64.argtypes = [_DP, _FP, _I64, _I64, _I64, ctypes.POINTER(OracleParams), ctypes.c_int,
                                        ctypes.c_int]
        l.oracle_evolve_f64.restype = ctypes.c_int
        l.oracle_gradient.argtypes = [_FP, _FP, _FP, _FP, _I64, _I64, _I64, ctypes.c_int]
        l.oracle_gradient.restype = None
        l.oracle_blur_padded.argtypes = [_FP, _FP, _I64, _I64, _I64, _FP, ctypes.c_int]
        l.oracle_blur_padded.restype = ctypes.c_int
        l.oracle_heaviside.argtypes = [_FP, _FP, _I64, ctypes.c_float, ctypes.c_int]
        l.oracle_dirac.argtypes = [_FP, _FP, _I64, ctypes.c_float, ctypes.c_int]
        l.oracle_normalise.argtypes = [_FP, _FP, _FP, _FP, _FP, _FP, _FP, _I64, ctypes.c_int, ctypes.c_int]
        l.oracle_atan.argtypes = [ctypes.c_float]
        l.oracle_atan.restype = ctypes.c_float
        l.oracle_max_threads.restype = ctypes.c_int
        _lib = l
    return _lib


def params(sigma=3.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=None, nu=65.025, eps=0.2, sigma2=0.0,
           boundary=0, mag_form=0, arith=0, data_term=0) -> OracleParams:
    return OracleParams(sigma, dt, mu, lambda1, lambda1 if lambda2 is None else lambda2, nu, eps, sigma2,
                        boundary, mag_form, arith, data_term)


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(_FP)


def taps(sigma: float) -> np.ndarray:
    buf = np.zeros(512, dtype=np.float32)
    k = lib().oracle_taps(ctypes.c_float(sigma), buf.ctypes.data_as(_FP), 512)
    if k < 0:
        raise ValueError(f"invalid sigma {sigma}")
    return buf[:k].copy()


def step(phi, image, p: OracleParams, debug: bool = False):
    """One iteration.  Returns phi_out, or (phi_out, fields[8]) with debug."""
    phi, pp = _f32(phi)
    img, ip = _f32(image)
    L, H, W = phi.shape
    out = np.empty_like(phi)
    dbg = np.empty((8, L, H, W), dtype=np.float32) if debug else None
    rc = lib().oracle_step_f32(pp, ip, out.ctypes.data_as(_FP), W, H, L, ctypes.byref(p),
                               dbg.ctypes.data_as(_FP) if debug else None)
    if rc != 0:
        raise RuntimeError(f"oracle_step_f32 failed ({rc})")
    return (out, dbg) if debug else out


def evolve(phi, image, p: OracleParams, iters: int, threads: int = 0) -> np.ndarray:
    phi = np.array(phi, dtype=np.float32, copy=True, order="C")
    img, ip = _f32(image)
    L, H, W = phi.shape
    rc = lib().oracle_evolve_f32(phi.ctypes.data_as(_FP), ip, W, H, L, ctypes.byref(p), int(iters), int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_evolve_f32 failed ({rc})")
    return phi


def evolve_f64(phi, image, p: OracleParams, iters: int, threads: int = 0) -> np.ndarray:
    phi = np.array(phi, dtype=np.float64, copy=True, order="C")
    img, ip = _f32(image)
    L, H, W = phi.shape
    rc = lib().oracle_evolve_f64(phi.ctypes.data_as(_DP), ip, W, H, L, ctypes.byref(p), int(iters), int(threads))
    if rc != 0:
        raise RuntimeError(f"oracle_evolve_f64 failed ({rc})")
    return phi


def gradient(f, boundary=0):
    f, fp = _f32(f)
    L, H, W = f.shape
    g = np.empty((3, L, H, W), dtype=np.float32)
    lib().oracle_gradient(fp, g[0].ctypes.data_as(_FP), g[1].ctypes.data_as(_FP), g[2].ctypes.data_as(_FP), W, H, L,
                          boundary)
    return g


def blur_padded(f, sigma):
    f, fp = _f32(f)
    L, H, W = f.shape
    g = taps(sigma)
    out = np.empty_like(f)
    rc = lib().oracle_blur_padded(fp, out.ctypes.data_as(_FP), W, H, L, g.ctypes.data_as(_FP), len(g))
    if rc != 0:
        raise RuntimeError("oracle_blur_padded failed")
    return out


def heaviside(phi, eps, arith=0):
    phi, pp = _f32(phi)
    out = np.empty_like(phi)
    lib().oracle_heaviside(pp, out.ctypes.data_as(_FP), phi.size, ctypes.c_float(eps), arith)
    return out


def dirac(phi, eps, arith=0):
    phi, pp = _f32(phi)
    out = np.empty_like(phi)
    lib().oracle_dirac(pp, out.ctypes.data_as(_FP), phi.size, ctypes.c_float(eps), arith)
    return out


def atan(x):
    x = np.asarray(x, dtype=np.float32)
    f = lib().oracle_atan
    return np.array([f(ctypes.c_float(v)) for v in x.ravel()], dtype=np.float32).reshape(x.shape)


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def update_field(phi, dh, eo, ei, kap, lap, p: OracleParams):
    """Final_phi (kernel.cu:365-387) applied element-wise."""
    l = lib()
    if not getattr(l.oracle_update_field, "argtypes", None):
        l.oracle_update_field.argtypes = [_FP] * 7 + [_I64, ctypes.POINTER(OracleParams)]
        l.oracle_update_field.restype = None
    arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (phi, dh, eo, ei, kap, lap)]
    out = np.empty_like(arrs[0])
    l.oracle_update_field(*[a.ctypes.data_as(_FP) for a in arrs], out.ctypes.data_as(_FP), out.size, ctypes.byref(p))
    return out


def normalise(gx, gy, gz, form=0, arith=0):
    """(|g|, nx, ny, nz) as kernel.cu:914-933 and 173-189 compute them."""
    g = [np.ascontiguousarray(a, dtype=np.float32) for a in (gx, gy, gz)]
    out = [np.empty_like(g[0]) for _ in range(4)]
    lib().oracle_normalise(*[a.ctypes.data_as(_FP) for a in g], out[1].ctypes.data_as(_FP), out[2].ctypes.data_as(_FP),
                           out[3].ctypes.data_as(_FP), out[0].ctypes.data_as(_FP), g[0].size, form, arith)
    return out


def signed_distance(seed, threshold: float = 13.0) -> np.ndarray:
    """phi0 of CUDA_RSF/main.cpp:174-183 as this project defines it: exact
    signed Euclidean distance of {seed > threshold}, positive inside.  Brute
    force per line, small volumes only.  Parity of this definition with the
    reference's tiralib sdf() is unpinned (tiralib is not in the reference)."""
    s = np.ascontiguousarray(seed, dtype=np.float32)
    if s.ndim != 3:
        raise ValueError("seed must be 3-D (L, H, W)")
    L, H, W = s.shape
    out = np.empty_like(s)
    l = lib()
    if not getattr(l.oracle_signed_distance, "argtypes", None):
        l.oracle_signed_distance.argtypes = [_FP, ctypes.c_float, _FP, _I64, _I64, _I64]
    rc = l.oracle_signed_distance(s.ctypes.data_as(_FP), threshold, out.ctypes.data_as(_FP), W, H, L)
    if rc:
        raise RuntimeError(f"oracle_signed_distance failed ({rc})")
    return out


def data_terms(I, fo, fi, s: int):
    """(e_out, e_in) of kernel.cu:25-55 for given fits and box radius s."""
    a = [np.ascontiguousarray(x, dtype=np.float32) for x in (I, fo, fi)]
    L, H, W = a[0].shape
    eo, ei = np.empty_like(a[0]), np.empty_like(a[0])
    l = lib()
    if not getattr(l.oracle_data_terms, "argtypes", None):
        l.oracle_data_terms.argtypes = [_FP] * 5 + [_I64, _I64, _I64, ctypes.c_int]
    l.oracle_data_terms(*[x.ctypes.data_as(_FP) for x in a], eo.ctypes.data_as(_FP), ei.ctypes.data_as(_FP),
                        W, H, L, int(s))
    return eo, ei
