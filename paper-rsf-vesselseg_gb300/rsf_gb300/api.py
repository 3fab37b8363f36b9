"""Python face of the C ABI: parameters with the reference's flag names and
evolution entry points over torch CUDA tensors or NumPy host arrays.

The reference's executable takes --sigma --t --dt --meu --e --v --sigma2
(CUDA_RSF/main.cpp:88-102); `Params` keeps those meanings (and defaults) and
adds the knobs the reference hard-codes: eps (kernel.cu:258,275), separate
lambda1/lambda2, the x = 0 boundary rule and the arithmetic definition, and
one mode of this project's own: the expanded Gaussian data term.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import RsfAdjointSubvol, RsfParams, RsfSubvol, check


@dataclass
class Params:
    sigma: float = 5.0      # --sigma
    dt: float = 0.1         # --dt
    mu: float = 1.0         # --meu
    lambda1: float = 0.1    # --e (weight of e_out)
    lambda2: float = 0.1    # --e (weight of e_in)
    nu: float = 0.0001      # --v
    eps: float = 0.2        # hard-coded in the reference
    sigma2: float = 0.0     # --sigma2
    boundary: str = "reference"  # or "clamp"
    arith: str = "portable"      # or "reference"
    data_term: str = "reference"  # or "gaussian" (expanded RSF data term, no counterpart in the reference)

    def to_c(self) -> RsfParams:
        p = RsfParams()
        p.sigma, p.dt, p.mu = self.sigma, self.dt, self.mu
        p.lambda1, p.lambda2, p.nu = self.lambda1, self.lambda2, self.nu
        p.eps, p.sigma2 = self.eps, self.sigma2
        p.boundary = {"reference": 0, "clamp": 1}[self.boundary]
        p.arith = {"portable": 0, "reference": 1}[self.arith]
        p.data_term = {"reference": 0, "gaussian": 1}[self.data_term]
        return p

    @classmethod
    def from_flags(cls, sigma=5.0, t=None, dt=0.1, meu=1.0, e=0.1, v=0.0001, sigma2=0.0, **kw):
        """Builds Params from the reference's flag names (`t` is ignored here)."""
        return cls(sigma=sigma, dt=dt, mu=meu, lambda1=e, lambda2=e, nu=v, sigma2=sigma2, **kw)


def gaussian_taps(sigma: float) -> np.ndarray:
    lib = _lib.load()
    k = ctypes.c_int(0)
    check(lib.rsf_gaussian_taps(ctypes.c_float(sigma), None, 0, ctypes.byref(k)))
    buf = (ctypes.c_float * k.value)()
    check(lib.rsf_gaussian_taps(ctypes.c_float(sigma), buf, k.value, ctypes.byref(k)))
    return np.frombuffer(buf, dtype=np.float32).copy()


def _dtype_code(dt) -> int:
    s = str(dt)
    if s in ("uint8", "torch.uint8"):
        return _lib.RSF_U8
    if s in ("float32", "torch.float32"):
        return _lib.RSF_F32
    raise TypeError(f"image dtype must be uint8 or float32, got {s}")


def _stream_ptr(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


class Workspace:
    """Device scratch for batches of up to `max_voxels` voxels in total."""

    def __init__(self, max_voxels: int, max_subvols: int = 1):
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.rsf_workspace_create(int(max_voxels), int(max_subvols), ctypes.byref(h)))
        self.handle = h
        self.max_voxels = int(max_voxels)
        self.max_subvols = int(max_subvols)

    @property
    def nbytes(self) -> int:
        return int(self._lib.rsf_workspace_bytes(self.handle))

    def close(self):
        if self.handle:
            check(self._lib.rsf_workspace_destroy(self.handle))
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_launch_shape(self, xpass_width: int = 0, stencil_planes: int = 0, z_tma: int = -1):
        """Overrides the per-batch launch-shape heuristics for later calls:
        x-pass outputs per lane (5 or 9), stencil planes per block (32, 64 or 128)
        and the TMA z-pass (1) or the streaming one (0); 0 / -1 restore the
        automatic choice.  Every shape gives bit-identical results."""
        check(self._lib.rsf_workspace_set_launch_shape(self.handle, int(xpass_width), int(stencil_planes),
                                                       int(z_tma)))

    def set_kernel_timing(self, enable: bool):
        check(self._lib.rsf_set_kernel_timing(self.handle, int(bool(enable))))

    KERNELS = ("xpass", "ypass", "zpass", "stencil")

    def kernel_times(self, reset: bool = False):
        """{kernel: (total ms, launches)} accumulated while timing was enabled."""
        ms = (ctypes.c_double * 4)()
        n = (ctypes.c_int64 * 4)()
        check(self._lib.rsf_kernel_times(self.handle, ms, n, int(bool(reset))))
        return {k: (ms[i], n[i]) for i, k in enumerate(self.KERNELS)}

    def check(self, stream=None):
        check(self._lib.rsf_workspace_check(self.handle, ctypes.c_void_p(_stream_ptr(stream))))

    # ---- device tensors -------------------------------------------------
    def evolve(self, image, phi, params: Params, iters: int, stream=None):
        """Evolves torch CUDA tensor `phi` (float32, shape (L, H, W)) in place."""
        _require_cuda(image, phi)
        _require_volume(phi, image)
        L, H, W = phi.shape
        check(self._lib.rsf_evolve(self.handle, ctypes.byref(params.to_c()), ctypes.c_void_p(image.data_ptr()),
                                   _dtype_code(image.dtype), ctypes.c_void_p(phi.data_ptr()), W, H, L, int(iters),
                                   ctypes.c_void_p(_stream_ptr(stream))))
        return phi

    def signed_distance(self, seed, threshold: float = 13.0, out=None, stream=None):
        """phi0 from a seed volume (CUDA_RSF/main.cpp:174-183): the exact signed
        Euclidean distance of {seed > threshold}, positive inside.  `seed` is a
        uint8 or float32 CUDA tensor (L, H, W); returns `out` (float32)."""
        import torch
        _require_cuda(seed)
        if seed.dim() != 3:
            raise ValueError("seed must be 3-D (L, H, W)")
        seed = seed.contiguous()
        if out is None:
            out = torch.empty(seed.shape, dtype=torch.float32, device=seed.device)
        _require_cuda(out)
        _require_volume(out, seed)
        L, H, W = seed.shape
        check(self._lib.rsf_signed_distance(self.handle, ctypes.c_void_p(seed.data_ptr()), _dtype_code(seed.dtype),
                                            ctypes.c_float(threshold), ctypes.c_void_p(out.data_ptr()), W, H, L,
                                            ctypes.c_void_p(_stream_ptr(stream))))
        return out

    def step_adjoint(self, image, phi, phi_bar, params: Params, out=None, param_grads=None, stream=None):
        """dL/dphi of one step phi -> phi' given phi_bar = dL/dphi'.  When
        `param_grads` (CUDA float64, 4 elements) is given, dL/d(lambda1,
        lambda2, mu, nu) are added to it.  Returns `out` (new if None)."""
        import torch
        _require_cuda(image, phi, phi_bar)
        _require_volume(phi, image, phi_bar)
        L, H, W = phi.shape
        if out is None:
            out = torch.empty_like(phi)
        _require_cuda(out)
        _require_volume(out, phi)
        gp = None
        if param_grads is not None:
            _require_cuda(param_grads)
            if param_grads.dtype != torch.float64 or param_grads.numel() < 4:
                raise TypeError("param_grads must be a CUDA float64 tensor of 4 elements")
            gp = ctypes.c_void_p(param_grads.data_ptr())
        check(self._lib.rsf_step_adjoint(self.handle, ctypes.byref(params.to_c()), ctypes.c_void_p(image.data_ptr()),
                                         _dtype_code(image.dtype), ctypes.c_void_p(phi.data_ptr()),
                                         ctypes.c_void_p(phi_bar.data_ptr()), ctypes.c_void_p(out.data_ptr()), gp,
                                         W, H, L, ctypes.c_void_p(_stream_ptr(stream))))
        return out

    def step_adjoint_batched(self, items, params: Params, param_grads=None, stream=None):
        """`step_adjoint` for a list of (image, phi, phi_bar, out) CUDA tensor
        tuples in one launch sequence; `out` (may be None) receives dL/dphi of
        its volume.  Parameter gradients, summed over the batch, are added to
        `param_grads` when given.  Returns the list of outputs."""
        import torch
        if not items:
            raise ValueError("empty batch")
        codes = {_dtype_code(img.dtype) for img, _, _, _ in items}
        if len(codes) != 1:
            raise TypeError("all images of a batch must share one dtype")
        arr = (RsfAdjointSubvol * len(items))()
        outs = []
        for i, (img, phi, pbar, out) in enumerate(items):
            _require_cuda(img, phi, pbar)
            _require_volume(phi, img, pbar)
            if out is None:
                out = torch.empty_like(phi)
            _require_cuda(out)
            _require_volume(out, phi)
            L, H, W = phi.shape
            arr[i] = RsfAdjointSubvol(phi.data_ptr(), img.data_ptr(), pbar.data_ptr(), out.data_ptr(), W, H, L)
            outs.append(out)
        gp = None
        if param_grads is not None:
            _require_cuda(param_grads)
            if param_grads.dtype != torch.float64 or param_grads.numel() < 4:
                raise TypeError("param_grads must be a CUDA float64 tensor of 4 elements")
            gp = ctypes.c_void_p(param_grads.data_ptr())
        check(self._lib.rsf_step_adjoint_batched(self.handle, ctypes.byref(params.to_c()), codes.pop(), arr,
                                                 len(items), gp, ctypes.c_void_p(_stream_ptr(stream))))
        return outs

    def evolve_batched(self, pairs, params: Params, iters: int, stream=None):
        """Evolves a list of (image, phi) CUDA tensor pairs, each phi in place."""
        if not pairs:
            raise ValueError("empty batch")
        codes = {_dtype_code(img.dtype) for img, _ in pairs}
        if len(codes) != 1:
            raise TypeError("all images of a batch must share one dtype")
        arr = (RsfSubvol * len(pairs))()
        for i, (img, phi) in enumerate(pairs):
            _require_cuda(img, phi)
            _require_volume(phi, img)
            L, H, W = phi.shape
            arr[i] = RsfSubvol(phi.data_ptr(), img.data_ptr(), W, H, L)
        check(self._lib.rsf_evolve_batched(self.handle, ctypes.byref(params.to_c()), codes.pop(), arr, len(pairs),
                                           int(iters), ctypes.c_void_p(_stream_ptr(stream))))
        return [phi for _, phi in pairs]

    def step_debug(self, image, phi, params: Params, stream=None):
        """One iteration; returns (phi_out, fields[8]) as new CUDA tensors."""
        import torch
        _require_cuda(image, phi)
        _require_volume(phi, image)
        L, H, W = phi.shape
        out = torch.empty_like(phi)
        fields = torch.empty((8, L, H, W), dtype=torch.float32, device=phi.device)
        check(self._lib.rsf_step_debug(self.handle, ctypes.byref(params.to_c()), ctypes.c_void_p(image.data_ptr()),
                                       _dtype_code(image.dtype), ctypes.c_void_p(phi.data_ptr()),
                                       ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(fields.data_ptr()), W, H, L,
                                       ctypes.c_void_p(_stream_ptr(stream))))
        return out, fields

    # ---- host arrays ----------------------------------------------------
    def evolve_host(self, image: np.ndarray, phi: np.ndarray, params: Params, iters: int) -> np.ndarray:
        """Host-buffer call shape of the reference: copies in, evolves, copies
        back.  `phi` (float32, C order) is updated in place and returned."""
        if phi.dtype != np.float32 or not phi.flags.c_contiguous:
            raise TypeError("phi must be a C-contiguous float32 array")
        if image.shape != phi.shape or not image.flags.c_contiguous:
            raise TypeError("image must be C-contiguous with phi's shape")
        L, H, W = phi.shape
        check(self._lib.rsf_evolve_host(self.handle, ctypes.byref(params.to_c()), ctypes.c_void_p(image.ctypes.data),
                                        _dtype_code(image.dtype), ctypes.c_void_p(phi.ctypes.data), W, H, L,
                                        int(iters)))
        return phi

    def evolve_host_ptr(self, image_ptr: int, image_dtype, phi_ptr: int, shape, params: Params, iters: int):
        """Same as evolve_host for raw host pointers (e.g. pinned torch tensors)."""
        L, H, W = shape
        check(self._lib.rsf_evolve_host(self.handle, ctypes.byref(params.to_c()), ctypes.c_void_p(image_ptr),
                                        _dtype_code(image_dtype), ctypes.c_void_p(phi_ptr), W, H, L, int(iters)))


def copy_async(dst, src, stream=None):
    """dst <- src (torch tensors of equal byte size, each on the device or in
    pinned host memory) with the device's SMs (rsf_copy_async): host <->
    device transfers that keep their rate where the copy engine slows."""
    nb = dst.numel() * dst.element_size()
    if nb != src.numel() * src.element_size():
        raise ValueError("dst and src differ in size")
    if not (dst.is_contiguous() and src.is_contiguous()):
        raise TypeError("expected contiguous tensors")
    lib = _lib.load()
    check(lib.rsf_copy_async(ctypes.c_void_p(dst.data_ptr()), ctypes.c_void_p(src.data_ptr()), nb,
                             ctypes.c_void_p(_stream_ptr(stream))))
    return dst


def _require_cuda(*ts):
    for t in ts:
        if not getattr(t, "is_cuda", False):
            raise TypeError("expected CUDA tensors")
        if not t.is_contiguous():
            raise TypeError("expected contiguous tensors")


def _require_volume(phi, *same_shape):
    """phi: 3-D float32; every other tensor has phi's shape and device.  The C
    ABI takes raw pointers and phi's extents, so a smaller image would be read
    out of bounds: the shapes are checked here."""
    import torch

    if phi.dim() != 3 or phi.dtype != torch.float32:
        raise TypeError(f"phi must be a 3-D float32 tensor (L, H, W), got {tuple(phi.shape)} {phi.dtype}")
    for t in same_shape:
        if tuple(t.shape) != tuple(phi.shape):
            raise ValueError(f"shape {tuple(t.shape)} differs from phi's {tuple(phi.shape)}")
        if t.device != phi.device:
            raise ValueError("all tensors must be on phi's device")
