"""Runs the reference's own kernels (CUDA_RSF/kernel.cu compiled unchanged
into oracle/_ref/kernel_sm103a.cubin) in the order of its iteration loop,
CUDA_RSF/main.cpp:233-300, with the launch shapes of its host wrappers.

TEST INFRASTRUCTURE ONLY: it produces the reference's outputs that the
oracle and the GPU path are checked against.  Device buffers are torch CUDA
tensors; kernels are launched through the CUDA driver API (libcuda) with
ctypes.  Every buffer that gradient_dx_cuda reads carries one extra leading
element holding the buffer's element 0: the reference reads element -1 at
voxel 0 (kernel.cu:64-73), which here stays inside the allocation and gives
the value the oracle defines for that read.
"""
from __future__ import annotations

import ctypes
import json
from pathlib import Path

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "kernel_sm103a.cubin"
NAMES = HERE / "_ref" / "kernels.json"


def available() -> bool:
    return CUBIN.exists() and NAMES.exists()


class RefKernels:
    def __init__(self):
        import torch

        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoadData.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        self.cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + [
            ctypes.c_uint, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        self.image = CUBIN.read_bytes()
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoadData(ctypes.byref(self.mod), self.image), "cuModuleLoadData")
        self.fn = {}
        for plain, mangled in json.loads(NAMES.read_text()).items():
            f = ctypes.c_void_p()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, mangled.encode()), plain)
            self.fn[plain] = f

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")

    def launch(self, name, grid, block, *args):
        import torch

        holders = []
        for a in args:
            if isinstance(a, ctypes._SimpleCData):
                holders.append(a)
            elif hasattr(a, "data_ptr"):
                holders.append(ctypes.c_void_p(a.data_ptr()))
            else:
                raise TypeError(f"argument {a!r}")
        ptrs = (ctypes.c_void_p * len(holders))(*[ctypes.cast(ctypes.byref(h), ctypes.c_void_p) for h in holders])
        stream = torch.cuda.current_stream().cuda_stream
        self._check(self.cu.cuLaunchKernel(self.fn[name], grid[0], grid[1], grid[2], block[0], block[1], block[2], 0,
                                           ctypes.c_void_p(stream), ptrs, None), name)


def _guarded(n, device):
    """A length-n float32 view with one readable element in front of it."""
    import torch

    store = torch.zeros(n + 64, dtype=torch.float32, device=device)
    return store, store[64:]


def _set_guard(store, view):
    store[63:64].copy_(view[0:1])


def iteration(rk: RefKernels, phi, img, taps, W, H, L, sigma, e, dt, v, meu, sigma2=0.0):
    """One reference iteration on device tensors phi, img (float32, L*H*W);
    returns (phi_new, dict of the reference's intermediate fields)."""
    import torch

    c_i = ctypes.c_int
    dev = phi.device
    n = W * H * L
    size = int(7.0 * sigma)          # main.cpp:121, K.X()
    p = int(7.0 * sigma)
    if p % 2 == 0:                   # main.cpp:152-154
        p += 1
    if size != p:
        raise ValueError("the reference's result is undefined for even floor(7 sigma)")
    k_size = int(7.0 * sigma)        # main.cpp:264
    pad_w = int((k_size - 1) // 2)   # main.cpp:273
    T = (16, 16, 4)
    G = (W // 16 + 1, H // 16 + 1, L // 4 + 1)
    T32 = (32, 32, 1)
    G32 = (W // 32 + 1, H // 32 + 1, L + 1)
    f = {}

    def buf():
        return torch.empty(n, dtype=torch.float32, device=dev)

    phi_store, phi_g = _guarded(n, dev)
    phi_g.copy_(phi)
    _set_guard(phi_store, phi_g)
    dims = (c_i(W), c_i(H), c_i(L))
    HD_out, I_out, HD_in, I_in = buf(), buf(), buf(), buf()
    rk.launch("heaviside", G, T, HD_out, phi_g, *dims)                       # main.cpp:234
    rk.launch("multiplication", G, T, I_out, img, HD_out, *dims)             # main.cpp:238
    rk.launch("inverse", G, T, HD_in, HD_out, *dims)                         # main.cpp:242
    rk.launch("multiplication", G, T, I_in, img, HD_in, *dims)               # main.cpp:246
    gx_store, gx = _guarded(n, dev)
    gy, gz = buf(), buf()
    rk.launch("gradient_dx_cuda", G, T, phi_g, gx, *dims)                    # main.cpp:250
    rk.launch("gradient_dy_cuda", G, T, phi_g, gy, *dims)
    rk.launch("gradient_dz_cuda", G, T, phi_g, gz, *dims)
    _set_guard(gx_store, gx)
    mag = buf()
    rk.launch("gradientmagnitude", G, T, mag, gx, gy, gz, *dims)             # main.cpp:252
    nx_store, nx = _guarded(n, dev)
    ny, nz = buf(), buf()
    rk.launch("division_grad", G, T, nx, gx, mag, *dims)                     # main.cpp:254
    rk.launch("division_grad", G, T, ny, gy, mag, *dims)
    rk.launch("division_grad", G, T, nz, gz, mag, *dims)
    _set_guard(nx_store, nx)
    dnx, dny, dnz = buf(), buf(), buf()
    rk.launch("gradient_dx_cuda", G32, T32, nx, dnx, *dims)                  # main.cpp:256
    rk.launch("gradient_dy_cuda", G32, T32, ny, dny, *dims)
    rk.launch("gradient_dz_cuda", G32, T32, nz, dnz, *dims)
    kappa = buf()
    rk.launch("plus", G, T, kappa, dnx, dny, dnz, *dims)                     # main.cpp:258
    dgx, dgy, dgz, lap = buf(), buf(), buf(), buf()
    rk.launch("gradient_dx_cuda", G, T, gx, dgx, *dims)                      # main.cpp:260
    rk.launch("gradient_dy_cuda", G, T, gy, dgy, *dims)
    rk.launch("gradient_dz_cuda", G, T, gz, dgz, *dims)
    rk.launch("plus", G, T, lap, dgx, dgy, dgz, *dims)
    xW, yH, zL = W - p + 1, H - p + 1, L - p + 1

    def blur(src):                                                           # kernel.cu:1051-1121
        ox = torch.empty(max(xW, 1) * H * L, dtype=torch.float32, device=dev)
        oy = torch.empty(max(xW, 1) * max(yH, 1) * L, dtype=torch.float32, device=dev)
        oz = torch.empty(max(xW, 1) * max(yH, 1) * max(zL, 1), dtype=torch.float32, device=dev)
        kk = ctypes.c_uint(p)
        rk.launch("Convolution__on_X", G, T, ox, src, taps, c_i(W), c_i(L), c_i(H), c_i(xW), c_i(H), c_i(L), kk)
        rk.launch("Convolution__on_Y", G, T, oy, ox, taps, c_i(xW), c_i(L), c_i(H), c_i(xW), c_i(yH), c_i(L), kk)
        rk.launch("Convolution__on_Z", G, T, oz, oy, taps, c_i(xW), c_i(L), c_i(yH), c_i(xW), c_i(yH), c_i(zL), kk)
        return oz

    def pad(src):                                                            # kernel.cu:331-362
        out = buf()
        pw, ph, pl = xW + 2 * pad_w, yH + 2 * pad_w, zL + 2 * pad_w
        rk.launch("pad_border", (pw // 16 + 1, ph // 16 + 1, pl // 4 + 1), T, out, src, c_i(xW), c_i(yH), c_i(zL),
                  c_i(pad_w), c_i(pw), c_i(ph), c_i(pl))
        return out

    I_ob, HD_ob = pad(blur(I_out)), pad(blur(HD_out))                       # main.cpp:268-275
    fout = buf()
    rk.launch("division", G, T, fout, I_ob, HD_ob, *dims)                    # main.cpp:277
    I_ib, HD_ib = pad(blur(I_in)), pad(blur(HD_in))                         # main.cpp:282-287
    fin = buf()
    rk.launch("division", G, T, fin, I_ib, HD_ib, *dims)                     # main.cpp:289
    Eo, Ei = buf(), buf()
    rk.launch("Eout_Ein_calculation", G, T, Eo, Ei, fout, fin, img, *dims, c_i(int(sigma2)))  # main.cpp:293
    dh = buf()
    rk.launch("deri_heaviside", G, T, dh, phi_g, *dims)                      # main.cpp:296
    out = buf()
    rk.launch("Final_phi", G, T, out, phi_g, dh, Eo, Ei, kappa, lap, ctypes.c_float(e), ctypes.c_float(dt),
              ctypes.c_float(v), ctypes.c_float(meu), *dims)                 # main.cpp:300
    torch.cuda.synchronize()
    f.update(H=HD_out, gx=gx, gy=gy, gz=gz, mag=mag, nx=nx, ny=ny, nz=nz, kappa=kappa, lap=lap, I_ob=I_ob,
             HD_ob=HD_ob, I_ib=I_ib, HD_ib=HD_ib, fout=fout, fin=fin, Eo=Eo, Ei=Ei, dh=dh)
    return out, f


def evolve(rk: RefKernels, phi, img, taps, W, H, L, iters, **params):
    fields = None
    for _ in range(iters):
        phi, fields = iteration(rk, phi, img, taps, W, H, L, **params)
    return phi, fields
