"""TEST INFRASTRUCTURE ONLY: the RSF step in float64 PyTorch, differentiable by
autograd.  It is the checker for the hand-written adjoint (gradients of phi0
and lambda1, lambda2, mu, nu) beside FP64 central differences of the C
oracle; no product path imports it.

It restates the same step as oracle/rsf_oracle.c (reference files cited
there): H = 0.5 (1 + 2/pi atan(phi/eps)) (CUDA_RSF/kernel.cu:248-263), the
valid separable correlation of I H, H, I (1-H), 1-H with the unnormalised
taps and a border band of 30 (kernel.cu:1000-1121, 300-362), f = blur ratio
(kernel.cu:191-207), e = (I - f)^2 (kernel.cu:25-55 with sigma2 = 0), central
differences with the reference boundary rules (kernel.cu:57-125),
n = g / (|g| + 1e-6) (kernel.cu:173-189), kappa = sum D_a n_a, Lap =
sum D_a D_a phi (kernel.cu:630-684, 744-909) and the update of
kernel.cu:365-387 with the data factor lambda1 e_out - lambda2 e_in.
Arithmetic is plain float64 (no attempt at the FP32 operation order).
"""
from __future__ import annotations

import math

import numpy as np
import torch


def _neighbours(shape, boundary=0, device=None):
    """(right, left) flat index arrays of the central difference on each axis."""
    L, H, W = shape
    idx = np.arange(L * H * W, dtype=np.int64).reshape(L, H, W)
    z, y, x = np.meshgrid(np.arange(L), np.arange(H), np.arange(W), indexing="ij")
    out = []
    # x: interior i +- 1; x = W-1 -> (i, i-1); x = 0 -> (i+1, i-1 linear) or (i+1, i) clamp; voxel 0 -> (1, 0)
    r = np.where(x + 1 < W, idx + 1, idx)
    if boundary == 0:
        l = np.where(x > 0, idx - 1, np.maximum(idx - 1, 0))
    else:
        l = np.where(x > 0, idx - 1, idx)
    l = np.where(x == W - 1, idx - 1, l)
    out.append((r.ravel(), l.ravel()))
    for q, n, stride in ((y, H, W), (z, L, W * H)):
        qr = np.minimum(q + 1, n - 1)
        ql = np.maximum(q - 1, 0)
        out.append(((idx + (qr - q) * stride).ravel(), (idx + (ql - q) * stride).ravel()))
    return [(torch.from_numpy(a).to(device), torch.from_numpy(b).to(device)) for a, b in out]


def _blur_valid(f, taps):
    k = taps.numel()
    w = taps.to(f.dtype)
    v = f[None, None]
    v = torch.nn.functional.conv3d(v, w.view(1, 1, 1, 1, k))
    v = torch.nn.functional.conv3d(v, w.view(1, 1, 1, k, 1))
    v = torch.nn.functional.conv3d(v, w.view(1, 1, k, 1, 1))
    return v[0, 0]


class Step:
    """phi' = step(phi, I, lambda1, lambda2, mu, nu) for one volume shape;
    `device` is where its index and tap tensors live (that of phi and I)."""

    def __init__(self, shape, taps, dt, eps, boundary=0, device=None):
        self.shape = tuple(shape)
        self.taps = torch.as_tensor(np.asarray(taps, dtype=np.float64)).to(device)
        self.k = self.taps.numel()
        self.r = (self.k - 1) // 2
        self.dt, self.eps = float(dt), float(eps)
        self.nb = _neighbours(self.shape, boundary, device)

    def _d(self, f, axis):
        r, l = self.nb[axis]
        flat = f.reshape(-1)
        return (0.5 * (flat[r] - flat[l])).view(self.shape)

    def _blur_padded(self, f):
        L, H, W = self.shape
        k, r = self.k, self.r
        if W - k + 1 <= 0 or H - k + 1 <= 0 or L - k + 1 <= 0:
            return torch.full_like(f, 30.0)
        b = _blur_valid(f, self.taps)
        Lv, Hv, Wv = b.shape
        return torch.nn.functional.pad(b, (r, W - Wv - r, r, H - Hv - r, r, L - Lv - r), value=30.0)

    def __call__(self, phi, I, lambda1, lambda2, mu, nu):
        eps, dt = self.eps, self.dt
        h = 0.5 * (1.0 + (2.0 / math.pi) * torch.atan(phi / eps))
        hi = 1.0 - h
        fo = self._blur_padded(I * h) / self._blur_padded(h)
        fi = self._blur_padded(I * hi) / self._blur_padded(hi)
        eo = (I - fo) ** 2
        ei = (I - fi) ** 2
        g = [self._d(phi, a) for a in range(3)]
        sq = g[0] * g[0] + g[1] * g[1] + g[2] * g[2]
        mag = torch.sqrt(torch.clamp(sq, min=1e-300))  # zero derivative where g = 0
        n = [ga / (mag + 1e-6) for ga in g]
        kap = self._d(n[0], 0) + self._d(n[1], 1) + self._d(n[2], 2)
        lap = self._d(g[0], 0) + self._d(g[1], 1) + self._d(g[2], 2)
        delta = (1.0 / math.pi) * eps / (eps * eps + phi * phi)
        data = lambda1 * eo - lambda2 * ei
        return phi - dt * delta * data + nu * dt * delta * kap + mu * dt * (lap - kap)


def evolve(phi0, I, taps, params: dict, iters: int, boundary=0):
    """phi_T in float64 with autograd through every step.  params: dt, eps,
    lambda1, lambda2, mu, nu (the last four floats or float64 tensors)."""
    step = Step(phi0.shape, taps, params["dt"], params["eps"], boundary, phi0.device)
    phi = phi0
    for _ in range(iters):
        phi = step(phi, I, params["lambda1"], params["lambda2"], params["mu"], params["nu"])
    return phi
