"""Differentiable RSF evolution for PyTorch callers (the U-Net side).

`evolve(phi0, image, params, iters, ...)` runs the same CUDA evolution as
`Workspace.evolve` and returns phi_T as a tensor that autograd can
differentiate with respect to phi0 and to lambda1, lambda2, mu, nu.

A batch of volumes of one shape, phi0 and image of shape (B, L, H, W), runs
as one batch: `rsf_evolve_batched` forward and `rsf_step_adjoint_batched`
backward, one launch sequence per step for the whole batch.

Forward keeps phi every `checkpoint_every` steps (T / C + 1 volumes).
Backward walks the segments from the last: it recomputes the segment's
states from its checkpoint with the forward kernels (bit-identical to the
first pass), then chains `rsf_step_adjoint` backwards through them, so the
memory is (T / C + C) volumes instead of T.  The reference has no derivative
of its evolution (CUDA_RSF/main.cpp:222-314 only steps forward).
"""
from __future__ import annotations

import dataclasses

import torch

from .api import Params, Workspace

_PARAM_NAMES = ("lambda1", "lambda2", "mu", "nu")


def _step(ws: Workspace, image: torch.Tensor, phi: torch.Tensor, p: Params, n: int) -> None:
    """n iterations of phi in place: one volume (L, H, W) or a batch (B, L, H, W)."""
    if image.dim() == 4:
        ws.evolve_batched(list(zip(image.unbind(0), phi.unbind(0))), p, n)
    else:
        ws.evolve(image, phi, p, n)


class _Evolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, phi0, image, lambda1, lambda2, mu, nu, params, iters, every, ws):
        # The kernels take the parameters by value: host tensors are read
        # without a device synchronisation, device tensors with one transfer
        # for all four.
        ts = [t.detach().reshape(()).to(torch.float64) for t in (lambda1, lambda2, mu, nu)]
        if any(t.is_cuda for t in ts):
            d = next(t.device for t in ts if t.is_cuda)
            ts = torch.stack([t.to(d) for t in ts]).cpu().unbind()
        vals = {n: float(t) for n, t in zip(_PARAM_NAMES, ts)}
        p = dataclasses.replace(params, **vals)
        phi = phi0.detach().to(torch.float32).contiguous().clone()
        ckpts = []
        t = 0
        while t < iters:
            ckpts.append(phi.clone())
            n = min(every, iters - t)
            _step(ws, image, phi, p, n)
            t += n
        ctx.save_for_backward(image, *ckpts)
        ctx.p, ctx.iters, ctx.every, ctx.ws = p, iters, every, ws
        ctx.pmeta = [(t.dtype, t.device, t.shape) for t in (lambda1, lambda2, mu, nu)]
        return phi

    @staticmethod
    def backward(ctx, grad):
        image, *ckpts = ctx.saved_tensors
        ws, p, iters, every = ctx.ws, ctx.p, ctx.iters, ctx.every
        u = grad.detach().to(torch.float32).contiguous().clone()
        tmp = torch.empty_like(u)
        g = torch.zeros(4, dtype=torch.float64, device=u.device)
        for s in reversed(range(len(ckpts))):
            n = min(every, iters - s * every)
            states = [ckpts[s]]
            for _ in range(1, n):
                nxt = states[-1].clone()
                _step(ws, image, nxt, p, 1)
                states.append(nxt)
            for i in reversed(range(n)):
                if image.dim() == 4:
                    ws.step_adjoint_batched(list(zip(image.unbind(0), states[i].unbind(0), u.unbind(0),
                                                     tmp.unbind(0))), p, param_grads=g)
                else:
                    ws.step_adjoint(image, states[i], u, p, out=tmp, param_grads=g)
                u, tmp = tmp, u
        out = [u if ctx.needs_input_grad[0] else None, None]
        for k, (dtype, device, shape) in enumerate(ctx.pmeta):
            out.append(g[k].to(dtype=dtype, device=device).reshape(shape) if ctx.needs_input_grad[2 + k] else None)
        return tuple(out) + (None, None, None, None)


def evolve(phi0: torch.Tensor, image: torch.Tensor, params: Params, iters: int, lambda1=None, lambda2=None, mu=None,
           nu=None, checkpoint_every: int = 10, workspace: Workspace | None = None) -> torch.Tensor:
    """phi_T after `iters` steps, differentiable in phi0 and in any of
    lambda1, lambda2, mu, nu passed as tensors (others come from `params`).
    phi0 and image are CUDA tensors (L, H, W), or (B, L, H, W) for a batch
    that shares the parameters; image uint8 or float32.
    Parameter tensors on the host are read without synchronising the device;
    CUDA parameter tensors cost one device-to-host transfer per call."""
    if iters < 1:
        raise ValueError("iters must be >= 1")
    if checkpoint_every < 1:
        raise ValueError("checkpoint_every must be >= 1")
    if phi0.dim() not in (3, 4) or image.shape != phi0.shape:
        raise ValueError("phi0 and image must both be (L, H, W) or both (B, L, H, W)")
    ws = workspace if workspace is not None else Workspace(phi0.numel(), phi0.shape[0] if phi0.dim() == 4 else 1)
    args = []
    for name, v in zip(_PARAM_NAMES, (lambda1, lambda2, mu, nu)):
        # parameters that are not tensors become host scalars (no gradient)
        if v is None:
            v = torch.tensor(float(getattr(params, name)), dtype=torch.float64)
        elif not torch.is_tensor(v):
            v = torch.tensor(float(v), dtype=torch.float64)
        args.append(v)
    return _Evolve.apply(phi0, image.contiguous(), *args, params, int(iters), int(checkpoint_every), ws)


def soft_dice_loss(phi: torch.Tensor, mask: torch.Tensor, eps: float) -> torch.Tensor:
    """1 - 2 sum(H m) / (sum H + sum m) with H = 0.5 (1 + 2/pi atan(phi/eps))."""
    h = 0.5 * (1.0 + (2.0 / torch.pi) * torch.atan(phi / eps))
    m = mask.to(h.dtype)
    return 1.0 - 2.0 * (h * m).sum() / (h.sum() + m.sum())
