"""A small, self-contained evolution for profiler captures.

    python profile_case.py --n 320 --sigma 3 --iters 2
    python profile_case.py --n 128 --sigma 3 --iters 1 --adjoint 2

Evolves one n^3 volume (a smooth level set and a random uint8 image, made on
the device) for `iters` iterations through the C ABI and exits.  At n = 320
the working set is about 1.4 GB, larger than L2, so DRAM counters of one
launch mean what they say.  `--adjoint S` then runs S adjoint steps
(rsf_step_adjoint) at the evolved level set; `--time N` then times N
forward iterations and N adjoint steps with CUDA events, and with
`--batch B` the same for a batch of B copies of the volume.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent / "paper-rsf-vesselseg_gb300"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=320)
    ap.add_argument("--sigma", type=float, default=3.0)
    ap.add_argument("--iters", type=int, default=2)
    ap.add_argument("--adjoint", type=int, default=0, help="adjoint steps after the evolution")
    ap.add_argument("--time", type=int, default=0,
                    help="then time this many forward iterations and adjoint steps with CUDA events")
    ap.add_argument("--batch", type=int, default=1,
                    help="with --time: also time a batch of this many volumes (rsf_evolve_batched, "
                         "rsf_step_adjoint_batched)")
    args = ap.parse_args()
    import torch

    from rsf_gb300 import Params, Workspace

    n = args.n
    dev = torch.device("cuda:0")
    ax = torch.arange(n, device=dev, dtype=torch.float32)
    z, y, x = torch.meshgrid(ax, ax, ax, indexing="ij")
    phi = (3 * torch.sin(x * 0.07) * torch.sin(y * 0.05 + 1) * torch.sin(z * 0.06 + 2)).clamp(-3, 3).contiguous()
    del x, y, z
    gen = torch.Generator(device=dev)
    gen.manual_seed(0)
    img = torch.randint(0, 256, (n, n, n), dtype=torch.uint8, device=dev, generator=gen)
    p = Params(sigma=args.sigma, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)
    with Workspace(n ** 3 * max(1, args.batch), max(1, args.batch)) as ws:
        ws.evolve(img, phi, p, args.iters)
        ws.check()
        if args.adjoint:
            u = torch.randn(phi.shape, device=dev, generator=gen)
            out = torch.empty_like(phi)
            grads = torch.zeros(4, dtype=torch.float64, device=dev)
            for _ in range(args.adjoint):
                ws.step_adjoint(img, phi, u, p, out=out, param_grads=grads)
            ws.check()
        if args.time:
            e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            u = torch.randn(phi.shape, device=dev, generator=gen)
            out = torch.empty_like(phi)
            grads = torch.zeros(4, dtype=torch.float64, device=dev)
            work = phi.clone()
            ws.evolve(img, work, p, 2)
            ws.step_adjoint(img, phi, u, p, out=out, param_grads=grads)
            torch.cuda.synchronize()
            e[0].record()
            ws.evolve(img, work, p, args.time)
            e[1].record()
            e[2].record()
            for _ in range(args.time):
                ws.step_adjoint(img, phi, u, p, out=out, param_grads=grads)
            e[3].record()
            torch.cuda.synchronize()
            ws.check()
            fwd = e[0].elapsed_time(e[1]) / args.time
            adj = e[2].elapsed_time(e[3]) / args.time
            print(f"forward step {fwd * 1e3:.1f} us, adjoint step {adj * 1e3:.1f} us, ratio {adj / fwd:.2f}")
            if args.batch > 1:
                B = args.batch
                works = [phi.clone() for _ in range(B)]
                pairs = [(img, w) for w in works]
                items = [(img, phi, u, torch.empty_like(phi)) for _ in range(B)]
                ws.evolve_batched(pairs, p, 2)
                ws.step_adjoint_batched(items, p, param_grads=grads)
                torch.cuda.synchronize()
                e[0].record()
                ws.evolve_batched(pairs, p, args.time)
                e[1].record()
                e[2].record()
                for _ in range(args.time):
                    ws.step_adjoint_batched(items, p, param_grads=grads)
                e[3].record()
                torch.cuda.synchronize()
                ws.check()
                fwd = e[0].elapsed_time(e[1]) / args.time
                adj = e[2].elapsed_time(e[3]) / args.time
                print(f"batch of {B}: forward step {fwd * 1e3:.1f} us, adjoint step {adj * 1e3:.1f} us, "
                      f"ratio {adj / fwd:.2f}")
    torch.cuda.synchronize()
    print(f"profile case done: {n}^3, sigma {args.sigma}, {args.iters} iterations, {args.adjoint} adjoint steps")


if __name__ == "__main__":
    main()
