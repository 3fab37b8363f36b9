"""Times the reference's own GPU kernels beside ours on the same GB300.

TEST INFRASTRUCTURE ONLY: the reference's kernels (CUDA_RSF/kernel.cu,
compiled unchanged into oracle/_ref by oracle/ref_build.py) run through
oracle/ref_harness.py in the order of CUDA_RSF/main.cpp:233-300 with their
own launch shapes, on device-resident buffers.  That is faster than the
reference executable, whose host wrappers copy every operand to and from
the host and allocate per call (kernel.cu:127-1236); the figure here is the
reference's kernels alone (plus the harness's launch overhead, about 40
launches per iteration from Python).

Ours runs through the C ABI (rsf_gb300.Workspace.evolve) on the same
inputs, in both arithmetic modes.  The reference-arithmetic result must be
bit-identical to the reference's after the same iterations, and the
portable one must keep >= 99.99 % sign agreement with it.

    python oracle/time_ref_kernels.py --shape 64 288 288 --sigma 3 --iters 10

Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
for p in (str(ROOT), str(ROOT / "paper-rsf-vesselseg_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def _inputs(shape, device):
    import torch

    from rsf_gb300.autotune import smooth_phi

    gen = torch.Generator(device=device)
    gen.manual_seed(5)
    img = torch.randint(0, 256, tuple(shape), generator=gen, device=device, dtype=torch.uint8)
    return img, smooth_phi(shape, device)


def _timed(fn, iters):
    import torch

    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    out = fn(iters)
    e1.record()
    torch.cuda.synchronize()
    return out, e0.elapsed_time(e1) / iters


def main(argv=None):
    import numpy as np
    import torch

    from oracle import ref_harness, rsf_oracle as orc
    from rsf_gb300 import Params, Workspace

    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", type=int, nargs=3, default=[64, 288, 288], help="L H W")
    ap.add_argument("--sigma", type=float, default=3.0)
    ap.add_argument("--iters", type=int, default=10)
    args = ap.parse_args(argv)
    if not ref_harness.available():
        raise SystemExit("the reference's kernels are not built (oracle/ref_build.py)")
    L, H, W = args.shape
    dev = torch.device("cuda:0")
    img, phi0 = _inputs(args.shape, dev)
    # the reference's command-line defaults (main.cpp:91-97) with --sigma
    e, dt, v, meu = 0.1, 0.1, 1e-4, 1.0
    rk = ref_harness.RefKernels()
    taps = torch.from_numpy(orc.taps(args.sigma)).to(dev)
    imf = img.float().ravel()

    def run_ref(n):
        out, _ = ref_harness.evolve(rk, phi0.ravel().clone(), imf, taps, W, H, L, n, sigma=args.sigma, e=e,
                                    dt=dt, v=v, meu=meu)
        return out

    run_ref(1)  # module load, allocator warm-up
    ref_out, ref_ms = _timed(run_ref, args.iters)

    res = {}
    with Workspace(L * H * W) as ws:
        for arith in ("reference", "portable"):
            p = Params.from_flags(sigma=args.sigma, dt=dt, meu=meu, e=e, v=v, arith=arith)

            def run_ours(n, p=p):
                phi = phi0.clone()
                ws.evolve(img, phi, p, n)
                return phi

            run_ours(1)
            out, ms = _timed(run_ours, args.iters)
            ws.check()
            res[arith] = (out.ravel(), ms)
    a = ref_out.cpu().numpy()
    b_ref = res["reference"][0].cpu().numpy()
    b_por = res["portable"][0].cpu().numpy()
    vox = L * H * W
    line = {
        "shape_lhw": [L, H, W], "sigma": args.sigma, "iterations": args.iters,
        "params": {"e": e, "dt": dt, "v": v, "meu": meu, "eps": 0.2},
        "reference_kernels": {"ms_per_iter": ref_ms, "gvoxel_iter_s": vox / ref_ms / 1e6,
                              "how": "kernel.cu compiled unchanged, launched per op from a Python harness, "
                                     "device-resident buffers (no per-op host copies)"},
        "ours_reference_arith": {"ms_per_iter": res["reference"][1], "gvoxel_iter_s": vox / res["reference"][1] / 1e6,
                                 "bit_identical_to_reference": bool(np.array_equal(a.view(np.uint32),
                                                                                   b_ref.view(np.uint32)))},
        "ours_portable": {"ms_per_iter": res["portable"][1], "gvoxel_iter_s": vox / res["portable"][1] / 1e6,
                          "sign_agreement_with_reference": float(np.mean(np.signbit(a) == np.signbit(b_por))),
                          "max_abs_diff_over_max_abs_phi": float(np.abs(a.astype(np.float64) - b_por).max()
                                                                 / max(float(np.abs(a).max()), 1e-30))},
    }
    line["speedup_portable_vs_reference_kernels"] = ref_ms / res["portable"][1]
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
