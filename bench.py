#!/usr/bin/env python
"""Benchmark of batched RSF level-set evolution on GB300.

Workload: 48 overlapping sub-volumes of uneven shape (extents 64-320 voxels)
cut from a 512 x 1024 x 1024 synthetic vessel volume (800 Catmull-Rom tubes,
radius U[1.5, 8], vessel N(180,20), background N(40,15), noise N(0,10), sine
bias field), phi0 the +-3-clipped signed distance of a per-tube dilated or
eroded mask; sigma 3 (21 taps), lambda1 = lambda2 = 1, mu 1,
nu 0.001*255^2, eps 1, dt 0.1, 150 iterations.  One step = one full
150-iteration evolution of all 48 sub-volumes (one batched call, the
iteration loop replayed from a captured CUDA graph).

Metric: Gvoxel-iterations/s (voxels of all sub-volumes, halos included,
times iterations, per second), aggregated over ranks.  With --gpus N every
rank evolves its own 48-sub-volume batch (weak scaling, no collective on
the data path).

--impl reference times the CPU oracle (the restatement of the reference's
kernel.cu arithmetic; the reference has no CPU implementation of its own)
on the host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "paper-rsf-vesselseg_gb300"))

METRIC = "Gvoxel-iterations/s (batched RSF evolution)"
UNIT = "Gvoxel-iter/s"
ITERS = 150
SIGMA = 3.0
PARAMS = dict(sigma=SIGMA, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=0.001 * 255.0 ** 2, eps=1.0)
WORKLOAD = ("config2: 48 uneven sub-volumes (extents 64-320 per axis, 256^3 cores + 32-voxel halos) cut from a "
            "512x1024x1024 synthetic vessel volume (800 tubes, radius U[1.5,8]); sigma 3 (21 taps), lambda 1, mu 1, "
            "nu 0.001*255^2, eps 1, dt 0.1; 150 iterations; phi float32, image uint8")
SPEC = "CONFIG2"        # synth volume spec of the workload
TILES = "config2_tiles"  # tiling of the workload

# --workload gigavoxel: the 1024^3 volume in 27 tiles (384/384/256 cores +
# 32-voxel halos, 1.53 G tile voxels), sigma 4, 200 iterations.  Not the
# default line: a second measurement of the same kernels at larger scale.
GIGAVOXEL = dict(
    ITERS=200, SIGMA=4.0, SPEC="CONFIG3", TILES="config3_tiles",
    WORKLOAD=("config3: 27 sub-volumes (384/384/256 cores + 32-voxel halos, extents 288-448) of a 1024^3 "
              "synthetic vessel volume (2000 tubes, radius U[1,10]); sigma 4 (29 taps), lambda 1, mu 1, "
              "nu 0.001*255^2, eps 1, dt 0.1; 200 iterations; phi float32, image uint8"))


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def algorithmic_bytes(tiles, k):
    return algorithmic_bytes_shapes([t.shape for t in tiles], k)


def algorithmic_bytes_shapes(shapes, k):
    """Bytes each kernel must move once per launch over the whole batch:
    x-pass reads phi (4) and I (1) and writes 4 fields of the x-valid extent;
    y-pass reads those and writes 4 fields of the xy-valid extent; z-pass
    reads those and I and writes the data factor of the valid region; the
    stencil reads phi and the data factor and writes phi."""
    out = {"xpass": 0, "ypass": 0, "zpass": 0, "stencil": 0}
    for shape in shapes:
        L, H, W = shape
        Wv, Hv, Lv = max(W - k + 1, 0), max(H - k + 1, 0), max(L - k + 1, 0)
        if min(Wv, Hv, Lv) == 0:
            Wv = Hv = Lv = 0
        n = W * H * L
        out["xpass"] += 5 * n + 16 * Wv * H * L
        out["ypass"] += 16 * Wv * H * L + 16 * Wv * Hv * L
        out["zpass"] += 16 * Wv * Hv * L + 5 * Wv * Hv * Lv
        out["stencil"] += 12 * n
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_ratio(kernel: str):
    """DRAM bytes / algorithmic bytes of `kernel` in the committed ncu capture
    (profiles/traffic.json: one launch of a 320^3 volume, larger than L2)."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    k = json.loads(p.read_text()).get("kernels", {}).get(kernel)
    return None if k is None else float(k["ratio"])


def ncu_warp_inst_per_voxel(kernel: str):
    """Warp instructions issued per voxel by `kernel` in the committed ncu
    capture (profiles/traffic.json), or None."""
    p = ROOT / "profiles" / "traffic.json"
    if not p.exists():
        return None
    k = json.loads(p.read_text()).get("kernels", {}).get(kernel)
    return None if k is None or "warp_inst_per_voxel" not in k else float(k["warp_inst_per_voxel"])


def cpu_sample(threads: int, budget_s: float = 15.0):
    """Times the CPU oracle on one sub-volume of the workload's shape class
    (the 64 x 288 x 288 corner tile), iterations sized to ~budget_s."""
    import numpy as np

    from oracle import rsf_oracle as orc
    from rsf_gb300 import synth

    shape = (64, 288, 288)
    img, phi0, _ = synth.make_volume(synth.VolumeSpec(shape, 12, 1.5, 8.0, 20))
    p = orc.params(**{k: v for k, v in PARAMS.items()})
    imgf = img.astype(np.float32)
    t0 = time.perf_counter()
    orc.evolve(phi0, imgf, p, 1, threads)
    one = max(time.perf_counter() - t0, 1e-3)
    iters = int(max(2, min(200, budget_s / one)))
    t0 = time.perf_counter()
    want = orc.evolve(phi0, imgf, p, iters, threads)
    dt = time.perf_counter() - t0
    vox = img.size * iters
    base = {"value": vox / dt / 1e9, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"CPU oracle (C, OpenMP, {threads} threads), one {shape[2]}x{shape[1]}x{shape[0]} sub-volume "
                      f"of the workload's shape class, {iters} iterations, {dt:.1f} s"}
    return base, (img, phi0, iters, want)


def parity_on_sample(sample):
    """The CUDA path on the CPU baseline's sample, against the oracle's result
    for the same iterations: bit equality, sign (mask) agreement, max |dphi|."""
    import numpy as np
    import torch

    from rsf_gb300 import Params, Workspace

    img, phi0, iters, want = sample
    dev = torch.device("cuda", torch.cuda.current_device())
    tp = torch.from_numpy(phi0).to(dev)
    with Workspace(phi0.size) as ws:
        ws.evolve(torch.from_numpy(img).to(dev), tp, Params(**PARAMS), iters)
        ws.check()
    got = tp.cpu().numpy()
    return {"checked_against": "CPU oracle on the cpu_baseline sample",
            "iterations": iters, "bit_identical": bool(np.array_equal(got.view(np.uint32), want.view(np.uint32))),
            "mask_agreement": float((np.sign(got) == np.sign(want)).mean()),
            "max_abs_diff_over_max_abs_phi": float(np.abs(got.astype(np.float64) - want).max() / np.abs(want).max())}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np

    from oracle import rsf_oracle as orc
    from rsf_gb300 import synth

    threads = os.cpu_count() or 1
    shape = (64, 288, 288)
    img, phi0, _ = synth.make_volume(synth.VolumeSpec(shape, 12, 1.5, 8.0, 20))
    imgf = img.astype(np.float32)
    p = orc.params(**PARAMS)
    iters_per_step = 10
    for _ in range(args.warmup):
        orc.evolve(phi0, imgf, p, iters_per_step, threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.evolve(phi0, imgf, p, iters_per_step, threads)
    dt = time.perf_counter() - t0
    value = img.size * iters_per_step * args.steps / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "reference_step": f"{iters_per_step} iterations of one {shape[2]}x{shape[1]}x"
                   f"{shape[0]} sub-volume of the workload (bounded CPU sample)", "parallelism": f"dp{args.gpus}"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"CPU oracle (C, OpenMP, {threads} threads); the reference has no CPU code path"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def _config0_volume(seed):
    """One 128^3 volume of the 128^3 generator (CPU, per-region perturbation)."""
    from rsf_gb300 import synth

    return synth.make_volume(synth.VolumeSpec((128, 128, 128), 12, 2.0, 6.0, seed))


def differentiable_sample(dev):
    """The differentiable workload as specified: a batch of 8 volumes of
    128^3 from the 128^3 generator (seeds 40-47; uint8 image in 0-255,
    phi0 the +-3-clipped signed distance of the perturbed mask), sigma 3,
    lambda1 = lambda2 = 1, mu 1, nu 0.001*255^2, eps 1, dt 0.1, 50 forward
    iterations with checkpoints every 10, loss = mean soft-Dice of H(phi_T)
    against the true tube mask, backward through the hand-written adjoint;
    gradients of phi0 and of lambda1, lambda2, mu, nu.  Returns the forward +
    backward time per batch and the throughput in forward voxel-iterations
    per second of the whole forward + backward job.

    At this phi0 the exact 50-step gradient overflows FP32: where the
    clipped distance is flat, n = g/(|g| + 1e-6) has derivative 1e6 and each
    step multiplies the gradient by up to ~1e5 (the float64 restatement
    measures ~1e80).  The kernels run the same work either way; the record
    says whether the workspace check reported the overflow."""
    import multiprocessing as mp

    import torch

    from rsf_gb300 import Params, RsfError, Workspace, autograd

    # the generator is CPU-bound: one spawned process per volume
    with mp.get_context("spawn").Pool(8) as pool:
        vols_np = pool.map(_config0_volume, range(40, 48))
    p = Params(sigma=3.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=0.001 * 255.0 ** 2, eps=1.0)
    imgs = torch.stack([torch.from_numpy(img) for img, _, _ in vols_np]).to(dev)
    phi0s = torch.stack([torch.from_numpy(phi0) for _, phi0, _ in vols_np]).to(dev)
    masks = torch.stack([torch.from_numpy(mask) for _, _, mask in vols_np]).to(dev)
    nb = imgs.shape[0]
    ws = Workspace(imgs.numel(), nb)
    names = ("lambda1", "lambda2", "mu", "nu")
    grads = {}

    def batch():
        # parameter leaves on the host: reading their values costs no device sync
        prm = {n: torch.tensor(float(getattr(p, n)), dtype=torch.float64, requires_grad=True) for n in names}
        x = phi0s.clone().requires_grad_(True)
        # the 8 volumes as one batch: one launch sequence per step forward
        # (rsf_evolve_batched) and backward (rsf_step_adjoint_batched)
        out = autograd.evolve(x, imgs, p, 50, checkpoint_every=10, workspace=ws, **prm)
        loss = sum(autograd.soft_dice_loss(out[b], masks[b], p.eps) for b in range(nb))
        (loss / nb).backward()
        grads["phi0_l2"] = float(torch.sqrt((x.grad.double() ** 2).sum()))
        for n in names:
            grads[n] = float(prm[n].grad)
        grads["loss"] = float(loss) / nb
        try:
            ws.check()
            grads["check"] = "ok"
        except RsfError as err:
            grads["check"] = str(err)

    batch()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    batch()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    ws.close()
    num = {k: v for k, v in grads.items() if isinstance(v, float)}
    finite = all(v == v and abs(v) != float("inf") for v in num.values())
    # JSON has no NaN or infinity: non-finite values are reported as null
    grads = {k: (v if not isinstance(v, float) or (v == v and abs(v) != float("inf")) else None)
             for k, v in grads.items()}
    return {"workload": "config4: 8 x 128^3 (128^3 generator, seeds 40-47, uint8 image 0-255, phi0 the +-3-clipped "
                        "signed distance), sigma 3, lambda1 = lambda2 = 1, mu 1, nu 0.001*255^2, eps 1, dt 0.1, "
                        "50 iterations, checkpoints every 10, mean soft-Dice loss; gradients of phi0, lambda1, "
                        "lambda2, mu, nu; the 8 volumes batched forward and backward",
            "fwd_bwd_ms_per_batch": ms, "value": 8 * 128 ** 3 * 50 / (ms / 1e3) / 1e9,
            "unit": "forward Gvoxel-iter/s through forward + backward",
            "gradients": grads, "gradients_finite": finite}


def _timed_evolutions(ws, pairs, p, iters, steps, batched):
    """Device time of `steps` evolutions of `iters` iterations (each from the
    same start, restored before the call) and the per-kernel times."""
    import torch

    starts = [phi.clone() for _, phi in pairs]

    def one():
        for (_, phi), s in zip(pairs, starts):
            phi.copy_(s)
        if batched:
            ws.evolve_batched(pairs, p, iters)
        else:
            for im, phi in pairs:
                ws.evolve(im, phi, p, iters)

    ws.set_kernel_timing(True)
    ws.kernel_times(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms = 0.0
    for _ in range(steps):
        one()
        torch.cuda.synchronize()
        e0.record()
        if batched:
            ws.evolve_batched(pairs, p, iters)
        else:
            for im, phi in pairs:
                ws.evolve(im, phi, p, iters)
        e1.record()
        torch.cuda.synchronize()
        ms += e0.elapsed_time(e1)
    kt = ws.kernel_times(reset=True)
    ws.set_kernel_timing(False)
    ws.check()
    del starts
    return ms / steps, kt


def _kernel_summary(kt, alg):
    out = {}
    tot = sum(v[0] for v in kt.values())
    for name, (kms, nl) in kt.items():
        if nl:
            per = kms / nl
            out[name] = {"ms_per_launch": per, "share": kms / max(tot, 1e-9),
                         "gbs": alg[name] / (per / 1e3) / 1e9}
    return out


def config1_sample(dev, peak):
    """One 512^3 uint8 volume (200 tubes, radius U[1.5, 8]), sigma 3 and 5,
    200 iterations through rsf_evolve (the single-volume path): value, the
    per-kernel times and the step's HBM fraction."""
    import torch

    from rsf_gb300 import Params, Workspace, gaussian_taps, synth

    img, phi0, _ = synth.make_volume_torch(synth.CONFIG1, dev)
    n = img.numel()
    out = {"workload": "config1: one 512^3 uint8 volume (200 tubes, radius U[1.5,8]), lambda 1, mu 1, "
                       "nu 0.001*255^2, eps 1, dt 0.1, 200 iterations, rsf_evolve", "unit": UNIT}
    ws = Workspace(n)
    for sigma in (3.0, 5.0):
        p = Params(**dict(PARAMS, sigma=sigma))
        k = len(gaussian_taps(sigma))
        phi = phi0.clone()
        pairs = [(img, phi)]
        ws.evolve(img, phi, p, 10)  # warm-up
        phi.copy_(phi0)
        ms, kt = _timed_evolutions(ws, pairs, p, 200, 1, batched=False)
        alg = algorithmic_bytes_shapes([tuple(img.shape)], k)
        value = n * 200 / (ms / 1e3) / 1e9
        out[f"sigma{int(sigma)}"] = {
            "taps": k, "value": value, "ms_per_iteration": ms / 200,
            "step_alg_bytes_per_voxel_iter": sum(alg.values()) / n,
            "step_hbm_frac": sum(alg.values()) * 200 / (ms / 1e3) / 1e9 / peak,
            "kernels": _kernel_summary(kt, alg)}
        del phi, pairs
    ws.close()
    del img, phi0
    torch.cuda.empty_cache()
    return out


def gigavoxel_sample(dev, peak):
    """The gigavoxel batch: the 1024^3 volume (2000 tubes, radius U[1, 10]) in
    27 tiles of 384/384/256 cores + 32-voxel halos (1.53 G tile voxels, all
    resident in HBM), sigma 4, 200 iterations, batched and one at a time."""
    import torch

    from rsf_gb300 import Params, Workspace, gaussian_taps, synth, tiling

    img_full, phi_full, _ = synth.make_volume_torch(synth.CONFIG3, dev)
    tiles = tiling.config3_tiles()
    imgs = [img_full[t.slices()].contiguous() for t in tiles]
    phis = [phi_full[t.slices()].contiguous() for t in tiles]
    del img_full, phi_full
    torch.cuda.empty_cache()
    total = sum(t.voxels for t in tiles)
    p = Params(**dict(PARAMS, sigma=4.0))
    k = len(gaussian_taps(4.0))
    ws = Workspace(total, len(tiles))
    pairs = list(zip(imgs, phis))
    ws.evolve_batched(pairs, p, 4)  # warm-up
    ms, kt = _timed_evolutions(ws, pairs, p, 200, 2, batched=True)
    plain_ms, _ = _timed_evolutions(ws, pairs, p, 200, 1, batched=False)
    alg = algorithmic_bytes(tiles, k)
    value = total * 200 / (ms / 1e3) / 1e9
    ws.close()
    del pairs, imgs, phis
    torch.cuda.empty_cache()
    return {"workload": "config3: 27 sub-volumes (384/384/256 cores + 32-voxel halos, extents 288-448) of a 1024^3 "
                        "synthetic vessel volume (2000 tubes, radius U[1,10]); sigma 4 (29 taps), 200 iterations",
            "voxels": total, "unit": UNIT, "value": value, "ms_per_step": ms, "steps": 2,
            "plain": total * 200 / (plain_ms / 1e3) / 1e9, "batched_vs_plain": plain_ms / ms,
            "step_hbm_frac": sum(alg.values()) * 200 / (ms / 1e3) / 1e9 / peak,
            "kernels": _kernel_summary(kt, alg)}


def run_ours(args):
    import torch
    import torch.distributed as dist

    from rsf_gb300 import Params, Workspace, copy_async, synth, tiling
    from rsf_gb300.dist import max_over_ranks

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    # ---- inputs resident in HBM --------------------------------------
    base = getattr(synth, SPEC)
    spec = synth.VolumeSpec(base.shape, base.n_tubes, base.r_min, base.r_max, base.seed + rank)
    img_full, phi_full, _ = synth.make_volume_torch(spec, dev)
    tiles = getattr(tiling, TILES)()
    imgs = [img_full[t.slices()].contiguous() for t in tiles]
    phi0s = [phi_full[t.slices()].contiguous() for t in tiles]
    del img_full, phi_full
    torch.cuda.empty_cache()
    work = [p.clone() for p in phi0s]
    total_vox = sum(t.voxels for t in tiles)
    p = Params(**PARAMS)
    from rsf_gb300 import gaussian_taps

    k = len(gaussian_taps(SIGMA))
    ws = Workspace(total_vox, len(tiles))
    pairs = list(zip(imgs, work))
    # kernel launch shapes measured on this batch, before the timed region
    from rsf_gb300 import autotune

    shape = autotune.tune_launch_shape(ws, pairs, p, iters=3)

    def step():
        for w, p0 in zip(work, phi0s):
            w.copy_(p0)
        ws.evolve_batched(pairs, p, ITERS)

    for _ in range(args.warmup):
        step()
    ws.check()
    torch.cuda.synchronize()

    # ---- timed region ------------------------------------------------
    ws.set_kernel_timing(True)
    ws.kernel_times(reset=True)
    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    kt = ws.kernel_times(reset=True)
    ws.set_kernel_timing(False)
    ws.check()
    ms = max_over_ranks(ms, dev)
    if world > 1:
        dist.barrier()
    vox_iters = total_vox * ITERS * args.steps * world
    value = vox_iters / (ms / 1e3) / 1e9

    # ---- plain per-volume path (one sub-volume at a time, no graph) ----
    batched_out = [w.clone() for w in work]
    for w, p0 in zip(work, phi0s):
        w.copy_(p0)
    torch.cuda.synchronize()
    e0.record()
    for (im, w) in pairs:
        ws.evolve(im, w, p, ITERS)
    e1.record()
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1)
    plain_value = total_vox * ITERS / (plain_ms / 1e3) / 1e9
    batched_equals_plain = all(torch.equal(a, b) for a, b in zip(batched_out, work))
    del batched_out

    # ---- end to end: pinned host buffers -> evolve -> host ------------
    # All tiles of a step live in one flat buffer per quantity (host and
    # device), so each direction is one copy; the tiles are views into it.
    # The copies run on the SMs (rsf_copy_async): on GB300 the copy engine's
    # host-to-device rate drops to 53-69 GB/s once kernels have run, SM
    # loads from pinned memory keep about 210 GB/s.
    offs = [0]
    for t in tiles:
        offs.append(offs[-1] + t.voxels)
    h_img = torch.empty(total_vox, dtype=torch.uint8, pin_memory=True)
    h_phi = torch.empty(total_vox, dtype=torch.float32, pin_memory=True)
    h_out = torch.empty(total_vox, dtype=torch.float32, pin_memory=True)
    for i, (im, p0) in enumerate(zip(imgs, phi0s)):
        h_img[offs[i]:offs[i + 1]].copy_(im.reshape(-1))
        h_phi[offs[i]:offs[i + 1]].copy_(p0.reshape(-1))
    h2d_bytes = h_img.numel() + 4 * h_phi.numel()
    d2h_bytes = 4 * h_out.numel()

    def device_set():
        di = torch.empty(total_vox, dtype=torch.uint8, device=dev)
        dp = torch.empty(total_vox, dtype=torch.float32, device=dev)
        views = [(di[offs[i]:offs[i + 1]].view(t.shape), dp[offs[i]:offs[i + 1]].view(t.shape))
                 for i, t in enumerate(tiles)]
        return di, dp, views

    del work, pairs, phi0s, imgs
    torch.cuda.empty_cache()
    sets = [device_set(), device_set()]

    def e2e_step():
        di, dp, views = sets[0]
        copy_async(di, h_img)
        copy_async(dp, h_phi)
        ws.evolve_batched(views, p, ITERS)
        copy_async(h_out, dp)
        torch.cuda.synchronize()

    e2e_step()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(max(1, args.steps // 2)):
        e2e_step()
    e2e_s = (time.perf_counter() - t0) / max(1, args.steps // 2)
    e2e_s = max_over_ranks(e2e_s, dev)
    e2e_serial_value = total_vox * ITERS * world / e2e_s / 1e9

    # Pipelined: step i+1's inputs go up and step i's level sets come down
    # on a second stream while the evolution runs, through two sets of
    # device buffers; every step's copies stay inside the timed region.
    cs = torch.cuda.Stream(device=dev)
    st = torch.cuda.current_stream(dev)
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_done = [torch.cuda.Event() for _ in range(2)]

    def h2d(b):
        copy_async(sets[b][0], h_img, stream=cs)
        copy_async(sets[b][1], h_phi, stream=cs)
        ev_in[b].record(cs)

    def d2h(b):
        cs.wait_event(ev_done[b])
        copy_async(h_out, sets[b][1], stream=cs)

    def pipeline(n):
        h2d(0)
        if n > 1:
            h2d(1)
        for i in range(n):
            b = i % 2
            st.wait_event(ev_in[b])
            ws.evolve_batched(sets[b][2], p, ITERS, stream=st)
            ev_done[b].record(st)
            d2h(b)
            if i + 2 < n:
                h2d(b)  # after this set's download on the copy stream
        torch.cuda.synchronize()

    pipeline(2)
    n_pipe = max(2, args.steps)
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    pipeline(n_pipe)
    pipe_s = (time.perf_counter() - t0) / n_pipe
    pipe_s = max_over_ranks(pipe_s, dev)
    e2e_value = total_vox * ITERS * world / pipe_s / 1e9

    # ---- roofline of the dominant kernel ------------------------------
    alg = algorithmic_bytes(tiles, k)
    peak, peak_kind = measured_peaks()
    kernels = {}
    for name, (kms, nl) in kt.items():
        if nl == 0:
            continue
        per = kms / nl
        kernels[name] = {"launches": int(nl), "ms_per_launch": per, "share": kms / max(1e-9, sum(v[0] for v in kt.values())),
                         "alg_bytes_per_launch": alg[name], "gbs": alg[name] / (per / 1e3) / 1e9}
    dom = max(kernels, key=lambda n: kernels[n]["ms_per_launch"] * kernels[n]["launches"])
    dk = kernels[dom]
    tr = ncu_traffic_ratio(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": dk["gbs"], "peak": peak, "unit": "GB/s",
                "frac": dk["gbs"] / peak, "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                "traffic": (tr * alg[dom] if tr is not None else None),
                "traffic_source": "ncu DRAM/algorithmic ratio of the same kernel on a 320^3 case "
                                  "(profiles/traffic.json) times this launch's algorithmic bytes",
                "step_alg_bytes_per_voxel_iter": sum(alg.values()) / total_vox,
                "step_gbs": sum(alg.values()) * ITERS * args.steps / (ms / 1e3) / 1e9}
    launches = sum(v[1] for v in kt.values())
    # The stencil, x-pass and z-pass are bound by instruction issue, not HBM:
    # their issue-side roofline is warp instructions per second (the ncu
    # count per voxel times this launch's voxels over its live time) against
    # the SMs x 4 schedulers x one warp instruction per cycle at the SM clock.
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    ipv = ncu_warp_inst_per_voxel(dom)
    if ipv is not None:
        issue_peak = n_sm * 4 * sm_mhz * 1e6
        achieved = ipv * total_vox / (dk["ms_per_launch"] / 1e3)
        roofline["issue"] = {"warp_inst_per_voxel": ipv, "achieved_warp_inst_per_s": achieved,
                             "peak_warp_inst_per_s": issue_peak, "frac": achieved / issue_peak,
                             "source": "ncu smsp__inst_executed.sum per voxel on the 320^3 case (profiles/traffic.json)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "subvolumes": len(tiles), "voxels": total_vox, "iterations": ITERS,
                       "sigma": SIGMA, "taps": k,
                       "launch_shape": {"xpass_width": shape.xpass_width, "stencil_planes": shape.stencil_planes,
                                        "z_tma": shape.z_tma, "tuned_ms_per_iteration": {
                                            f"{a}/{b}/{z}": round(ms, 3) for (a, b, z), ms in shape.table}},
                       "step": f"one {ITERS}-iteration evolution of all {len(tiles)} sub-volumes",
                       "l2": f"inputs larger than L2 (phi {total_vox * 4 / 1e9:.1f} GB, y-pass fields "
                             f"{total_vox * 16 / 1e9:.0f} GB per iteration)",
                       "parallelism": f"dp{world}"},
            "plain": {"value": plain_value, "unit": UNIT,
                      "how": "same sub-volumes evolved one at a time (rsf_evolve, no graph)"},
            "batched_vs_plain": value / world / plain_value,
            "batched_equals_plain": batched_equals_plain,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes,
                    "how": f"rsf_evolve_batched over {n_pipe} steps from pinned host buffers; each step's inputs "
                           "copied up and results copied down on a second stream, overlapping the neighbouring "
                           "steps' evolution (two device buffer sets)",
                    "serial": {"value": e2e_serial_value,
                               "how": "copy in, evolve, copy out, synchronise, one step at a time"}},
            "gpu_launches": int(launches),
            "roofline": roofline,
            "kernels": kernels,
            "clocks": clk,
        }
        # FP32 work of the separable 4-field schedule: 4 fields x 3 axes x k
        # FMAs (2 flops each) plus ~120 pointwise flops per voxel-iteration,
        # against the non-tensor FP32 rate of the SMs x 128 lanes x 2 flops at
        # the SM clock seen during the timed region (a nominal figure).
        f_alg = 24 * k + 120
        fp32_peak = n_sm * 128 * 2 * sm_mhz * 1e6 / 1e12
        line["fp32"] = {"flops_per_voxel_iter": f_alg, "achieved_tflops": value * f_alg / 1e3,
                        "nominal_peak_tflops": fp32_peak, "frac": value * f_alg / 1e3 / world / fp32_peak}
        if world == 1:
            # the other workloads, after the headline's buffers are released
            ws.close()
            del sets, h_img, h_phi, h_out
            torch.cuda.empty_cache()
            base, sample = cpu_sample(os.cpu_count() or 1)
            line["cpu_baseline"] = base
            line["parity"] = parity_on_sample(sample)
            if not args.headline_only:
                line["config1"] = config1_sample(dev, peak)
                if args.workload == "config2":
                    line["gigavoxel"] = gigavoxel_sample(dev, peak)
                line["differentiable"] = differentiable_sample(dev)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the 512^3, gigavoxel and differentiable records after the headline")
    ap.add_argument("--workload", choices=["config2", "gigavoxel"], default="config2",
                    help="config2 (default, the 48-sub-volume batch) or gigavoxel (1024^3 in 27 tiles)")
    args = ap.parse_args()
    if args.workload == "gigavoxel":
        g = globals()
        g.update(GIGAVOXEL)
        g["PARAMS"] = dict(PARAMS, sigma=g["SIGMA"])
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
