"""Autotuners: tile shapes for whole-volume evolution (`tune_cores`) and
kernel launch shapes for a batch (`tune_launch_shape`).

The batch driver evolves a volume as a grid of cores grown by a halo.  The
halo is fixed by correctness (it bounds how far missing context reaches a
core: r + 2 voxels per iteration); the core size is a performance choice:
small cores waste work on halos (evolved voxels / owned voxels grows), large
cores make few, long sub-volumes whose last wave of blocks leaves SMs idle.
`tune_cores` measures candidate core sizes on the device with the real
kernels (a short batched evolution of every tile of each candidate plan, on
synthetic data of the volume's shape) and returns the one that owns the most
voxels per second.  Results are cached per (shape, sigma, halo, dtype) for
the life of the process.

The reference has no counterpart: its tiling is fixed by hand in the
missing disassemble.py (README.md:6).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Callable, Dict, List, Optional, Sequence, Tuple

from .api import Params, Workspace
from .tiling import Tile, plan

_CACHE: Dict[tuple, "TuneResult"] = {}

DEFAULT_CANDIDATES = (128, 192, 256, 320, 384, 512)


@dataclass
class TuneResult:
    cores: int
    owned_voxels_per_s: float
    table: List[Tuple[int, float, int, int]]  # (core, owned voxels/s, tiles, evolved voxels)


def candidate_plans(shape: Sequence[int], halo: int, candidates: Sequence[int] = DEFAULT_CANDIDATES):
    """(core, tiles) for each candidate that gives a distinct plan and whose
    tiles are at least 2 voxels per axis."""
    out, seen = [], set()
    for c in candidates:
        c = min(int(c), max(shape))
        tiles = plan(tuple(shape), c, halo)
        key = tuple((t.lo, t.hi) for t in tiles)
        if key in seen or any(min(t.shape) < 2 for t in tiles):
            continue
        seen.add(key)
        out.append((c, tiles))
    return out


def pick(shape: Sequence[int], measurements: Sequence[Tuple[int, Sequence[Tile], float]]) -> TuneResult:
    """Chooses among (core, tiles, seconds per iteration) by owned voxels per second."""
    owned = 1
    for s in shape:
        owned *= int(s)
    table = []
    for c, tiles, sec in measurements:
        table.append((c, owned / sec, len(tiles), sum(t.voxels for t in tiles)))
    best = max(table, key=lambda r: r[1])
    return TuneResult(best[0], best[1], table)


def smooth_phi(shape: Sequence[int], device="cpu"):
    """A smooth level set in [-3, 3], float32 (L, H, W): a product of sines
    whose sign changes every 8 to 14 voxels along each axis.  The timing runs
    evolve it rather than noise, so that they stay finite for any parameters."""
    import torch

    z, y, x = (torch.arange(int(n), device=device, dtype=torch.float32) for n in shape)
    return (3.0 * torch.sin(0.37 * x)[None, None, :] * torch.sin(0.29 * y + 1.0)[None, :, None]
            * torch.sin(0.23 * z + 2.0)[:, None, None]).contiguous()


def _time_plan(tiles: Sequence[Tile], params: Params, dtype, iters: int, device) -> float:
    import torch

    total = sum(t.voxels for t in tiles)
    gen = torch.Generator(device=device)
    gen.manual_seed(0)
    pairs = []
    with Workspace(total, len(tiles)) as ws:
        for t in tiles:
            img = (torch.randint(0, 256, t.shape, generator=gen, device=device, dtype=torch.uint8)
                   if dtype == "u8" else torch.rand(t.shape, generator=gen, device=device))
            pairs.append((img, smooth_phi(t.shape, device)))
        ws.evolve_batched(pairs, params, 1)  # warm-up (graph capture, table upload)
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ws.evolve_batched(pairs, params, iters)
        e1.record()
        torch.cuda.synchronize(device)
        ws.check()
    return e0.elapsed_time(e1) / 1e3 / iters


def tune_cores(shape: Sequence[int], params: Params, halo: int = 32, dtype: str = "u8", iters: int = 4,
               candidates: Sequence[int] = DEFAULT_CANDIDATES, device="cuda:0",
               timer: Optional[Callable[[Sequence[Tile]], float]] = None) -> TuneResult:
    """Core size with the highest owned-voxel throughput for `shape`.
    `timer(tiles) -> seconds per iteration` replaces the device measurement
    (for tests); results with the device timer are cached."""
    key = (tuple(int(s) for s in shape), float(params.sigma), int(halo), dtype, tuple(candidates))
    if timer is None and key in _CACHE:
        return _CACHE[key]
    meas = []
    for c, tiles in candidate_plans(shape, halo, candidates):
        sec = timer(tiles) if timer is not None else _time_plan(tiles, params, dtype, iters, device)
        meas.append((c, tiles, sec))
    if not meas:
        raise ValueError("no candidate core size fits the volume")
    res = pick(shape, meas)
    if timer is None:
        _CACHE[key] = res
    return res


# ---------------------------------------------------------------------------
# Kernel launch shapes.  The kernels take three shape choices per launch: the
# x-pass lane width (5 or 9 outputs per lane: which wastes fewer outputs past
# the valid width depends on the batch's row lengths), the stencil's planes
# per block (128 or 64, or 32 for batches too small to fill the GPU several
# times)
# and, for 21 and 35 taps, whether the z-pass takes its planes through TMA.
# The workspace picks them by heuristics; `tune_launch_shape` times every
# combination on the caller's batch and keeps the fastest.
# ---------------------------------------------------------------------------
LAUNCH_CANDIDATES = tuple((xb, zc, zt) for xb in (5, 9) for zc in (128, 64, 32) for zt in (0, 1))


@dataclass
class LaunchShape:
    xpass_width: int
    stencil_planes: int
    z_tma: int
    ms_per_iteration: float
    table: List[Tuple[Tuple[int, int, int], float]]


def pick_launch_shape(measurements: Sequence[Tuple[Tuple[int, int, int], float]]) -> LaunchShape:
    """The fastest of (shape, ms per iteration); ties keep the first."""
    best = min(measurements, key=lambda m: m[1])
    (xb, zc, zt), ms = best
    return LaunchShape(xb, zc, zt, ms, list(measurements))


def tune_launch_shape(ws: Workspace, pairs, params: Params, iters: int = 4,
                      candidates: Sequence[Tuple[int, int, int]] = LAUNCH_CANDIDATES,
                      timer: Optional[Callable[[Tuple[int, int, int]], float]] = None) -> LaunchShape:
    """Times `iters` batched iterations of `pairs` (image, phi) for every
    launch shape, restoring each phi between the runs, sets the fastest on
    `ws` and returns it.  `timer(shape) -> ms per iteration` replaces the
    device measurement (for tests)."""
    meas = []
    if timer is not None:
        for shape in candidates:
            meas.append((tuple(shape), float(timer(tuple(shape)))))
    else:
        import torch

        starts = [phi.clone() for _, phi in pairs]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for shape in candidates:
            ws.set_launch_shape(*shape)
            ws.evolve_batched(pairs, params, 1)  # graph capture and table upload
            for (_, phi), s0 in zip(pairs, starts):
                phi.copy_(s0)
            torch.cuda.synchronize()
            e0.record()
            ws.evolve_batched(pairs, params, iters)
            e1.record()
            torch.cuda.synchronize()
            meas.append((tuple(shape), e0.elapsed_time(e1) / iters))
            for (_, phi), s0 in zip(pairs, starts):
                phi.copy_(s0)
        ws.check()
    best = pick_launch_shape(meas)
    ws.set_launch_shape(best.xpass_width, best.stencil_planes, best.z_tma)
    return best
