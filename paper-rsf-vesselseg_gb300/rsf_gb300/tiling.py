"""Overlapping sub-volume tiling and reassembly.

The reference's pipeline cuts a large 8-bit stack into overlapping NumPy
sub-volumes (`disassemble.py`, README.md:6), evolves each one independently
(one `rsf3d` process each, README.md:56) and stitches the level sets back
(`reassemble.py`, README.md:9); none of those scripts ships with it.  The
only stitching code present, interpolating_volumes.py:10-40, blends two
halves linearly across their overlap along one axis.

Here a tile is a core box (the voxels it owns in the output) grown by a halo
on every side and clipped at the volume faces.  A halo wider than the blur
radius plus the 2-voxel stencil reach makes one iteration of a tile's core
independent of its neighbours; longer evolutions let information travel
(r + 2) voxels per iteration, so the halo bounds how far a tile's core can be
influenced by the missing context.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence, Tuple

import numpy as np


@dataclass(frozen=True)
class Tile:
    """Extent [lo, hi) per axis (z, y, x) and the core [clo, chi) it owns."""
    lo: Tuple[int, int, int]
    hi: Tuple[int, int, int]
    clo: Tuple[int, int, int]
    chi: Tuple[int, int, int]

    @property
    def shape(self):
        return tuple(h - l for l, h in zip(self.lo, self.hi))

    @property
    def voxels(self) -> int:
        s = self.shape
        return s[0] * s[1] * s[2]

    def slices(self):
        return tuple(slice(l, h) for l, h in zip(self.lo, self.hi))

    def core_slices(self):
        return tuple(slice(l, h) for l, h in zip(self.clo, self.chi))

    def core_in_tile(self):
        return tuple(slice(cl - l, ch - l) for l, cl, ch in zip(self.lo, self.clo, self.chi))


def _axis_bounds(n: int, cores) -> List[int]:
    """Core boundaries along one axis: an int core size or explicit bounds."""
    if isinstance(cores, int):
        b = list(range(0, n, cores)) + [n]
    else:
        b = list(cores)
    if b[0] != 0 or b[-1] != n or any(b[i] >= b[i + 1] for i in range(len(b) - 1)):
        raise ValueError(f"core bounds {b} do not partition [0, {n})")
    return b


def plan(shape: Sequence[int], cores, halo: int) -> List[Tile]:
    """Tiles covering `shape` (z, y, x).  `cores` is one entry per axis, each
    a core size or an explicit list of core boundaries."""
    if isinstance(cores, int):
        cores = (cores, cores, cores)
    bounds = [_axis_bounds(n, c) for n, c in zip(shape, cores)]
    tiles = []
    for z0, z1 in zip(bounds[0][:-1], bounds[0][1:]):
        for y0, y1 in zip(bounds[1][:-1], bounds[1][1:]):
            for x0, x1 in zip(bounds[2][:-1], bounds[2][1:]):
                clo, chi = (z0, y0, x0), (z1, y1, x1)
                lo = tuple(max(0, c - halo) for c in clo)
                hi = tuple(min(n, c + halo) for c, n in zip(chi, shape))
                tiles.append(Tile(lo, hi, clo, chi))
    return tiles


def config2_tiles() -> List[Tile]:
    """48 uneven tiles of a 512 x 1024 x 1024 (z, y, x) volume: 256-voxel cores
    in x and y, z cores [0,32) [32,288) [288,512), 32-voxel halos clipped at
    the faces (extents 288/320/320/288 in x and y, 64/320/256 in z)."""
    return plan((512, 1024, 1024), ([0, 32, 288, 512], 256, 256), 32)


def config3_tiles() -> List[Tile]:
    """27 tiles of a 1024^3 volume: cores 384/384/256 per axis, 32 halo."""
    b = [0, 384, 768, 1024]
    return plan((1024, 1024, 1024), (b, b, b), 32)


def lpt_shards(tiles: Sequence[Tile], n: int) -> List[List[int]]:
    """Longest-processing-time assignment of tile indices to n workers by
    voxel count (no data moves between workers during evolution)."""
    order = sorted(range(len(tiles)), key=lambda i: -tiles[i].voxels)
    loads = [0] * n
    out: List[List[int]] = [[] for _ in range(n)]
    for i in order:
        w = min(range(n), key=lambda j: loads[j])
        out[w].append(i)
        loads[w] += tiles[i].voxels
    return [sorted(s) for s in out]


def cut(volume: np.ndarray, tiles: Sequence[Tile]):
    """Copies of every tile's extent (C-contiguous)."""
    return [np.ascontiguousarray(volume[t.slices()]) for t in tiles]


def grid_bounds(tiles: Sequence[Tile]):
    """Core boundaries per axis (z, y, x) of a tile grid as `plan` makes it,
    checking that the tiles are listed z-major, then y, then x."""
    bounds = [sorted({t.clo[a] for t in tiles} | {t.chi[a] for t in tiles}) for a in range(3)]
    n = [len(b) - 1 for b in bounds]
    if n[0] * n[1] * n[2] != len(tiles):
        raise ValueError("tiles do not form a grid")
    for i, t in enumerate(tiles):
        iz, iy, ix = i // (n[1] * n[2]), (i // n[2]) % n[1], i % n[2]
        if (t.clo, t.chi) != ((bounds[0][iz], bounds[1][iy], bounds[2][ix]),
                              (bounds[0][iz + 1], bounds[1][iy + 1], bounds[2][ix + 1])):
            raise ValueError("tiles are not in grid order (z-major, then y, then x)")
    return bounds


def reassemble_device(ws, tiles: Sequence[Tile], parts, shape, mode: str = "core", out=None, stream=None):
    """Stitches evolved tiles (CUDA float32 tensors, one per tile, in `plan`
    order) into `out` (CUDA float32, `shape` = (L, H, W)) on the device with
    rsf_reassemble: "core" copies each tile's core, "blend" blends linearly
    across the overlaps (interpolating_volumes.py:10-40 generalised to a grid)."""
    import ctypes

    import torch

    from . import _lib
    from .api import _stream_ptr

    bz, by, bx = grid_bounds(tiles)
    if out is None:
        out = torch.empty(tuple(shape), dtype=torch.float32, device=parts[0].device)
    arr = (_lib.RsfTile * len(tiles))()
    for i, (t, p) in enumerate(zip(tiles, parts)):
        if tuple(p.shape) != t.shape or p.dtype != torch.float32 or not p.is_cuda or not p.is_contiguous():
            raise TypeError(f"part {i} must be a contiguous CUDA float32 tensor of shape {t.shape}")
        arr[i] = _lib.RsfTile(p.data_ptr(), t.lo[2], t.lo[1], t.lo[0], t.shape[2], t.shape[1], t.shape[0])
    cx = (ctypes.c_int64 * len(bx))(*bx)
    cy = (ctypes.c_int64 * len(by))(*by)
    cz = (ctypes.c_int64 * len(bz))(*bz)
    L, H, W = shape
    _lib.check(ws._lib.rsf_reassemble(ws.handle, arr, len(bx) - 1, len(by) - 1, len(bz) - 1, cx, cy, cz,
                                      {"core": 0, "blend": 1}[mode], ctypes.c_void_p(out.data_ptr()), W, H, L,
                                      ctypes.c_void_p(_stream_ptr(stream))))
    return out
