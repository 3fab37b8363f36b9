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


def reassemble_cores(shape, tiles: Sequence[Tile], parts, dtype=np.float32) -> np.ndarray:
    """Writes every tile's core region into a full volume (core crop)."""
    out = np.empty(shape, dtype=dtype)
    for t, p in zip(tiles, parts):
        out[t.core_slices()] = np.asarray(p)[t.core_in_tile()]
    return out


def blend_halves(a: np.ndarray, b: np.ndarray, overlap: int, axis: int = 1) -> np.ndarray:
    """Linear blend of two volumes that overlap by `overlap` voxels along
    `axis`: the weight of `b` rises from 0 to 1 across the overlap (the
    behaviour of interpolating_volumes.py:10-40, which blends along axis 1)."""
    if overlap < 1:
        return np.concatenate([a, b], axis=axis)
    w = np.linspace(0.0, 1.0, overlap)
    shape = [1] * a.ndim
    shape[axis] = overlap
    w = w.reshape(shape)
    a_keep = np.take(a, range(a.shape[axis] - overlap), axis=axis)
    b_keep = np.take(b, range(overlap, b.shape[axis]), axis=axis)
    a_ov = np.take(a, range(a.shape[axis] - overlap, a.shape[axis]), axis=axis)
    b_ov = np.take(b, range(overlap), axis=axis)
    mid = (1.0 - w) * a_ov + w * b_ov
    return np.concatenate([a_keep, mid, b_keep], axis=axis)
