"""TEST INFRASTRUCTURE ONLY: host restatements of the reassembly step, the
checkers of rsf_reassemble (tests/ call them; no product path does).

interpolating_volumes.py:10-40 of the reference blends two volumes that
overlap along axis 1: the first keeps weight 1 - a, the second a, with
a = linspace(0, 1, overlap).  `blend_halves` restates it for any axis;
`blend_grid` applies the same ramps per axis to a grid of tiles, multiplies
them and normalises, which is the definition the device blend implements;
`reassemble_cores` is the core-crop stitch.
"""
from __future__ import annotations

import numpy as np


def reassemble_cores(shape, tiles, parts, dtype=np.float32) -> np.ndarray:
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


def blend_grid(shape, tiles, parts) -> np.ndarray:
    """Host restatement of the "blend" reassembly (float64): per axis a
    tile's weight rises as linspace(0, 1, overlap) across its overlap with the
    previous tile and falls as 1 - linspace across its overlap with the next;
    weights multiply over the axes and the sum is normalised."""
    from rsf_gb300.tiling import grid_bounds

    bounds = grid_bounds(tiles)
    n = [len(b) - 1 for b in bounds]
    ext = []  # per axis: list of (lo, hi) per cell
    for a in range(3):
        seen = {}
        for i, t in enumerate(tiles):
            idx = (i // (n[1] * n[2]), (i // n[2]) % n[1], i % n[2])[a]
            seen[idx] = (t.lo[a], t.hi[a])
        ext.append([seen[j] for j in range(n[a])])

    def ramp(a, j):
        lo, hi = ext[a][j]
        w = np.ones(hi - lo)
        if j > 0 and ext[a][j - 1][1] > lo:
            ov = ext[a][j - 1][1] - lo
            w[:ov] *= np.linspace(0.0, 1.0, ov)
        if j + 1 < n[a] and ext[a][j + 1][0] < hi:
            ov = hi - ext[a][j + 1][0]
            w[hi - lo - ov:] *= 1.0 - np.linspace(0.0, 1.0, ov)
        return w

    acc = np.zeros(shape)
    wsum = np.zeros(shape)
    for i, (t, p) in enumerate(zip(tiles, parts)):
        iz, iy, ix = i // (n[1] * n[2]), (i // n[2]) % n[1], i % n[2]
        w = ramp(0, iz)[:, None, None] * ramp(1, iy)[None, :, None] * ramp(2, ix)[None, None, :]
        acc[t.slices()] += w * np.asarray(p, dtype=np.float64)
        wsum[t.slices()] += w
    return acc / wsum
