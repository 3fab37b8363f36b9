"""Seeded synthetic microvascular volumes and initial level sets.

The reference evolves sub-volumes of KESM / LSFM / micro-CT stacks that are not
distributed with it (README.md:14-15).  This module produces stand-ins with the
same shape, dtype and value ranges:

* tubes: cubic Catmull-Rom splines through 4-6 uniformly drawn control points,
  constant radius per tube; the vessel mask is "distance to centreline <= r";
* intensities: vessel N(180, 20), background N(40, 15), multiplied by a smooth
  bias field 1 + 0.3 sin(2pi(x/Lx+ax)) sin(2pi(y/Ly+ay)) sin(2pi(z/Lz+az)),
  plus additive N(0, 10) noise, clipped to [0, 255] and rounded to uint8;
* phi0: the true mask perturbed by one binary dilation or erosion (radius 1-2)
  per connected region, turned into an exact signed Euclidean distance
  (positive inside) and clipped to [-3, 3], float32.

Arrays use NumPy C order (Z, Y, X): x is the fastest axis, matching the
reference's linear index z*W*H + y*W + x (CUDA_RSF/kernel.cu:73).
All randomness comes from numpy.random.default_rng(seed) (PCG64).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class VolumeSpec:
    shape: tuple  # (Z, Y, X)
    n_tubes: int
    r_min: float
    r_max: float
    seed: int


# Workloads quoted by the benchmark configurations.
CONFIG0 = VolumeSpec((128, 128, 128), 12, 2.0, 6.0, 0)
CONFIG1 = VolumeSpec((512, 512, 512), 200, 1.5, 8.0, 1)


def _catmull_rom(points: np.ndarray, step: float = 0.5) -> np.ndarray:
    """Samples a uniform Catmull-Rom spline through every control point.

    The end tangents come from reflected phantom points, so the curve starts at
    the first control point and ends at the last.  Consecutive samples are at
    most `step` voxels apart (chord-length bound)."""
    p = np.concatenate([2 * points[:1] - points[1:2], points, 2 * points[-1:] - points[-2:-1]])
    out = []
    for i in range(1, len(p) - 2):
        p0, p1, p2, p3 = p[i - 1], p[i], p[i + 1], p[i + 2]
        # Upper bound of the segment length by its control polygon.
        poly = np.linalg.norm(p2 - p1) + 0.5 * (np.linalg.norm(p2 - p0) + np.linalg.norm(p3 - p1))
        n = max(2, int(math.ceil(poly / step)) + 1)
        t = np.linspace(0.0, 1.0, n, endpoint=(i == len(p) - 3))[:, None]
        t2, t3 = t * t, t * t * t
        seg = 0.5 * ((2 * p1) + (-p0 + p2) * t + (2 * p0 - 5 * p1 + 4 * p2 - p3) * t2
                     + (-p0 + 3 * p1 - 3 * p2 + p3) * t3)
        out.append(seg)
    return np.concatenate(out)


def _stamp_tube(mask: np.ndarray, samples: np.ndarray, radius: float) -> None:
    """Sets every voxel centre within `radius` of any sample point."""
    Z, Y, X = mask.shape
    rc = int(math.ceil(radius)) + 1
    ax = np.arange(-rc, rc + 1)
    oz, oy, ox = np.meshgrid(ax, ax, ax, indexing="ij")
    offs = np.stack([ox.ravel(), oy.ravel(), oz.ravel()], axis=1)  # (B, 3) as x, y, z
    r2 = radius * radius
    chunk = max(1, 2_000_000 // len(offs))
    for s in range(0, len(samples), chunk):
        pts = samples[s:s + chunk]  # (S, 3) x, y, z
        base = np.floor(pts).astype(np.int64)
        vox = base[:, None, :] + offs[None, :, :]  # (S, B, 3)
        d = vox - pts[:, None, :]
        hit = (d * d).sum(-1) <= r2
        hit &= (vox[..., 0] >= 0) & (vox[..., 0] < X) & (vox[..., 1] >= 0) & (vox[..., 1] < Y)
        hit &= (vox[..., 2] >= 0) & (vox[..., 2] < Z)
        v = vox[hit]
        mask[v[:, 2], v[:, 1], v[:, 0]] = True


def tube_mask(spec: VolumeSpec, rng: np.random.Generator) -> np.ndarray:
    Z, Y, X = spec.shape
    mask = np.zeros(spec.shape, dtype=bool)
    hi = np.array([X - 1, Y - 1, Z - 1], dtype=np.float64)
    for _ in range(spec.n_tubes):
        n_ctrl = int(rng.integers(4, 7))
        ctrl = rng.uniform(0.0, 1.0, size=(n_ctrl, 3)) * hi
        radius = float(rng.uniform(spec.r_min, spec.r_max))
        _stamp_tube(mask, _catmull_rom(ctrl), radius)
    return mask


def intensity(mask: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    Z, Y, X = mask.shape
    vessel = rng.normal(180.0, 20.0, size=mask.shape)
    back = rng.normal(40.0, 15.0, size=mask.shape)
    img = np.where(mask, vessel, back)
    del vessel, back
    ph = rng.uniform(0.0, 1.0, size=3)
    bz = np.sin(2 * np.pi * (np.arange(Z) / Z + ph[2]))[:, None, None]
    by = np.sin(2 * np.pi * (np.arange(Y) / Y + ph[1]))[None, :, None]
    bx = np.sin(2 * np.pi * (np.arange(X) / X + ph[0]))[None, None, :]
    img *= 1.0 + 0.3 * bz * by * bx
    img += rng.normal(0.0, 10.0, size=mask.shape)
    np.clip(img, 0.0, 255.0, out=img)
    return np.rint(img).astype(np.uint8)


def _ball(r: int) -> np.ndarray:
    ax = np.arange(-r, r + 1)
    z, y, x = np.meshgrid(ax, ax, ax, indexing="ij")
    return (x * x + y * y + z * z) <= r * r


def perturb(mask: np.ndarray, rng: np.random.Generator) -> np.ndarray:
    """One random dilation or erosion (radius 1 or 2) per connected region."""
    from scipy import ndimage

    labels, n = ndimage.label(mask)
    if n == 0:
        return mask.copy()
    op = rng.integers(0, 2, size=n + 1)   # 0 erode, 1 dilate
    rad = rng.integers(1, 3, size=n + 1)  # 1 or 2
    ids = np.arange(n + 1)
    out = np.zeros_like(mask)
    for r in (1, 2):
        b = _ball(r)
        sel_e = np.isin(labels, ids[(ids > 0) & (op == 0) & (rad == r)])
        if sel_e.any():
            out |= ndimage.binary_erosion(mask, structure=b) & sel_e
        sel_d = np.isin(labels, ids[(ids > 0) & (op == 1) & (rad == r)])
        if sel_d.any():
            out |= ndimage.binary_dilation(sel_d, structure=b)
    return out


def signed_distance(mask: np.ndarray, clip: float | None = 3.0) -> np.ndarray:
    """Exact Euclidean signed distance, positive inside, optionally clipped."""
    from scipy import ndimage

    if mask.all() or not mask.any():
        v = (clip if clip is not None else 1e6) * (1.0 if mask.all() else -1.0)
        return np.full(mask.shape, v, dtype=np.float32)
    din = ndimage.distance_transform_edt(mask)
    dout = ndimage.distance_transform_edt(~mask)
    sd = np.where(mask, din, -dout)
    if clip is not None:
        np.clip(sd, -clip, clip, out=sd)
    return sd.astype(np.float32)


def make_volume(spec: VolumeSpec):
    """Returns (I uint8, phi0 float32, true mask bool), all shaped (Z, Y, X)."""
    rng = np.random.default_rng(spec.seed)
    mask = tube_mask(spec, rng)
    img = intensity(mask, rng)
    phi0 = signed_distance(perturb(mask, rng))
    return img, phi0, mask


def make_small(shape=(24, 20, 18), n_tubes=3, r_min=1.5, r_max=3.0, seed=0):
    """A small instance of the same generator for unit tests."""
    return make_volume(VolumeSpec(tuple(shape), n_tubes, r_min, r_max, seed))


# ---------------------------------------------------------------------------
# Device path for gigavoxel volumes.  Same spec; tube geometry comes from the
# same NumPy RNG stream, intensities from a seeded torch generator on the
# device, and the perturbation is one dilation or erosion (radius 1-2) per
# tube rather than per connected region.  The signed distance is exact up to
# the clip: every voxel within `clip` of the opposite label is found by
# checking all integer offsets of length <= clip.
# ---------------------------------------------------------------------------
CONFIG2 = VolumeSpec((512, 1024, 1024), 800, 1.5, 8.0, 2)
CONFIG3 = VolumeSpec((1024, 1024, 1024), 2000, 1.0, 10.0, 3)


def _stamp_tube_torch(mask_flat, shape, samples, radius):
    import torch

    Z, Y, X = shape
    dev = mask_flat.device
    rc = int(math.ceil(radius)) + 1
    ax = torch.arange(-rc, rc + 1, device=dev)
    oz, oy, ox = torch.meshgrid(ax, ax, ax, indexing="ij")
    offs = torch.stack([ox.reshape(-1), oy.reshape(-1), oz.reshape(-1)], dim=1)
    pts_all = torch.as_tensor(samples, dtype=torch.float32, device=dev)
    r2 = float(radius) * float(radius)
    chunk = max(1, 8_000_000 // offs.shape[0])
    for s in range(0, pts_all.shape[0], chunk):
        pts = pts_all[s:s + chunk]
        vox = torch.floor(pts).long()[:, None, :] + offs[None, :, :]
        d = vox.float() - pts[:, None, :]
        hit = (d * d).sum(-1) <= r2
        hit &= (vox[..., 0] >= 0) & (vox[..., 0] < X) & (vox[..., 1] >= 0) & (vox[..., 1] < Y)
        hit &= (vox[..., 2] >= 0) & (vox[..., 2] < Z)
        v = vox[hit]
        mask_flat[(v[:, 2] * Y + v[:, 1]) * X + v[:, 0]] = True


def signed_distance_torch(mask, clip: float = 3.0):
    """Exact Euclidean signed distance (positive inside) clipped to +-clip."""
    import torch

    c = int(math.floor(clip))
    Z, Y, X = mask.shape
    pad = torch.full((Z + 2 * c, Y + 2 * c, X + 2 * c), 2, dtype=torch.int8, device=mask.device)
    pad[c:c + Z, c:c + Y, c:c + X] = mask.to(torch.int8)
    big = float(clip * clip)
    d_in = torch.full(mask.shape, big, dtype=torch.float32, device=mask.device)
    d_out = torch.full(mask.shape, big, dtype=torch.float32, device=mask.device)
    inside = mask
    outside = ~mask
    for dz in range(-c, c + 1):
        for dy in range(-c, c + 1):
            for dx in range(-c, c + 1):
                r2 = dz * dz + dy * dy + dx * dx
                if r2 == 0 or r2 > clip * clip:
                    continue
                nb = pad[c + dz:c + dz + Z, c + dy:c + dy + Y, c + dx:c + dx + X]
                d_in = torch.where(inside & (nb == 0), torch.clamp(d_in, max=float(r2)), d_in)
                d_out = torch.where(outside & (nb == 1), torch.clamp(d_out, max=float(r2)), d_out)
    return torch.where(inside, torch.sqrt(d_in), -torch.sqrt(d_out))


def make_volume_torch(spec: VolumeSpec, device):
    """Returns (I uint8, phi0 float32, true mask bool) as CUDA tensors."""
    import torch

    rng = np.random.default_rng(spec.seed)
    Z, Y, X = spec.shape
    hi = np.array([X - 1, Y - 1, Z - 1], dtype=np.float64)
    true_flat = torch.zeros(Z * Y * X, dtype=torch.bool, device=device)
    pert_flat = torch.zeros(Z * Y * X, dtype=torch.bool, device=device)
    for _ in range(spec.n_tubes):
        n_ctrl = int(rng.integers(4, 7))
        ctrl = rng.uniform(0.0, 1.0, size=(n_ctrl, 3)) * hi
        radius = float(rng.uniform(spec.r_min, spec.r_max))
        delta = float(rng.choice([-2.0, -1.0, 1.0, 2.0]))
        samples = _catmull_rom(ctrl)
        _stamp_tube_torch(true_flat, spec.shape, samples, radius)
        if radius + delta >= 0.5:
            _stamp_tube_torch(pert_flat, spec.shape, samples, radius + delta)
    mask = true_flat.view(Z, Y, X)
    gen = torch.Generator(device=device)
    gen.manual_seed(spec.seed)
    img = torch.empty((Z, Y, X), dtype=torch.float32, device=device)
    for z0 in range(0, Z, 64):  # slabs bound the temporaries
        sl = slice(z0, min(Z, z0 + 64))
        m = mask[sl]
        v = torch.randn(m.shape, generator=gen, device=device) * 20.0 + 180.0
        b = torch.randn(m.shape, generator=gen, device=device) * 15.0 + 40.0
        img[sl] = torch.where(m, v, b)
    ph = rng.uniform(0.0, 1.0, size=3)
    tz = torch.arange(Z, device=device, dtype=torch.float32)
    ty = torch.arange(Y, device=device, dtype=torch.float32)
    tx = torch.arange(X, device=device, dtype=torch.float32)
    bz = torch.sin(2 * math.pi * (tz / Z + float(ph[2])))[:, None, None]
    by = torch.sin(2 * math.pi * (ty / Y + float(ph[1])))[None, :, None]
    bx = torch.sin(2 * math.pi * (tx / X + float(ph[0])))[None, None, :]
    for z0 in range(0, Z, 64):
        sl = slice(z0, min(Z, z0 + 64))
        t = img[sl] * (1.0 + 0.3 * bz[sl] * by * bx)
        t += torch.randn(t.shape, generator=gen, device=device) * 10.0
        img[sl] = torch.clamp(t, 0.0, 255.0)
    img_u8 = torch.round(img).to(torch.uint8)
    del img
    phi0 = signed_distance_torch(pert_flat.view(Z, Y, X), 3.0)
    return img_u8, phi0.contiguous(), mask
