"""Batch driver: cut, evolve, stitch.

The reference's pipeline cuts a large 8-bit stack into overlapping NumPy
sub-volumes (disassemble.py, README.md:6), runs one `rsf3d` process per
sub-volume (rsfbatch.py, README.md:56), each building phi0 = sdf(seed - 13)
from its own seed (CUDA_RSF/main.cpp:174-183), and stitches the level sets
(reassemble.py, README.md:9); none of those scripts ships.  `segment` does
the whole job on one GPU: tiles come from `tiling.plan`, every tile's phi0 is
built on the device (rsf_signed_distance of its own seed, as each rsf3d
process did), chunks of tiles sized to the device evolve together through
rsf_evolve_batched, and rsf_reassemble stitches the evolved tiles.  Inputs
may be NumPy arrays (memory-mapped .npy files are read tile by tile) or CUDA
tensors; a probability volume from a model passes straight in as the seed
with threshold 0.5, with no file in between.

    python -m rsf_gb300.driver --image vol.npy --binary seed.npy --ouput phi.npy \\
        --cores 256 --halo 32 --t 150 --sigma 3 --e 1 --v 65.025 --eps 1
"""
from __future__ import annotations

import argparse
from typing import List, Sequence

import numpy as np

from .api import Params, Workspace
from .tiling import Tile, lpt_shards, plan, reassemble_device

# Device bytes per tile voxel while a chunk evolves: workspace 36, phi 4,
# image up to 4, seed up to 4.
_BYTES_PER_VOXEL = 48


def chunk_tiles(tiles: Sequence[Tile], max_voxels: int) -> List[List[int]]:
    """Consecutive groups of tile indices whose voxel sums stay within
    `max_voxels` (a tile larger than the budget gets a group of its own)."""
    groups: List[List[int]] = []
    cur: List[int] = []
    load = 0
    for i, t in enumerate(tiles):
        if cur and load + t.voxels > max_voxels:
            groups.append(cur)
            cur, load = [], 0
        cur.append(i)
        load += t.voxels
    if cur:
        groups.append(cur)
    return groups


def _tile_to_device(src, t: Tile, device):
    import torch

    if torch.is_tensor(src):
        return src[t.slices()].contiguous()
    part = np.ascontiguousarray(src[t.slices()])
    if part.dtype not in (np.uint8, np.float32):
        part = part.astype(np.float32)
    return torch.from_numpy(part).pin_memory().to(device, non_blocking=True)


def segment(image, seed, params: Params, iters: int, cores=256, halo: int = 32, mode: str = "core",
            threshold: float = 13.0, max_chunk_voxels: int | None = None, device="cuda:0", tiles=None,
            distributed: bool = False):
    """Evolved level set of the whole volume as a CUDA float32 tensor (L, H, W).

    image: uint8 or float32 (L, H, W) array or CUDA tensor; seed: same shape,
    inside where seed > threshold.  Tiles: `tiles` if given, else
    plan(shape, cores, halo); cores="auto" lets the autotuner measure the
    candidate core sizes first.  mode: "core" or "blend" stitching.

    distributed=True shards the tiles over the ranks of the initialised
    torch.distributed process group (one process per GPU, `device` its own):
    rank r evolves lpt_shards(tiles, world)[r] with no collective during the
    evolution, then every rank sends its evolved tiles to rank 0 (host
    tensors with the gloo backend, device tensors with NCCL), which stitches
    and returns the volume; the other ranks return None.  Every rank must
    pass the same volume and parameters; with cores="auto" rank 0's choice
    is broadcast."""
    import torch

    device = torch.device(device)
    shape = tuple(int(s) for s in image.shape)
    if tuple(seed.shape) != shape:
        raise ValueError(f"image {shape} and seed {tuple(seed.shape)} differ in shape")
    rank, world = 0, 1
    if distributed:
        import torch.distributed as dist

        if not dist.is_initialized():
            raise RuntimeError("distributed=True needs an initialised torch.distributed process group")
        rank, world = dist.get_rank(), dist.get_world_size()
    if tiles is None and cores == "auto":
        from .autotune import tune_cores

        dt = "u8" if str(image.dtype) in ("uint8", "torch.uint8") else "f32"
        if rank == 0:
            cores = tune_cores(shape, params, halo, dt, device=device).cores
        if world > 1:
            box = [cores]
            dist.broadcast_object_list(box, src=0)
            cores = box[0]
    tiles = list(tiles) if tiles is not None else plan(shape, cores, halo)
    shards = lpt_shards(tiles, world)
    mine = shards[rank]
    if max_chunk_voxels is None:
        free, _ = torch.cuda.mem_get_info(device)
        reserve = 4 * (np.prod(shape) + sum(t.voxels for t in tiles))  # output + evolved tiles
        max_chunk_voxels = max(int((free - reserve) * 0.8) // _BYTES_PER_VOXEL, max(t.voxels for t in tiles))
    local = [tiles[i] for i in mine]
    groups = [[mine[j] for j in g] for g in chunk_tiles(local, max_chunk_voxels)] if mine else []
    ws_voxels = max([sum(tiles[i].voxels for i in g) for g in groups] + [1])
    ws_tiles = max([len(tiles)] + [len(g) for g in groups])
    parts: List = [None] * len(tiles)
    with torch.cuda.device(device), Workspace(ws_voxels, ws_tiles) as ws:
        for g in groups:
            pairs = []
            for i in g:
                img = _tile_to_device(image, tiles[i], device)
                sd = _tile_to_device(seed, tiles[i], device)
                phi = ws.signed_distance(sd, threshold)
                pairs.append((img, phi))
                parts[i] = phi
            ws.evolve_batched(pairs, params, iters)
            ws.check()
        if world > 1:
            _gather_tiles(parts, tiles, shards, rank, device)
            if rank != 0:
                return None
        out = reassemble_device(ws, tiles, parts, shape, mode)
        ws.check()
    return out


def _gather_tiles(parts, tiles, shards, rank, device):
    """Every rank's evolved tiles into rank 0's `parts`, in shard order, by
    point-to-point sends (host tensors with gloo, device tensors with NCCL)."""
    import torch
    import torch.distributed as dist

    on_host = dist.get_backend() == "gloo"
    if rank != 0:
        for i in shards[rank]:
            t = parts[i]
            dist.send(t.cpu() if on_host else t.contiguous(), dst=0)
        return
    for src in range(1, len(shards)):
        for i in shards[src]:
            buf = torch.empty(tiles[i].shape, dtype=torch.float32, device="cpu" if on_host else device)
            dist.recv(buf, src=src)
            parts[i] = buf.to(device) if on_host else buf


def main(argv=None):
    ap = argparse.ArgumentParser(description="Cut, evolve and stitch one large volume on the GPU.")
    ap.add_argument("--image", required=True)
    ap.add_argument("--binary", required=True, help="seed volume (.npy); inside where seed > --threshold")
    ap.add_argument("--ouput", "--output", dest="output", default="out.npy")
    ap.add_argument("--sigma", type=float, default=5.0)
    ap.add_argument("--t", type=int, default=30)
    ap.add_argument("--dt", type=float, default=0.1)
    ap.add_argument("--meu", type=float, default=1.0)
    ap.add_argument("--e", type=float, default=0.1)
    ap.add_argument("--v", type=float, default=0.0001)
    ap.add_argument("--eps", type=float, default=0.2)
    ap.add_argument("--threshold", type=float, default=13.0)
    ap.add_argument("--cores", default="256", help="core size in voxels, or 'auto' to measure candidates")
    ap.add_argument("--halo", type=int, default=32)
    ap.add_argument("--mode", choices=("core", "blend"), default="core")
    args = ap.parse_args(argv)
    image = np.load(args.image, mmap_mode="r")
    seed = np.load(args.binary, mmap_mode="r")
    while image.ndim > 3 and image.shape[0] == 1:
        image = image[0]
    while seed.ndim > 3 and seed.shape[0] == 1:
        seed = seed[0]
    p = Params.from_flags(sigma=args.sigma, dt=args.dt, meu=args.meu, e=args.e, v=args.v, eps=args.eps)
    cores = args.cores if args.cores == "auto" else int(args.cores)
    out = segment(image, seed, p, args.t, cores=cores, halo=args.halo, mode=args.mode,
                  threshold=args.threshold)
    np.save(args.output, out.cpu().numpy())
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
