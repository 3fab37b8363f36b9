"""Full-size checks through a size-independent property: locality.

One RSF iteration changes a voxel from values within r + 2 voxels of it
(r = blur radius: the valid correlation; 2: the curvature's nested central
differences), so after t iterations a tile's core that lies at least
t (r + 2) voxels inside the tile's extent, or on a face the tile shares with
the volume, is bit-identical to the same region of the whole volume evolved
in one piece.  These tests evolve the 512^3 and 1024^3 volumes whole, and as
the batched tiles of the workloads (cores plus 32-voxel halos), stitch the
cores on the device and compare every voxel.  They use the clamp rule at
x = 0: the reference rule reads the previous row's last voxel there, which
is a different voxel in a tile than in the whole volume, so locality does not
hold on that column.
"""
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _volume(shape, dev, seed):
    """A smooth level set with many interfaces and a random uint8 image."""
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    L, H, W = shape
    z = torch.arange(L, device=dev, dtype=torch.float32).view(L, 1, 1)
    y = torch.arange(H, device=dev, dtype=torch.float32).view(1, H, 1)
    x = torch.arange(W, device=dev, dtype=torch.float32).view(1, 1, W)
    phi = (3 * torch.sin(x * 0.07) * torch.sin(y * 0.05 + 1) * torch.sin(z * 0.06 + 2)).clamp_(-3, 3).contiguous()
    img = torch.randint(0, 256, shape, dtype=torch.uint8, device=dev, generator=gen)
    return img, phi


def _tiled_equals_whole(shape, cores, halo, sigma, iters, seed):
    from rsf_gb300 import Params, Workspace, gaussian_taps, tiling

    r = (len(gaussian_taps(sigma)) - 1) // 2
    assert iters * (r + 2) <= halo
    dev = torch.device("cuda:0")
    img, phi = _volume(shape, dev, seed)
    p = Params(sigma=sigma, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0, boundary="clamp")
    tiles = tiling.plan(shape, cores, halo)
    parts = [phi[t.slices()].contiguous() for t in tiles]
    imgs = [img[t.slices()].contiguous() for t in tiles]
    with Workspace(sum(t.voxels for t in tiles), len(tiles)) as ws:
        ws.evolve_batched(list(zip(imgs, parts)), p, iters)
        ws.check()
        stitched = tiling.reassemble_device(ws, tiles, parts, shape, "core")
        ws.check()
    del parts, imgs
    torch.cuda.empty_cache()
    with Workspace(phi.numel()) as ws:
        ws.evolve(img, phi, p, iters)
        ws.check()
    torch.cuda.synchronize()
    same = torch.equal(stitched, phi)
    if not same:
        bad = (stitched != phi).nonzero()
        raise AssertionError(f"{bad.shape[0]} voxels differ, first at {bad[0].tolist()}")


@pytest.mark.parametrize("sigma,iters", [(3.0, 2), (5.0, 1)])
def test_512_cubed_tiles_equal_whole_volume(cuda, rsflib, sigma, iters):
    """The single-volume workload (512^3) against its 256-core tiling."""
    _tiled_equals_whole((512, 512, 512), 256, 32, sigma, iters, seed=1)


def test_1024_cubed_tiles_equal_whole_volume(cuda, rsflib):
    """The gigavoxel workload: 1024^3, sigma 4 (29 taps), 27 tiles of 384/384/256 cores
    with 32-voxel halos (1.53 G tile voxels), two iterations."""
    free, _ = torch.cuda.mem_get_info()
    if free < 140e9:
        pytest.skip("needs about 120 GB of free device memory")
    b = [0, 384, 768, 1024]
    _tiled_equals_whole((1024, 1024, 1024), (b, b, b), 32, 4.0, 2, seed=3)
