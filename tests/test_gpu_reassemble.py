"""GPU checks of the reassembly gather (rsf_reassemble) and of the batch
driver (cut -> per-tile phi0 -> batched evolution -> stitch).

Checkers: oracle/reassembly.py (core crop; the linear blend of
interpolating_volumes.py:10-40 generalised to a grid) and the C oracle's
evolution and signed distance per tile.  Core stitching and everything before
it are bit-exact; the blend is floating point and is held to 1e-6 of the
values' magnitude.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _grid_case(shape, cores, halo, seed=0):
    from rsf_gb300 import tiling

    tiles = tiling.plan(shape, cores, halo)
    rng = np.random.default_rng(seed)
    parts = [rng.standard_normal(t.shape).astype(np.float32) * 5 for t in tiles]
    return tiles, parts


GRIDS = [((40, 48, 56), ([0, 8, 30, 40], 16, [0, 20, 56]), 5),
         ((20, 30, 33), (20, 15, 11), 3),
         ((17, 19, 23), ([0, 17], [0, 9, 19], [0, 4, 12, 23]), 1),
         ((12, 40, 14), ([0, 12], [0, 20, 40], [0, 14]), 0)]


@pytest.mark.parametrize("shape,cores,halo", GRIDS)
def test_reassemble_core_and_blend(ws_big, shape, cores, halo):
    from oracle import reassembly
    from rsf_gb300 import tiling

    tiles, parts = _grid_case(shape, cores, halo)
    dparts = [torch.from_numpy(p).cuda() for p in parts]
    got = tiling.reassemble_device(ws_big, tiles, dparts, shape, "core").cpu().numpy()
    assert np.array_equal(got, reassembly.reassemble_cores(shape, tiles, parts))
    got = tiling.reassemble_device(ws_big, tiles, dparts, shape, "blend").cpu().numpy()
    want = reassembly.blend_grid(shape, tiles, parts)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()


def test_blend_of_two_halves_is_the_reference_blend(ws_big):
    from oracle import reassembly
    from rsf_gb300 import tiling

    # two volumes overlapping by 46 voxels along y, as interpolating_volumes.py blends them
    shape, ov = (10, 200, 12), 46
    tiles = [tiling.Tile((0, 0, 0), (10, 100 + ov // 2, 12), (0, 0, 0), (10, 100, 12)),
             tiling.Tile((0, 100 - ov // 2, 0), (10, 200, 12), (0, 100, 0), (10, 200, 12))]
    rng = np.random.default_rng(3)
    a = rng.standard_normal(tiles[0].shape).astype(np.float32)
    b = rng.standard_normal(tiles[1].shape).astype(np.float32)
    got = tiling.reassemble_device(ws_big, tiles, [torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()], shape,
                                   "blend").cpu().numpy()
    want = reassembly.blend_halves(a, b, ov, axis=1)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()


def _driver_case(shape=(36, 40, 44), seed=4):
    from rsf_gb300 import Params, synth

    img, _, mask = synth.make_small(shape, n_tubes=4, r_min=2.0, r_max=4.0, seed=seed)
    seed_vol = mask.astype(np.float32) * 26.0
    p = Params(sigma=1.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)
    return img, seed_vol, p


def _oracle_tiles(orc, img, seed_vol, p, tiles, iters):
    P = orc.params(sigma=p.sigma, dt=p.dt, mu=p.mu, lambda1=p.lambda1, lambda2=p.lambda2, nu=p.nu, eps=p.eps)
    out = []
    for t in tiles:
        phi0 = orc.signed_distance(seed_vol[t.slices()], 13.0)
        out.append(orc.evolve(phi0, img[t.slices()].astype(np.float32), P, iters))
    return out


def test_driver_core_mode_is_bit_exact_per_tile(cuda, rsflib, orc):
    from oracle import reassembly
    from rsf_gb300 import driver, tiling

    img, seed_vol, p = _driver_case()
    tiles = tiling.plan(img.shape, (12, 20, [0, 30, 44]), 4)
    got = driver.segment(img, seed_vol, p, 3, tiles=tiles).cpu().numpy()
    want = reassembly.reassemble_cores(img.shape, tiles, _oracle_tiles(orc, img, seed_vol, p, tiles, 3))
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # chunked into several batched calls: same bits
    got2 = driver.segment(img, seed_vol, p, 3, tiles=tiles, max_chunk_voxels=6000).cpu().numpy()
    assert np.array_equal(got2.view(np.uint32), got.view(np.uint32))


def test_driver_blend_mode_and_tensor_handoff(cuda, rsflib, orc):
    from oracle import reassembly
    from rsf_gb300 import driver, tiling

    img, seed_vol, p = _driver_case(seed=6)
    tiles = tiling.plan(img.shape, 20, 5)
    want = reassembly.blend_grid(img.shape, tiles, _oracle_tiles(orc, img, seed_vol, p, tiles, 2))
    got = driver.segment(img, seed_vol, p, 2, tiles=tiles, mode="blend").cpu().numpy()
    assert np.abs(got - want).max() <= 1e-6 * np.abs(want).max()
    # a probability volume on the device as the seed (threshold 0.5), no file
    prob = torch.from_numpy(seed_vol / 26.0).cuda()
    got_t = driver.segment(torch.from_numpy(img).cuda(), prob, p, 2, tiles=tiles, mode="blend",
                           threshold=0.5).cpu().numpy()
    assert np.array_equal(got_t.view(np.uint32), got.view(np.uint32))


def test_autotuner_measures_candidates_on_device(cuda, rsflib):
    from rsf_gb300 import Params, autotune, driver

    p = Params(sigma=1.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)
    res = autotune.tune_cores((48, 64, 64), p, halo=4, candidates=(16, 32, 64), iters=2)
    assert res.cores in (16, 32, 64) and len(res.table) == 3 and all(r[1] > 0 for r in res.table)
    img, seed_vol, _ = _driver_case((24, 30, 32))
    out = driver.segment(img, seed_vol, p, 2, cores="auto", halo=4)
    assert out.shape == img.shape and bool(torch.isfinite(out).all())
