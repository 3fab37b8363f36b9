"""Full-size workloads against the CPU oracle, voxel for voxel.

* The gigavoxel batch: the 1024^3 synthetic vessel volume (2000 tubes,
  radius U[1, 10]) cut into its 27 tiles (384/384/256 cores + 32-voxel
  halos), all evolved in one batched call for 200 iterations at sigma 4
  (29 taps) with the reference's x = 0 rule.  The far corner tile (288^3)
  and the tile that is interior along x (448 x 288 x 288) are evolved by the
  oracle from the same tile inputs and compared block by block.
* The single-volume workload: one 512^3 volume (200 tubes) at sigma 5
  (35 taps) through rsf_evolve for 20 iterations; one iteration reaches
  r + 2 = 19 voxels, so after 20 the faces, the 30-valued border band and
  the interior have all influenced each other.

The bar is bit equality (tolerance 0); sign agreement and max|dphi| are
reported with every failure.  The oracle runs on all host cores (about two
minutes on 16 cores for all three comparisons).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

PARAMS = dict(dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=0.001 * 255.0 ** 2, eps=1.0)


def _compare(got, want, what):
    same = np.array_equal(got.view(np.uint32), want.view(np.uint32))
    agree = float((np.sign(got) == np.sign(want)).mean())
    maxrel = float(np.abs(got.astype(np.float64) - want).max() / np.abs(want).max())
    assert same, (f"{what}: {int((got != want).sum())} voxels differ, sign agreement {agree:.6f}, "
                  f"max|dphi|/max|phi| {maxrel:.3g}")
    assert agree >= 0.9999 and maxrel <= 1e-4


def _oracle(orc, phi0, img, sigma, iters):
    p = orc.params(sigma=sigma, **PARAMS)
    return orc.evolve(phi0, img.astype(np.float32), p, iters, os.cpu_count() or 1)


def test_gigavoxel_batch_blockwise_against_oracle(cuda, rsflib, orc):
    from rsf_gb300 import Params, Workspace, synth, tiling

    free, _ = torch.cuda.mem_get_info()
    if free < 100e9:
        pytest.skip("needs about 80 GB of free device memory")
    img_full, phi_full, _ = synth.make_volume_torch(synth.CONFIG3, cuda)
    tiles = tiling.config3_tiles()
    imgs = [img_full[t.slices()].contiguous() for t in tiles]
    phis = [phi_full[t.slices()].contiguous() for t in tiles]
    del img_full, phi_full
    torch.cuda.empty_cache()
    picks = {26: "far corner tile (288^3)", 25: "x-interior tile (448 x 288 x 288)"}
    starts = {i: (imgs[i].cpu().numpy(), phis[i].cpu().numpy()) for i in picks}
    p = Params(sigma=4.0, **PARAMS)
    with Workspace(sum(t.voxels for t in tiles), len(tiles)) as ws:
        ws.evolve_batched(list(zip(imgs, phis)), p, 200)
        ws.check()
    got = {i: phis[i].cpu().numpy() for i in picks}
    del imgs, phis
    torch.cuda.empty_cache()
    for i, what in picks.items():
        assert tiles[i].shape == starts[i][1].shape
        img, phi0 = starts[i]
        _compare(got[i], _oracle(orc, phi0, img, 4.0, 200), what)


def test_512_cubed_sigma5_against_oracle(cuda, rsflib, orc):
    from rsf_gb300 import Params, Workspace, synth

    img, phi0, _ = synth.make_volume_torch(synth.CONFIG1, cuda)
    start = phi0.cpu().numpy()
    with Workspace(phi0.numel()) as ws:
        ws.evolve(img, phi0, Params(sigma=5.0, **PARAMS), 20)
        ws.check()
    got = phi0.cpu().numpy()
    _compare(got, _oracle(orc, start, img.cpu().numpy(), 5.0, 20), "512^3, sigma 5, 20 iterations")
