"""GPU checks of the initial level set and of the rsf3d executable.

rsf_signed_distance against the oracle's brute-force restatement (exact
integer squared distances, so tolerance 0), and rsf3d end to end against the
Python API and the oracle on the same .npy inputs.
"""
import subprocess

import numpy as np
import pytest

from conftest import PKG

pytestmark = pytest.mark.gpu

CLI = PKG / "bin" / "rsf3d"


def _blobs(shape, seed, scale=30.0):
    from scipy import ndimage

    rng = np.random.default_rng(seed)
    return ndimage.uniform_filter((rng.random(shape) * scale).astype(np.float32), 3)


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


SDF_CASES = [
    ((9, 11, 13), "f32"), ((1, 1, 40), "f32"), ((40, 1, 1), "f32"), ((1, 37, 1), "u8"), ((6, 7, 1), "f32"),
    ((33, 31, 65), "u8"), ((20, 70, 3), "f32"), ((64, 48, 40), "f32"),
]


@pytest.mark.parametrize("shape,dt", SDF_CASES)
def test_signed_distance_bit_exact_vs_oracle(ws_big, orc, shape, dt):
    import torch

    seed = _blobs(shape, sum(shape))
    if dt == "u8":
        seed = np.round(seed * 4).astype(np.uint8)
    thr = float(np.median(seed))
    want = orc.signed_distance(seed.astype(np.float32), thr)
    got = ws_big.signed_distance(torch.from_numpy(seed).cuda(), thr).cpu().numpy()
    assert _bits_equal(got, want), f"{int((got != want).sum())} voxels differ"


def test_signed_distance_matches_scipy_at_128_cubed(ws_big):
    import torch
    from scipy import ndimage

    seed = _blobs((128, 128, 128), 11)
    thr = float(np.quantile(seed, 0.7))
    m = seed > thr
    want = np.where(m, ndimage.distance_transform_edt(m), -ndimage.distance_transform_edt(~m)).astype(np.float32)
    got = ws_big.signed_distance(torch.from_numpy(seed).cuda(), thr).cpu().numpy()
    assert _bits_equal(got, want)


def test_signed_distance_one_class_and_errors(cuda, rsflib):
    import torch

    from rsf_gb300 import RsfError, Workspace

    with Workspace(1000) as ws:
        s = torch.full((4, 5, 6), 13.0, device=cuda)
        assert torch.all(ws.signed_distance(s, 13.0) == -15.0)
        assert torch.all(ws.signed_distance(s, 12.0) == 15.0)
        with pytest.raises(RsfError):
            ws.signed_distance(torch.zeros((11, 10, 10), device=cuda), 0.5)  # 1100 voxels > workspace


def _save_inputs(tmp_path, shape, seed_num, fortran=False):
    from rsf_gb300 import synth

    img, _, mask = synth.make_small(shape, n_tubes=3, r_min=1.5, r_max=3.5, seed=seed_num)
    seed = (mask.astype(np.float32) * 26.0)  # inside 26 > 13, outside 0
    ip, sp = tmp_path / "img.npy", tmp_path / "seed.npy"
    np.save(ip, np.asfortranarray(img) if fortran else img)
    np.save(sp, np.asfortranarray(seed) if fortran else seed)
    return img, seed, ip, sp


def _cli_run(*args):
    r = subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r


@pytest.mark.parametrize("fortran", [False, True])
def test_rsf3d_equals_api_and_oracle(tmp_path, cuda, rsflib, orc, fortran):
    import torch

    from rsf_gb300 import Params, Workspace

    img, seed, ip, sp = _save_inputs(tmp_path, (18, 22, 26), 5, fortran)
    out = tmp_path / "phi.npy"
    T = 4
    r = _cli_run("--image", ip, "--binary", sp, "--ouput", out, "--t", T, "--sigma", 1.5, "--e", 1.0, "--v", 65.025,
                 "--eps", 1.0)
    assert r.stdout.count("It takes ") == T and " ms to calculate" in r.stdout
    got = np.load(out)
    assert got.dtype == np.float32 and got.shape == img.shape
    p = Params(sigma=1.5, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)
    with Workspace(img.size) as ws:
        phi = ws.signed_distance(torch.from_numpy(seed).cuda(), 13.0)
        ws.evolve(torch.from_numpy(img).cuda(), phi, p, T)
        ws.check()
        api = phi.cpu().numpy()
    assert _bits_equal(got, api)
    phi0 = orc.signed_distance(seed, 13.0)
    want = orc.evolve(phi0, img.astype(np.float32),
                      orc.params(sigma=1.5, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0), T)
    assert _bits_equal(got, want)


def test_rsf3d_quiet_output_alias_and_reference_defaults(tmp_path, cuda, rsflib):
    img, seed, ip, sp = _save_inputs(tmp_path, (40, 40, 40), 9)
    a, b = tmp_path / "a.npy", tmp_path / "b.npy"
    r1 = _cli_run("--image", ip, "--binary", sp, "--output", a, "--t", 3, "--sigma", 2, "--quiet")
    assert r1.stdout.count("It takes ") == 1
    r2 = _cli_run("--image", ip, "--binary", sp, "--ouput", b, "--t", 3, "--sigma", 2, "--debug")
    assert r2.stdout.count("It takes ") == 3 and "stencil/update" in r2.stdout
    assert _bits_equal(np.load(a), np.load(b))
