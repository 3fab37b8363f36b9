"""GPU checks of concurrent use and of the command-line front ends.

* Two workspaces on two streams evolve different volumes at the same time;
  each result equals the same evolution run alone (workspaces are
  independent; one stream per workspace).
* `python -m rsf_gb300.driver` on .npy files equals `driver.segment`.
* `rsf3d` with a float32 image and a uint8 seed equals the Python API.
"""
import subprocess
import sys

import numpy as np
import pytest

from conftest import PKG, ROOT

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _case(shape, seed):
    from rsf_gb300 import synth

    img, phi0, mask = synth.make_small(shape, n_tubes=3, r_min=1.5, r_max=3.5, seed=seed)
    return img, phi0, mask


def test_two_workspaces_on_two_streams(cuda, rsflib):
    from rsf_gb300 import Params, Workspace

    p = Params(sigma=1.5, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)
    cases = [_case((40, 44, 48), 1), _case((36, 50, 42), 2)]
    alone = []
    with Workspace(200_000) as ws:
        for img, phi0, _ in cases:
            t = torch.from_numpy(phi0).cuda()
            ws.evolve(torch.from_numpy(img).cuda(), t, p, 12)
            alone.append(t.clone())
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    wss = [Workspace(200_000), Workspace(200_000)]
    outs = []
    for (img, phi0, _), s, ws in zip(cases, streams, wss):
        with torch.cuda.stream(s):
            ti = torch.from_numpy(img).cuda(non_blocking=True)
            tp = torch.from_numpy(phi0).cuda(non_blocking=True)
            ws.evolve(ti, tp, p, 12, stream=s)
            outs.append(tp)
    for s, ws in zip(streams, wss):
        ws.check(stream=s)
        ws.close()
    torch.cuda.synchronize()
    for a, b in zip(alone, outs):
        assert torch.equal(a, b)


def test_driver_command_line_equals_segment(tmp_path, cuda, rsflib):
    from rsf_gb300 import Params, driver

    img, _, mask = _case((30, 34, 38), 4)
    seed = mask.astype(np.float32) * 26.0
    np.save(tmp_path / "img.npy", img)
    np.save(tmp_path / "seed.npy", seed[None])  # a leading channel axis is squeezed
    out = tmp_path / "phi.npy"
    r = subprocess.run([sys.executable, "-m", "rsf_gb300.driver", "--image", str(tmp_path / "img.npy"), "--binary",
                        str(tmp_path / "seed.npy"), "--ouput", str(out), "--t", "3", "--sigma", "1", "--e", "1",
                        "--v", "65.025", "--eps", "1", "--cores", "16", "--halo", "4", "--mode", "blend"],
                       cwd=str(PKG), capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    p = Params.from_flags(sigma=1.0, dt=0.1, meu=1.0, e=1.0, v=65.025, eps=1.0)
    want = driver.segment(img, seed, p, 3, cores=16, halo=4, mode="blend").cpu().numpy()
    assert np.array_equal(np.load(out).view(np.uint32), want.view(np.uint32))


def test_rsf3d_float_image_and_uint8_seed(tmp_path, cuda, rsflib):
    from rsf_gb300 import Params, Workspace

    img, _, mask = _case((18, 20, 22), 6)
    imgf = img.astype(np.float32) / 2.0
    seed = (mask.astype(np.uint8) * 200)
    np.save(tmp_path / "img.npy", imgf)
    np.save(tmp_path / "seed.npy", seed)
    out = tmp_path / "phi.npy"
    r = subprocess.run([str(PKG / "bin" / "rsf3d"), "--image", str(tmp_path / "img.npy"), "--binary",
                        str(tmp_path / "seed.npy"), "--ouput", str(out), "--t", "2", "--sigma", "1.5", "--quiet"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    p = Params(sigma=1.5)  # reference defaults otherwise (e 0.1, v 1e-4, eps 0.2)
    with Workspace(img.size) as ws:
        phi = ws.signed_distance(torch.from_numpy(seed).cuda(), 13.0)
        ws.evolve(torch.from_numpy(imgf).cuda(), phi, p, 2)
        want = phi.cpu().numpy()
    assert np.array_equal(np.load(out).view(np.uint32), want.view(np.uint32))
