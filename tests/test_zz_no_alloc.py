"""The allocation-free entry point (rsf_evolve_noalloc) against rsf_evolve.

rsf_evolve_noalloc serves callers that cannot allocate device memory while
running (plug-ins inside an application that owns the device memory budget
through its own pool, real-time loops that forbid allocation after start-up):
it keeps its scratch in one static device array of the library instead of a
workspace.  This test calls
it through the C ABI twice in a row, on two different volumes, so that the
second call runs on the scratch contents the first call left behind, and
requires each result to be bit-identical to the workspace entry point's
(the tolerance every parity test here uses).  It lives in its own file that
pytest collects last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib):
    from rsf_gb300._lib import RsfParams

    fn = lib.rsf_evolve_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(RsfParams), ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
                   ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p]
    return fn


def _volume(shape, seed):
    from rsf_gb300 import synth

    img, phi0, _ = synth.make_small(shape, n_tubes=4, r_min=1.5, r_max=4.0, seed=seed)
    return img, phi0


@pytest.mark.parametrize("sigma", [3.0, 1.5])
def test_noalloc_matches_workspace_entry_point(sigma, cuda, rsflib):
    import torch
    from rsf_gb300 import Params, Workspace

    fn = _noalloc(rsflib)
    p = Params(sigma=sigma, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)
    cases = [((64, 80, 96), 31, 5), ((40, 50, 44), 32, 4)]  # second call is smaller: stale scratch behind it
    with Workspace(64 * 80 * 96) as ws:
        for shape, seed, iters in cases:
            img, phi0 = _volume(shape, seed)
            ti = torch.from_numpy(img).to(cuda)
            want = torch.from_numpy(phi0).to(cuda)
            ws.evolve(ti, want, p, iters)
            ws.check()
            got = torch.from_numpy(phi0).to(cuda)
            torch.cuda.synchronize()
            L, H, W = shape
            st = fn(ctypes.byref(p.to_c()), ctypes.c_void_p(ti.data_ptr()), 0, ctypes.c_void_p(got.data_ptr()),
                    W, H, L, iters, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
            assert st == 0, rsflib.rsf_last_error().decode()
            torch.cuda.synchronize()
            assert torch.equal(got, want), f"{int((got != want).sum())} voxels differ for shape {shape}"


def test_noalloc_rejects_volumes_above_its_limit(cuda, rsflib):
    import torch
    from rsf_gb300 import Params

    fn = _noalloc(rsflib)
    p = Params(sigma=3.0)
    buf = torch.zeros(16, device=cuda)
    st = fn(ctypes.byref(p.to_c()), ctypes.c_void_p(buf.data_ptr()), 1, ctypes.c_void_p(buf.data_ptr()),
            1024, 1024, 2, 1, None)
    assert st == 6  # RSF_ERR_WORKSPACE_TOO_SMALL, before any device work
    assert b"1048576" in rsflib.rsf_last_error()
