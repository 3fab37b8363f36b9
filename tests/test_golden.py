"""The oracle against golden outputs of the reference's own kernels.

tests/golden/reference_kernels_*.npz hold inputs and the outputs of
CUDA_RSF/kernel.cu (compiled unchanged, run on a GB300 by
tests/golden/make_reference_goldens.py) for one and three iterations.  Every
oracle stage fed the reference's own stage inputs must reproduce the stored
output bit for bit; H (CUDA atanf) and the whole iterations, which inherit
it, are compared with tolerances.
"""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = sorted((Path(__file__).resolve().parent / "golden").glob("reference_kernels_*.npz"))


def _eq(a, b):
    return np.array_equal(np.ascontiguousarray(a, np.float32).view(np.uint32),
                          np.ascontiguousarray(b, np.float32).view(np.uint32))


@pytest.fixture(params=GOLDEN, ids=lambda p: p.stem)
def gold(request):
    return dict(np.load(request.param))


def test_goldens_present():
    assert len(GOLDEN) >= 2


def test_stages_bit_exact_against_reference(orc, gold):
    phi0, I = gold["phi0"], gold["image"].astype(np.float32)
    sigma = float(gold["sigma"])
    g = orc.gradient(phi0, boundary=0)
    assert _eq(g[0], gold["gx"]) and _eq(g[1], gold["gy"]) and _eq(g[2], gold["gz"])
    mag, nx, ny, nz = orc.normalise(gold["gx"], gold["gy"], gold["gz"], form=0, arith=1)
    assert _eq(mag, gold["mag"]) and _eq(nx, gold["nx"])
    dg = [orc.gradient(gold[c], boundary=0)[a] for a, c in enumerate(("gx", "gy", "gz"))]
    assert _eq((dg[0] + dg[1]) + dg[2], gold["lap"])
    H = gold["H"]
    assert _eq(orc.blur_padded(I * H, sigma), gold["I_ob"])
    assert _eq(orc.blur_padded(H, sigma), gold["HD_ob"])
    assert _eq(gold["I_ob"] / gold["HD_ob"], gold["fout"])
    assert _eq(orc.dirac(phi0, 0.2, 1), gold["dh"])
    assert _eq(orc.dirac(phi0, 0.2, 0), gold["dh"]) or int(
        np.abs(orc.dirac(phi0, 0.2, 0).view(np.int32).astype(np.int64) - gold["dh"].view(np.int32)).max()) <= 1


def test_curvature_and_update_bit_exact_against_reference(orc, gold):
    phi0, I = gold["phi0"], gold["image"].astype(np.float32)
    _, nx, ny, nz = orc.normalise(gold["gx"], gold["gy"], gold["gz"], form=0, arith=1)
    dn = [orc.gradient(f, boundary=0)[a] for a, f in enumerate((nx, ny, nz))]
    kap = (dn[0] + dn[1]) + dn[2]
    assert _eq(kap, gold["kappa"])
    eo = (I - gold["fout"]) * (I - gold["fout"])
    ei = (I - gold["fin"]) * (I - gold["fin"])
    p = orc.params(sigma=float(gold["sigma"]), eps=0.2, lambda1=1.0, mu=1.0, nu=65.025, dt=0.1)
    assert _eq(orc.update_field(phi0, gold["dh"], eo, ei, gold["kappa"], gold["lap"], p), gold["phi1"])


@pytest.mark.parametrize("arith", [0, 1])
def test_heaviside_within_atan_tolerance(orc, gold, arith):
    h = orc.heaviside(gold["phi0"], 0.2, arith)
    assert float(np.abs(h.astype(np.float64) - gold["H"]).max()) <= 1.2e-7


@pytest.mark.parametrize("arith", [0, 1])
def test_whole_iterations_track_reference(orc, gold, arith):
    """Whole iterations against the reference's own: sign agreement >= 99.99 %
    and max|dphi| <= 1e-4 max|phi|, except the portable arithmetic after
    three iterations.  Its atan differs from CUDA's atanf by up to 1.2e-7 in
    H, and the normalisation n = g/(|g| + 1e-6) amplifies that where phi is
    flat: measured 3.2e-4 (sigma 1) and 2.3e-5 (sigma 3) of max|phi| after
    three iterations, so that case is held to 1e-3."""
    phi0, I = gold["phi0"], gold["image"].astype(np.float32)
    p = orc.params(sigma=float(gold["sigma"]), eps=0.2, lambda1=1.0, mu=1.0, nu=65.025, dt=0.1, arith=arith)
    for iters, key in ((1, "phi1"), (3, "phi3")):
        got = orc.evolve(phi0, I, p, iters)
        want = gold[key]
        assert float((np.sign(got) == np.sign(want)).mean()) >= 0.9999
        bound = 1e-3 if (arith == 0 and iters == 3) else 1e-4
        assert float(np.abs(got - want).max()) <= bound * float(np.abs(want).max())
