"""CPU checks of the adjoint's checkers: the float64 autograd step
(oracle/rsf_autograd.py) against the C oracle's FP64 evolution, and its
gradients against FP64 central differences of that evolution.

The step is smooth only where |grad phi| stays away from 0: n = g / (|g| + 1e-6)
has derivative 1e6 at g = 0, so a signed distance with a medial axis (g = 0 on
it) gives finite differences that do not converge.  Gradient checks therefore
use a level set without critical points (a ramp plus smooth noise) and an
image scaled to [0, 1]; the forward checks also cover the clipped signed
distance.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def f32(v):
    return float(np.float32(v))


def smooth_case(shape, seed=3):
    from scipy import ndimage

    from rsf_gb300 import synth

    img, _, mask = synth.make_small(shape, n_tubes=3, seed=seed)
    rng = np.random.default_rng(seed + 4)
    z = np.arange(shape[0], dtype=np.float64)[:, None, None]
    phi0 = (0.5 * (z - shape[0] / 2) + 40.0 * ndimage.gaussian_filter(rng.standard_normal(shape), 3)).astype(np.float32)
    return (img.astype(np.float32) / 255.0), phi0, mask


PP = dict(sigma=1.5, dt=0.1, mu=0.2, lambda1=1.0, lambda2=1.0, nu=0.1, eps=1.0)


def soft_dice_np(phi, mask, eps=1.0):
    h = 0.5 * (1 + (2 / np.pi) * np.arctan(phi / eps))
    m = mask.astype(np.float64)
    return 1 - 2 * (h * m).sum() / (h.sum() + m.sum())


@pytest.mark.parametrize("boundary", [0, 1])
def test_torch_step_equals_c_fp64_twin(orc, boundary):
    from oracle import rsf_autograd as ra
    from rsf_gb300 import synth

    img, phi0, _ = synth.make_small((14, 16, 18), n_tubes=3, seed=2)
    pp = dict(sigma=1.5, dt=0.1, mu=1.0, lambda1=1.0, lambda2=0.5, nu=65.025, eps=1.0)
    want = orc.evolve_f64(phi0.astype(np.float64), img.astype(np.float32), orc.params(**pp, boundary=boundary), 3)
    got = ra.evolve(torch.from_numpy(phi0.astype(np.float64)), torch.from_numpy(img.astype(np.float64)),
                    orc.taps(1.5), dict(dt=f32(0.1), eps=1.0, lambda1=1.0, lambda2=0.5, mu=1.0, nu=f32(65.025)), 3,
                    boundary=boundary).numpy()
    assert np.abs(got - want).max() <= 1e-11 * np.abs(want).max()


def test_torch_autograd_matches_fp64_central_differences(orc):
    from oracle import rsf_autograd as ra

    shape, T = (16, 18, 20), 8
    img, phi0, mask = smooth_case(shape)
    pp = {k: f32(v) for k, v in PP.items()}
    p0 = torch.from_numpy(phi0.astype(np.float64)).requires_grad_(True)
    prm = {k: torch.tensor(pp[k], dtype=torch.float64, requires_grad=True) for k in ("lambda1", "lambda2", "mu", "nu")}
    phiT = ra.evolve(p0, torch.from_numpy(img.astype(np.float64)), orc.taps(PP["sigma"]),
                     dict(dt=pp["dt"], eps=pp["eps"], **prm), T)
    m = torch.from_numpy(mask.astype(np.float64))
    h = 0.5 * (1 + (2 / np.pi) * torch.atan(phiT / pp["eps"]))
    (1 - 2 * (h * m).sum() / (h.sum() + m.sum())).backward()

    def loss(phi0_, **kw):
        P = orc.params(**dict(PP, **kw))
        return soft_dice_np(orc.evolve_f64(phi0_.astype(np.float64), img, P, T), mask)

    from scipy import ndimage

    v = ndimage.gaussian_filter(np.random.default_rng(1).standard_normal(shape), 2.0)
    v /= np.abs(v).max()
    hs = 1e-4
    fd = (loss(phi0 + hs * v) - loss(phi0 - hs * v)) / (2 * hs)
    ad = float((p0.grad.numpy() * v).sum())
    assert abs(fd - ad) <= 1e-6 * abs(fd)
    for k in ("lambda1", "lambda2", "mu", "nu"):
        up, dn = f32(pp[k] * (1 + 1e-3)), f32(pp[k] * (1 - 1e-3))
        fd = (loss(phi0, **{k: up}) - loss(phi0, **{k: dn})) / (up - dn)
        assert abs(fd - prm[k].grad.item()) <= 1e-4 * abs(fd), k
