"""GPU checks of the hand-written adjoint (rsf_step_adjoint) and of the
checkpointed torch.autograd.Function built on it.

Checkers: the float64 autograd restatement (oracle/rsf_autograd.py) for
vector-Jacobian products of one step and of whole evolutions, and FP64
central differences of the C oracle for the 50-step, checkpoint-every-10
case.  The adjoint runs in FP32, so the bars are relative: 1e-4 (L2 norm) for
one step, 1e-3 for chains, as the gradient tolerance of the benchmark spec states.
"""
import numpy as np
import pytest

from test_adjoint_ref_cpu import PP, f32, smooth_case, soft_dice_np

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _params(**kw):
    from rsf_gb300 import Params

    d = dict(PP)
    d.update(kw)
    return Params(**{k: d[k] for k in ("sigma", "dt", "mu", "lambda1", "lambda2", "nu", "eps")},
                  sigma2=d.get("sigma2", 0.0), boundary=d.get("boundary", "reference"))


def _rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def _vjp_fp64(orc, phi, img, u, p, boundary):
    from oracle import rsf_autograd as ra

    step = ra.Step(phi.shape, orc.taps(p.sigma), f32(p.dt), f32(p.eps), 0 if boundary == "reference" else 1)
    x = torch.from_numpy(phi.astype(np.float64)).requires_grad_(True)
    prm = {k: torch.tensor(f32(getattr(p, k)), dtype=torch.float64, requires_grad=True)
           for k in ("lambda1", "lambda2", "mu", "nu")}
    out = step(x, torch.from_numpy(img.astype(np.float64)), prm["lambda1"], prm["lambda2"], prm["mu"], prm["nu"])
    (out * torch.from_numpy(u.astype(np.float64))).sum().backward()
    return x.grad.numpy(), np.array([prm[k].grad.item() for k in ("lambda1", "lambda2", "mu", "nu")])


STEP_CASES = [
    ((16, 18, 20), 1.5, "reference", "smooth", "f32"),
    ((16, 18, 20), 1.5, "clamp", "smooth", "f32"),
    ((24, 20, 30), 1.0, "reference", "sdf3", "u8"),
    ((9, 8, 10), 1.5, "reference", "smooth", "f32"),  # 11 taps: no valid blur region
    ((2, 3, 40), 1.0, "reference", "smooth", "f32"),
    ((40, 24, 26), 3.0, "reference", "smooth", "u8"),
    # the streaming recompute (21, 29, 35 taps): an odd valid width over two
    # z-pass tiles, and both boundary rules
    ((36, 40, 91), 3.0, "reference", "sdf3", "u8"),
    ((34, 31, 40), 4.0, "clamp", "smooth", "f32"),
    ((40, 38, 45), 5.0, "reference", "smooth", "u8"),
]


@pytest.mark.parametrize("shape,sigma,boundary,kind,dt", STEP_CASES)
def test_single_step_adjoint_matches_fp64_autograd(ws_big, orc, shape, sigma, boundary, kind, dt):
    from rsf_gb300 import synth

    rng = np.random.default_rng(sum(shape))
    img, phi, mask = smooth_case(shape)
    if kind == "sdf3":  # clipped signed distance: flat regions where g = 0 exactly
        phi = synth.signed_distance(mask, clip=3.0)
    if dt == "u8":
        img_dev = torch.from_numpy(np.round(img * 255).astype(np.uint8)).cuda()
        img_ref = np.round(img * 255).astype(np.float32)
        p = _params(sigma=sigma, boundary=boundary, lambda1=1e-4, lambda2=2e-4)
    else:
        img_dev = torch.from_numpy(img).cuda()
        img_ref = img
        p = _params(sigma=sigma, boundary=boundary, lambda2=0.7)
    u = rng.standard_normal(shape).astype(np.float32)
    g = torch.zeros(4, dtype=torch.float64, device="cuda")
    got = ws_big.step_adjoint(img_dev, torch.from_numpy(phi).cuda(), torch.from_numpy(u).cuda(), p,
                              param_grads=g).cpu().numpy()
    want, want_p = _vjp_fp64(orc, phi, img_ref, u, p, boundary)
    assert _rel(got, want) <= 1e-4
    gp = g.cpu().numpy()
    for k in range(4):
        assert abs(gp[k] - want_p[k]) <= 1e-4 * max(abs(want_p[k]), 1e-3 * np.abs(want_p).max()), k


def _grads_gpu(img, phi0, mask, p, T, every):
    from rsf_gb300 import autograd

    prm = {k: torch.tensor(f32(getattr(p, k)), dtype=torch.float64, device="cuda", requires_grad=True)
           for k in ("lambda1", "lambda2", "mu", "nu")}
    x = torch.from_numpy(phi0).cuda().requires_grad_(True)
    phiT = autograd.evolve(x, torch.from_numpy(img).cuda(), p, T, checkpoint_every=every, **prm)
    loss = autograd.soft_dice_loss(phiT.double(), torch.from_numpy(mask).cuda(), p.eps)
    loss.backward()
    return x.grad.cpu().numpy(), np.array([prm[k].grad.item() for k in ("lambda1", "lambda2", "mu", "nu")])


def test_checkpointed_chain_matches_fp64_autograd(cuda, rsflib, orc):
    from oracle import rsf_autograd as ra

    shape, T = (20, 22, 24), 12
    img, phi0, mask = smooth_case(shape)
    p = _params(lambda2=0.8)
    got, got_p = _grads_gpu(img, phi0, mask, p, T, 5)
    x = torch.from_numpy(phi0.astype(np.float64)).requires_grad_(True)
    prm = {k: torch.tensor(f32(getattr(p, k)), dtype=torch.float64, requires_grad=True)
           for k in ("lambda1", "lambda2", "mu", "nu")}
    phiT = ra.evolve(x, torch.from_numpy(img.astype(np.float64)), orc.taps(p.sigma),
                     dict(dt=f32(p.dt), eps=f32(p.eps), **prm), T)
    from rsf_gb300 import autograd

    autograd.soft_dice_loss(phiT, torch.from_numpy(mask), p.eps).backward()
    assert _rel(got, x.grad.numpy()) <= 1e-3
    for k, name in enumerate(("lambda1", "lambda2", "mu", "nu")):
        assert abs(got_p[k] - prm[name].grad.item()) <= 1e-3 * abs(prm[name].grad.item()), name


def test_checkpoint_interval_does_not_change_the_gradient(cuda, rsflib):
    shape, T = (16, 18, 20), 7
    img, phi0, mask = smooth_case(shape, seed=5)
    p = _params()
    ref, ref_p = _grads_gpu(img, phi0, mask, p, T, T)
    for every in (1, 3):
        got, got_p = _grads_gpu(img, phi0, mask, p, T, every)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))  # recompute is bit-identical
        assert np.allclose(got_p, ref_p, rtol=1e-9, atol=0)


def test_fifty_steps_every_ten_against_fp64_central_differences(cuda, rsflib, orc):
    """The differentiable workload at reduced size: T = 50, checkpoints every
    10, soft-Dice loss, FP64 central differences with h = 1e-4."""
    from scipy import ndimage

    shape, T = (40, 40, 40), 50
    img, phi0, mask = smooth_case(shape, seed=11)
    p = _params()
    got, got_p = _grads_gpu(img, phi0, mask, p, T, 10)

    def loss(phi0_, **kw):
        P = orc.params(**dict(PP, **kw))
        return soft_dice_np(orc.evolve_f64(phi0_.astype(np.float64), img, P, T), mask)

    for seed in (1, 2):
        v = ndimage.gaussian_filter(np.random.default_rng(seed).standard_normal(shape), 2.0)
        v /= np.abs(v).max()
        h = 1e-4
        fd = (loss(phi0 + h * v) - loss(phi0 - h * v)) / (2 * h)
        ad = float((got.astype(np.float64) * v).sum())
        assert abs(ad - fd) <= 1e-3 * abs(fd), (ad, fd)
    for k, name in enumerate(("lambda1", "lambda2", "mu", "nu")):
        base = PP[name]
        up, dn = f32(base * (1 + 1e-3)), f32(base * (1 - 1e-3))
        fd = (loss(phi0, **{name: up}) - loss(phi0, **{name: dn})) / (up - dn)
        assert abs(got_p[k] - fd) <= 1e-3 * abs(fd), (name, got_p[k], fd)


def test_adjoint_argument_errors(cuda, rsflib):
    from rsf_gb300 import RsfError, Workspace

    img = torch.rand((10, 10, 10), device=cuda)
    phi = torch.rand((10, 10, 10), device=cuda)
    u = torch.rand((10, 10, 10), device=cuda)
    with Workspace(1000) as ws:
        with pytest.raises(RsfError):
            ws.step_adjoint(img, phi, u, _params(), out=u)  # output overlaps an input
        with pytest.raises(RsfError):
            ws.step_adjoint(img, phi, u, _params(sigma2=1.0))
    with Workspace(999) as ws:
        with pytest.raises(RsfError):
            ws.step_adjoint(img, phi, u, _params())


def _config4_volume(seed):
    from rsf_gb300 import Params, synth

    img, phi0, mask = synth.make_volume(synth.VolumeSpec((128, 128, 128), 12, 2.0, 6.0, seed))
    p = Params(sigma=3.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=0.001 * 255.0 ** 2, eps=1.0)
    return img, phi0, mask, p


def _fp64_vjp(step, x, img64, u, p, device):
    names = ("lambda1", "lambda2", "mu", "nu")
    xt = x.double().requires_grad_(True)
    pr = [torch.tensor(f32(getattr(p, k)), dtype=torch.float64, device=device, requires_grad=True) for k in names]
    (step(xt, img64, *pr) * u).sum().backward()
    return xt.grad, np.array([v.grad.item() for v in pr])


@pytest.mark.parametrize("seed", [40, 41])
def test_config4_volume_step_adjoints_against_fp64_autograd(cuda, rsflib, orc, seed):
    """Volumes of the differentiable workload at their stated size and inputs:
    128^3 from the 128^3 generator (uint8 image 0-255, phi0 the +-3-clipped
    signed distance), sigma 3, lambda1 = lambda2 = 1, mu 1, nu 0.001*255^2,
    eps 1, dt 0.1.  The CUDA adjoint of one step at states 0, 10, 25 and 49
    of the 50-step evolution, for a random upstream gradient, against the
    float64 autograd restatement run on the GPU at the same FP32 state:
    relative L2 error of dL/dphi and relative errors of the four parameter
    gradients <= 1e-4."""
    from oracle import rsf_autograd as ra
    from rsf_gb300 import Workspace

    img, phi0, mask, p = _config4_volume(seed)
    ti = torch.from_numpy(img).to(cuda)
    img64 = ti.double()
    step = ra.Step(img.shape, orc.taps(p.sigma), f32(p.dt), f32(p.eps), 0, cuda)
    gen = torch.Generator(device=cuda)
    gen.manual_seed(seed)
    with Workspace(img.size) as ws:
        phi = torch.from_numpy(phi0).to(cuda)
        for t in range(50):
            if t in (0, 10, 25, 49):
                u = torch.randn(phi.shape, device=cuda, generator=gen)
                g = torch.zeros(4, dtype=torch.float64, device=cuda)
                got = ws.step_adjoint(ti, phi, u, p, param_grads=g).double()
                ws.check()
                want, want_p = _fp64_vjp(step, phi, img64, u.double(), p, cuda)
                rel = float(torch.linalg.vector_norm(got - want) / torch.linalg.vector_norm(want))
                assert rel <= 1e-4, f"state {t}: dL/dphi relative L2 error {rel:.3g}"
                gp = g.cpu().numpy()
                for k in range(4):
                    assert abs(gp[k] - want_p[k]) <= 1e-4 * max(abs(want_p[k]), 1e-3 * np.abs(want_p).max()), \
                        (t, k, gp[k], want_p[k])
            ws.evolve(ti, phi, p, 1)
        ws.check()


@pytest.mark.parametrize("seed", [40, 41])
def test_config4_volume_chain_against_fp64_autograd(cuda, rsflib, orc, seed):
    """The checkpointed chain on the same volumes, soft-Dice loss, against the
    float64 vector-Jacobian products chained at the FP32 states of the CUDA
    evolution (the trajectory the adjoint differentiates).

    The horizon is 5 steps, not 50: where the clipped distance is flat
    (g = 0), n = g/(|g| + 1e-6) has derivative 1e6, so each step multiplies
    the gradient by up to ~1e5.  The float64 restatement measures
    max|dL/dphi0| ~ 1e19 after 5 steps, ~1e46 after 10 and ~1e80 after 50
    on a 64^3 volume of the same generator: beyond 5 steps the exact
    gradient does not fit in FP32 (the adjoint then reports
    RSF_ERR_NONFINITE), and finite differences do not converge.  Bars:
    relative L2 error of dL/dphi0 <= 1e-3; relative errors of the parameter
    gradients <= 2e-3.  A parameter gradient is a sum over all voxels of
    dL/dphi' times the step's derivative, whose terms reach ~1e19 here and
    cancel: dL/dmu of the second volume (3.9e-4) was measured 1.2e-3 from the
    float64 chain, the other parameters within 1e-3."""
    from oracle import rsf_autograd as ra
    from rsf_gb300 import Workspace, autograd

    img, phi0, mask, p = _config4_volume(seed)
    T = 5
    names = ("lambda1", "lambda2", "mu", "nu")
    ti = torch.from_numpy(img).to(cuda)
    tm = torch.from_numpy(mask).to(cuda)
    with Workspace(img.size) as ws:
        prm = {k: torch.tensor(f32(getattr(p, k)), dtype=torch.float64, requires_grad=True) for k in names}
        x = torch.from_numpy(phi0).to(cuda).requires_grad_(True)
        out = autograd.evolve(x, ti, p, T, checkpoint_every=2, workspace=ws, **prm)
        autograd.soft_dice_loss(out.double(), tm, p.eps).backward()
        ws.check()
        got = x.grad.double()
        got_p = np.array([prm[k].grad.item() for k in names])
        states = [torch.from_numpy(phi0).to(cuda)]
        for _ in range(T):
            nxt = states[-1].clone()
            ws.evolve(ti, nxt, p, 1)
            states.append(nxt)
        ws.check()
    assert torch.equal(states[-1], out.detach())
    step = ra.Step(img.shape, orc.taps(p.sigma), f32(p.dt), f32(p.eps), 0, cuda)
    img64 = ti.double()
    xT = states[-1].double().requires_grad_(True)
    autograd.soft_dice_loss(xT, tm, p.eps).backward()
    u = xT.grad
    want_p = np.zeros(4)
    for t in reversed(range(T)):
        u, gp = _fp64_vjp(step, states[t], img64, u, p, cuda)
        want_p += gp
    assert bool(torch.isfinite(got).all())
    rel = float(torch.linalg.vector_norm(got - u) / torch.linalg.vector_norm(u))
    assert rel <= 1e-3, f"dL/dphi0 relative L2 error {rel:.3g} (max|dL/dphi0| {float(u.abs().max()):.3g})"
    for i, k in enumerate(names):
        assert abs(got_p[i] - want_p[i]) <= 2e-3 * abs(want_p[i]), (k, got_p[i], want_p[i])


def test_adjoint_reports_gradient_overflow(cuda, rsflib):
    """An upstream gradient that overflows FP32 in the step's adjoint is
    reported by the workspace check instead of passing silently."""
    from rsf_gb300 import RsfError, Workspace

    img, phi0, mask, p = _config4_volume(40)
    ti = torch.from_numpy(img).to(cuda)
    phi = torch.from_numpy(phi0).to(cuda)
    u = torch.full(phi.shape, 3e38, device=cuda)
    with Workspace(img.size) as ws:
        ws.step_adjoint(ti, phi, u, p)
        with pytest.raises(RsfError, match="overflowed"):
            ws.check()
        ws.check()  # the flag is cleared once reported


BATCH_SHAPES = [(24, 26, 40), (9, 8, 10), (40, 38, 45), (2, 3, 40), (30, 33, 29)]


@pytest.mark.parametrize("sigma", [1.5, 3.0, 5.0])
def test_batched_adjoint_equals_per_volume(ws_big, sigma):
    """rsf_step_adjoint_batched over volumes of different shapes (one
    without a valid blur region, one thinner than two voxels) writes, for
    each volume, the same dL/dphi bit for bit as rsf_step_adjoint on that
    volume alone; the parameter gradients are the sum of the per-volume ones
    (double atomics in another order: relative 1e-9)."""
    gen = torch.Generator(device="cuda")
    gen.manual_seed(int(sigma * 10))
    items = []
    for shape in BATCH_SHAPES:
        img = torch.randint(0, 256, shape, generator=gen, device="cuda", dtype=torch.uint8)
        phi = (torch.rand(shape, generator=gen, device="cuda") * 6 - 3).contiguous()
        u = torch.randn(shape, generator=gen, device="cuda")
        items.append((img, phi, u, torch.empty_like(phi)))
    p = _params(sigma=sigma, lambda1=1e-4, lambda2=2e-4)
    g_b = torch.zeros(4, dtype=torch.float64, device="cuda")
    ws_big.step_adjoint_batched(items, p, param_grads=g_b)
    g_s = torch.zeros(4, dtype=torch.float64, device="cuda")
    for img, phi, u, out in items:
        single = ws_big.step_adjoint(img, phi, u, p, param_grads=g_s)
        assert torch.equal(single, out)
    ws_big.check()
    assert torch.allclose(g_b, g_s, rtol=1e-9, atol=0.0)


def test_batched_autograd_equals_per_volume(cuda, rsflib):
    """autograd.evolve on a (B, L, H, W) batch (rsf_evolve_batched forward,
    rsf_step_adjoint_batched backward) gives each volume's phi0 gradient bit
    for bit as the per-volume call, and the parameter gradients of the
    summed loss (relative 1e-9)."""
    from rsf_gb300 import Workspace, autograd

    shape, T = (20, 22, 24), 7
    cases = [smooth_case(shape, seed=s) for s in (3, 5)]
    p = _params(lambda2=0.8)
    names = ("lambda1", "lambda2", "mu", "nu")
    imgs = torch.stack([torch.from_numpy(c[0]) for c in cases]).cuda()
    phi0 = torch.stack([torch.from_numpy(c[1]) for c in cases]).cuda()
    masks = torch.stack([torch.from_numpy(c[2]) for c in cases]).cuda()
    with Workspace(phi0.numel(), 2) as ws:
        prm = {k: torch.tensor(f32(getattr(p, k)), dtype=torch.float64, requires_grad=True) for k in names}
        x = phi0.clone().requires_grad_(True)
        out = autograd.evolve(x, imgs, p, T, checkpoint_every=3, workspace=ws, **prm)
        loss = sum(autograd.soft_dice_loss(out[b].double(), masks[b], p.eps) for b in range(2))
        loss.backward()
        gb, gpb = x.grad.clone(), np.array([prm[k].grad.item() for k in names])
        gs, gps = [], np.zeros(4)
        for b in range(2):
            prm = {k: torch.tensor(f32(getattr(p, k)), dtype=torch.float64, requires_grad=True) for k in names}
            xb = phi0[b].clone().requires_grad_(True)
            ob = autograd.evolve(xb, imgs[b], p, T, checkpoint_every=3, workspace=ws, **prm)
            autograd.soft_dice_loss(ob.double(), masks[b], p.eps).backward()
            gs.append(xb.grad)
            gps += np.array([prm[k].grad.item() for k in names])
        ws.check()
    for b in range(2):
        assert torch.equal(gb[b], gs[b])
    assert np.allclose(gpb, gps, rtol=1e-9, atol=0.0)
