"""GPU parity: the CUDA path against the CPU oracle, through the C ABI.

The portable arithmetic of the CUDA kernels performs the oracle's exact IEEE
operation sequence, so the bar is bit equality of every voxel (tolerance 0),
which also meets max|dphi| <= 1e-4 max|phi| and >= 99.99% sign agreement.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(shape, seed, dtype="u8", n_tubes=3):
    from rsf_gb300 import synth

    img, phi0, mask = synth.make_small(shape, n_tubes=n_tubes, r_min=1.5, r_max=3.5, seed=seed)
    if phi0.min() >= 0 or phi0.max() <= 0:
        # too thin for a tube to survive the perturbation: use a random contour
        phi0 = np.random.default_rng(seed).uniform(-3.0, 3.0, size=shape).astype(np.float32)
    if dtype == "f32":
        img = img.astype(np.float32)
    return img, phi0, mask


def _oracle_params(orc, p):
    return orc.params(sigma=p.sigma, dt=p.dt, mu=p.mu, lambda1=p.lambda1, lambda2=p.lambda2, nu=p.nu, eps=p.eps,
                      sigma2=p.sigma2, boundary=0 if p.boundary == "reference" else 1)


def _bits_equal(a, b):
    return np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))


def _diff_report(got, want):
    d = np.abs(got.astype(np.float64) - want)
    return (f"{int((got != want).sum())} voxels differ, max|d|={d.max():.3g}, "
            f"first at {np.unravel_index(int(np.argmax(got != want)), got.shape)}")


CASES = [
    # shape (L, H, W), sigma, eps, lambda1, lambda2, boundary, dtype, iters
    ((20, 26, 30), 1.5, 1.0, 1.0, 1.0, "reference", "u8", 3),      # k = 11, generic-k kernels
    ((40, 44, 48), 3.0, 0.2, 1.0, 1.0, "reference", "u8", 2),      # k = 21 specialisation
    ((40, 36, 50), 3.0, 1.0, 1.0, 2.0, "clamp", "f32", 2),         # lambda1 != lambda2, clamp rule
    ((64, 40, 38), 5.0, 0.2, 0.1, 0.1, "reference", "u8", 2),      # k = 35, reference defaults
    ((33, 45, 37), 4.0, 0.2, 1.0, 1.0, "reference", "u8", 2),      # k = 29 (even floor(7 sigma))
    ((9, 12, 10), 3.0, 0.2, 1.0, 1.0, "reference", "u8", 3),       # smaller than the kernel: all border
    ((17, 2, 5), 1.0, 0.2, 1.0, 1.0, "reference", "f32", 4),       # two-voxel extent
    ((3, 70, 2), 1.0, 0.2, 1.0, 1.0, "clamp", "u8", 2),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}-s{c[1]}-e{c[2]}-{c[5]}-{c[6]}")
def test_evolve_bit_exact(case, orc, ws_big, cuda):
    import torch
    from rsf_gb300 import Params

    shape, sigma, eps, l1, l2, boundary, dtype, iters = case
    img, phi0, _ = _inputs(shape, seed=hash(shape) % 1000, dtype=dtype)
    p = Params(sigma=sigma, dt=0.1, mu=1.0, lambda1=l1, lambda2=l2, nu=65.025, eps=eps, boundary=boundary)
    ti = torch.from_numpy(img).to(cuda)
    tp = torch.from_numpy(phi0).to(cuda)
    ws_big.evolve(ti, tp, p, iters)
    ws_big.check()
    got = tp.cpu().numpy()
    want = orc.evolve(phi0, img.astype(np.float32), _oracle_params(orc, p), iters)
    assert _bits_equal(got, want), _diff_report(got, want)


@pytest.mark.parametrize("sigma,boundary", [(3.0, "reference"), (1.5, "clamp"), (5.0, "reference")])
def test_debug_fields_bit_exact(sigma, boundary, orc, ws_big, cuda):
    import torch
    from rsf_gb300 import Params

    img, phi0, _ = _inputs((44, 41, 47), seed=3)
    p = Params(sigma=sigma, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=0.2, boundary=boundary)
    out, fields = ws_big.step_debug(torch.from_numpy(img).to(cuda), torch.from_numpy(phi0).to(cuda), p)
    torch.cuda.synchronize()
    want_out, want_fields = orc.step(phi0, img.astype(np.float32), _oracle_params(orc, p), debug=True)
    names = ["f_out", "f_in", "e_out", "e_in", "delta", "kappa", "laplacian", "|grad|"]
    got_fields = fields.cpu().numpy()
    for i, n in enumerate(names):
        assert _bits_equal(got_fields[i], want_fields[i]), f"{n}: {_diff_report(got_fields[i], want_fields[i])}"
    assert _bits_equal(out.cpu().numpy(), want_out)


BOX_CASES = [
    # shape, sigma, sigma2, lambda1, lambda2, dtype, iters
    ((20, 26, 30), 1.5, 1.0, 1.0, 1.0, "u8", 2),
    ((24, 22, 28), 3.0, 2.5, 1.0, 0.5, "f32", 2),    # (int)sigma2 = 2, lambda1 != lambda2
    ((9, 12, 10), 3.0, 1.0, 1.0, 1.0, "u8", 2),      # no valid blur region: f = 1 everywhere
    ((30, 31, 33), 5.0, 1.0, 0.1, 0.1, "u8", 1),     # k = 35
]


@pytest.mark.parametrize("case", BOX_CASES, ids=lambda c: f"{c[0]}-s{c[1]}-box{c[2]}")
def test_box_e_term_bit_exact(case, orc, ws_big, cuda):
    """sigma2 >= 1: e = box sum of w (I_n - f(c))^2 (kernel.cu:25-55)."""
    import torch
    from rsf_gb300 import Params

    shape, sigma, sigma2, l1, l2, dtype, iters = case
    img, phi0, _ = _inputs(shape, seed=7, dtype=dtype)
    p = Params(sigma=sigma, dt=0.1, mu=1.0, lambda1=l1, lambda2=l2, nu=65.025, eps=1.0, sigma2=sigma2)
    tp = torch.from_numpy(phi0).to(cuda)
    ws_big.evolve(torch.from_numpy(img).to(cuda), tp, p, iters)
    ws_big.check()
    got = tp.cpu().numpy()
    want = orc.evolve(phi0, img.astype(np.float32), _oracle_params(orc, p), iters)
    assert _bits_equal(got, want), _diff_report(got, want)
    out, fields = ws_big.step_debug(torch.from_numpy(img).to(cuda), torch.from_numpy(phi0).to(cuda), p)
    want_out, want_fields = orc.step(phi0, img.astype(np.float32), _oracle_params(orc, p), debug=True)
    got_fields = fields.cpu().numpy()
    for i, n in enumerate(["f_out", "f_in", "e_out", "e_in"]):
        assert _bits_equal(got_fields[i], want_fields[i]), f"{n}: {_diff_report(got_fields[i], want_fields[i])}"
    assert _bits_equal(out.cpu().numpy(), want_out)


def test_box_radius_limit(ws_big, cuda):
    import torch
    from rsf_gb300 import Params, RsfError

    img, phi0, _ = _inputs((12, 12, 12), seed=1)
    with pytest.raises(RsfError):
        ws_big.evolve(torch.from_numpy(img).to(cuda), torch.from_numpy(phi0).to(cuda),
                      Params(sigma=1.0, sigma2=9.0), 1)


def test_batched_matches_plain(ws_big, cuda):
    import torch
    from rsf_gb300 import Params

    shapes = [(30, 40, 50), (64, 33, 29), (25, 25, 25), (12, 70, 41), (9, 9, 9)]
    p = Params(sigma=3.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)
    pairs, plain = [], []
    for i, s in enumerate(shapes):
        img, phi0, _ = _inputs(s, seed=10 + i)
        ti = torch.from_numpy(img).to(cuda)
        pairs.append((ti, torch.from_numpy(phi0).to(cuda)))
        tp = torch.from_numpy(phi0).to(cuda)
        ws_big.evolve(ti, tp, p, 5)
        plain.append(tp)
    ws_big.evolve_batched(pairs, p, 5)
    ws_big.check()
    for (_, b), a in zip(pairs, plain):
        assert torch.equal(a, b)


@pytest.mark.parametrize("sigma2", [1.0, 2.0])
def test_batched_box_e_term_matches_plain_and_oracle(sigma2, orc, ws_big, cuda):
    """Batches with the box e-term, including a thin sub-volume (4 valid x
    columns) before a larger one and an all-border one: each sub-volume's
    scratch holds its fits and the data factor of every voxel without
    reaching into the next sub-volume's."""
    import torch
    from rsf_gb300 import Params

    shapes = [(64, 64, 24), (9, 9, 9), (40, 44, 48), (64, 64, 64)]
    p = Params(sigma=3.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=0.5, nu=65.025, eps=1.0, sigma2=sigma2)
    iters = 2
    inputs, pairs, plain = [], [], []
    for i, s in enumerate(shapes):
        img, phi0, _ = _inputs(s, seed=20 + i)
        inputs.append((img, phi0))
        ti = torch.from_numpy(img).to(cuda)
        pairs.append((ti, torch.from_numpy(phi0).to(cuda)))
        tp = torch.from_numpy(phi0).to(cuda)
        ws_big.evolve(ti, tp, p, iters)
        plain.append(tp)
    ws_big.evolve_batched(pairs, p, iters)
    ws_big.check()
    for (img, phi0), (_, b), a in zip(inputs, pairs, plain):
        got = b.cpu().numpy()
        assert _bits_equal(got, a.cpu().numpy()), f"shape {img.shape}: batched differs from plain"
        want = orc.evolve(phi0, img.astype(np.float32), _oracle_params(orc, p), iters)
        assert _bits_equal(got, want), f"shape {img.shape}: {_diff_report(got, want)}"


@pytest.mark.parametrize("eps", [1.0, 0.2])
def test_config0_full_evolution_bit_exact(eps, orc, ws_big, cuda):
    """128^3 volume, 12 tubes, sigma 3, lambda 1, mu 1, nu 0.001*255^2, dt 0.1, 100 iterations."""
    import torch
    from rsf_gb300 import Params, synth

    img, phi0, mask = synth.make_volume(synth.CONFIG0)
    p = Params(sigma=3.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=0.001 * 255 ** 2, eps=eps)
    tp = torch.from_numpy(phi0).to(cuda)
    ws_big.evolve(torch.from_numpy(img).to(cuda), tp, p, 100)
    ws_big.check()
    got = tp.cpu().numpy()
    want = orc.evolve(phi0, img.astype(np.float32), _oracle_params(orc, p), 100)
    maxphi = float(np.abs(want).max())
    assert float(np.abs(got - want).max()) <= 1e-4 * maxphi
    assert float((np.sign(got) == np.sign(want)).mean()) >= 0.9999
    assert _bits_equal(got, want), _diff_report(got, want)


def test_reference_arith_close_to_portable(ws_big, cuda):
    """RSF_ARITH_REFERENCE (CUDA atanf, double spots) differs from the portable
    definition by at most a few ulp per stage after one iteration."""
    import torch
    from rsf_gb300 import Params

    img, phi0, _ = _inputs((40, 44, 48), seed=5)
    ti = torch.from_numpy(img).to(cuda)
    outs = []
    for arith in ("portable", "reference"):
        p = Params(sigma=3.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=0.2, arith=arith)
        tp = torch.from_numpy(phi0).to(cuda)
        ws_big.evolve(ti, tp, p, 1)
        outs.append(tp.cpu().numpy())
    a, b = outs
    assert float((np.sign(a) == np.sign(b)).mean()) >= 0.9999
    assert float(np.abs(a - b).max()) <= 1e-3 * float(np.abs(a).max())


def test_python_api_rejects_mismatched_shapes(ws_big, cuda):
    """The C ABI reads the image with phi's extents, so the Python face checks
    the shapes before any launch."""
    import torch
    from rsf_gb300 import Params

    p = Params(sigma=1.0)
    phi = torch.zeros((10, 12, 14), device=cuda)
    small = torch.zeros((10, 12, 13), dtype=torch.uint8, device=cuda)
    with pytest.raises(ValueError):
        ws_big.evolve(small, phi, p, 1)
    with pytest.raises(ValueError):
        ws_big.evolve_batched([(small, phi)], p, 1)
    with pytest.raises(ValueError):
        ws_big.step_adjoint(small, phi, phi.clone(), p)
    with pytest.raises(TypeError):
        ws_big.evolve(torch.zeros_like(phi, dtype=torch.uint8), phi.double(), p, 1)


def test_copy_async_between_pinned_host_and_device(cuda, rsflib):
    import torch
    from rsf_gb300 import RsfError, copy_async

    src = torch.randint(0, 256, (1 << 20,), dtype=torch.uint8).pin_memory()
    dev = torch.empty(1 << 20, dtype=torch.uint8, device=cuda)
    copy_async(dev, src)
    back = torch.empty_like(src).pin_memory()
    copy_async(back, dev)
    torch.cuda.synchronize()
    assert torch.equal(back, src)
    # unaligned ranges and odd sizes take the byte path
    d2 = torch.zeros(1000, dtype=torch.uint8, device=cuda)
    copy_async(d2[3:1000], src[5:1002])
    torch.cuda.synchronize()
    assert torch.equal(d2[3:].cpu(), src[5:1002])
    with pytest.raises(RsfError):
        copy_async(dev, torch.empty(1 << 20, dtype=torch.uint8))  # pageable host memory


def test_evolve_host_pinned_and_pageable_agree(orc, ws_big, cuda):
    import torch
    from rsf_gb300 import Params

    img, phi0, _ = _inputs((20, 24, 28), seed=9)
    p = Params(sigma=1.5, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)
    a = ws_big.evolve_host(img.copy(), phi0.copy(), p, 3)
    ti = torch.from_numpy(img).pin_memory()
    tp = torch.from_numpy(phi0.copy()).pin_memory()
    ws_big.evolve_host_ptr(ti.data_ptr(), "uint8", tp.data_ptr(), phi0.shape, p, 3)
    want = orc.evolve(phi0, img.astype(np.float32), _oracle_params(orc, p), 3)
    assert _bits_equal(a, want) and _bits_equal(tp.numpy(), want)


@pytest.mark.parametrize("sigma", [3.0, 5.0])
def test_tma_z_pass_bit_exact(sigma, orc, ws_big, cuda, monkeypatch):
    """The z-pass fed by TMA tile loads (selected with RSF_ZPASS=tma, 21 and
    35 taps) against the oracle and against the default streaming z-pass, on
    a batch with a thin and an all-border sub-volume and on an image of
    float32."""
    import torch
    from rsf_gb300 import Params

    shapes = [(40, 44, 48), (30, 33, 70), (9, 9, 9), (64, 38, 52)]
    p = Params(sigma=sigma, dt=0.1, mu=1.0, lambda1=1.0, lambda2=0.5, nu=65.025, eps=1.0)
    for dtype in ("u8", "f32"):
        inputs = [_inputs(s, seed=30 + i, dtype=dtype)[:2] for i, s in enumerate(shapes)]
        outs = {}
        for mode in ("tma", "stream"):
            monkeypatch.setenv("RSF_ZPASS", mode)
            pairs = [(torch.from_numpy(img).to(cuda), torch.from_numpy(phi0).to(cuda)) for img, phi0 in inputs]
            ws_big.evolve_batched(pairs, p, 3)
            ws_big.check()
            outs[mode] = [b.cpu().numpy() for _, b in pairs]
        monkeypatch.delenv("RSF_ZPASS")
        for (img, phi0), a, b in zip(inputs, outs["tma"], outs["stream"]):
            assert _bits_equal(a, b), f"{img.shape} {dtype}: TMA and streaming z-pass differ"
            want = orc.evolve(phi0, img.astype(np.float32), _oracle_params(orc, p), 3)
            assert _bits_equal(a, want), f"{img.shape} {dtype}: {_diff_report(a, want)}"


GAUSS_CASES = [
    # shape, sigma, lambda1, lambda2, dtype, iters
    ((26, 28, 30), 1.5, 1.0, 1.0, "u8", 3),      # k = 11
    ((40, 44, 48), 3.0, 1.0, 0.5, "f32", 2),     # k = 21, lambda1 != lambda2
    ((9, 12, 10), 3.0, 1.0, 1.0, "u8", 2),       # no valid blur region: border form only
]


def _gauss_oracle_params(orc, p):
    return orc.params(sigma=p.sigma, dt=p.dt, mu=p.mu, lambda1=p.lambda1, lambda2=p.lambda2, nu=p.nu, eps=p.eps,
                      data_term=1)


@pytest.mark.parametrize("case", GAUSS_CASES, ids=lambda c: f"{c[0]}-s{c[1]}-{c[4]}")
def test_gaussian_data_term_bit_exact(case, orc, ws_big, cuda):
    """The expanded Gaussian data term (data_term = "gaussian"): evolution,
    one step's e_out / e_in fields and a batch of all three shapes against the
    oracle's FP32 restatement, bit for bit.  The mode has no counterpart in
    the reference, so its parity is pinned to the oracle only."""
    import torch
    from rsf_gb300 import Params

    shape, sigma, l1, l2, dtype, iters = case
    img, phi0, _ = _inputs(shape, seed=41, dtype=dtype)
    p = Params(sigma=sigma, dt=0.1, mu=1.0, lambda1=l1, lambda2=l2, nu=65.025, eps=1.0, data_term="gaussian")
    tp = torch.from_numpy(phi0).to(cuda)
    ws_big.evolve(torch.from_numpy(img).to(cuda), tp, p, iters)
    ws_big.check()
    got = tp.cpu().numpy()
    want = orc.evolve(phi0, img.astype(np.float32), _gauss_oracle_params(orc, p), iters)
    assert _bits_equal(got, want), _diff_report(got, want)
    out, fields = ws_big.step_debug(torch.from_numpy(img).to(cuda), torch.from_numpy(phi0).to(cuda), p)
    want_out, want_fields = orc.step(phi0, img.astype(np.float32), _gauss_oracle_params(orc, p), debug=True)
    got_fields = fields.cpu().numpy()
    for i, n in enumerate(["f_out", "f_in", "e_out", "e_in"]):
        assert _bits_equal(got_fields[i], want_fields[i]), f"{n}: {_diff_report(got_fields[i], want_fields[i])}"
    assert _bits_equal(out.cpu().numpy(), want_out)


def test_gaussian_data_term_batched_and_rejections(orc, ws_big, cuda):
    import torch
    from rsf_gb300 import Params, RsfError

    shapes = [(26, 28, 30), (9, 12, 10), (40, 44, 48)]
    p = Params(sigma=3.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0, data_term="gaussian")
    inputs = [_inputs(s, seed=50 + i)[:2] for i, s in enumerate(shapes)]
    pairs = [(torch.from_numpy(img).to(cuda), torch.from_numpy(phi0).to(cuda)) for img, phi0 in inputs]
    ws_big.evolve_batched(pairs, p, 2)
    ws_big.check()
    for (img, phi0), (_, b) in zip(inputs, pairs):
        want = orc.evolve(phi0, img.astype(np.float32), _gauss_oracle_params(orc, p), 2)
        assert _bits_equal(b.cpu().numpy(), want), f"{img.shape}: {_diff_report(b.cpu().numpy(), want)}"
    img, phi0 = inputs[0]
    ti, tp = torch.from_numpy(img).to(cuda), torch.from_numpy(phi0).to(cuda)
    with pytest.raises(RsfError, match="sigma2"):
        ws_big.evolve(ti, tp, Params(sigma=3.0, sigma2=1.0, data_term="gaussian"), 1)
    with pytest.raises(RsfError, match="Gaussian data term"):
        ws_big.step_adjoint(ti.float(), tp, tp.clone(), p)


def test_launch_shapes_are_bit_identical_and_autotuned(ws_big, cuda):
    """Every kernel launch shape (x-pass lane width, stencil planes per
    block, TMA or streaming z-pass) gives the same bits; the launch-shape
    autotuner measures them on a batch and leaves the fastest set."""
    import torch
    from rsf_gb300 import Params, RsfError, autotune

    shapes = [(40, 44, 48), (64, 33, 70), (9, 9, 9)]
    p = Params(sigma=3.0, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)
    inputs = [_inputs(s, seed=60 + i)[:2] for i, s in enumerate(shapes)]
    ref = None
    try:
        for shape in autotune.LAUNCH_CANDIDATES:
            ws_big.set_launch_shape(*shape)
            pairs = [(torch.from_numpy(img).to(cuda), torch.from_numpy(phi0).to(cuda)) for img, phi0 in inputs]
            ws_big.evolve_batched(pairs, p, 3)
            ws_big.check()
            out = [b.cpu().numpy() for _, b in pairs]
            if ref is None:
                ref = out
            for a, b in zip(out, ref):
                assert _bits_equal(a, b), f"launch shape {shape} changes the result"
        with pytest.raises(RsfError):
            ws_big.set_launch_shape(7, 0, -1)
        pairs = [(torch.from_numpy(img).to(cuda), torch.from_numpy(phi0).to(cuda)) for img, phi0 in inputs]
        best = autotune.tune_launch_shape(ws_big, pairs, p, iters=2)
        assert (best.xpass_width, best.stencil_planes, best.z_tma) in autotune.LAUNCH_CANDIDATES
        assert best.ms_per_iteration == min(ms for _, ms in best.table)
        for (_, b), (_, phi0) in zip(pairs, inputs):  # phi restored after the measurements
            assert torch.equal(b.cpu(), torch.from_numpy(phi0))
    finally:
        ws_big.set_launch_shape(0, 0, -1)
