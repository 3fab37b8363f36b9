"""CPU tests of the oracle: each stage against an independent NumPy
restatement of the reference's arithmetic (CUDA_RSF/kernel.cu, main.cpp)."""
import math

import numpy as np
import pytest

f32 = np.float32


def taps_numpy(sigma):
    """main.cpp:152-166 evaluated with float32 NumPy scalars."""
    p = int(f32(7.0) * f32(sigma))
    if p % 2 == 0:
        p += 1
    miu = f32(p // 2)
    u = int(f32(2.0) * f32(sigma) * f32(sigma))
    s = np.sqrt(f32(u) * f32(math.pi), dtype=f32)
    out = []
    for xi in range(p):
        d = f32(xi) - miu
        a = (-d * d) / f32(u)
        out.append((f32(1.0) / s) * f32(math.exp(float(a))))
    return np.array(out, dtype=f32)


@pytest.mark.parametrize("sigma,k", [(1.0, 7), (1.5, 11), (2.5, 17), (3.0, 21), (4.0, 29), (5.0, 35), (7.3, 51)])
def test_taps_match_main_cpp_formula(orc, sigma, k):
    g = orc.taps(sigma)
    assert len(g) == k
    assert np.array_equal(g, taps_numpy(sigma))
    assert np.allclose(g, g[::-1])  # symmetric
    assert 0.99 < float(g.sum()) < 1.001  # unnormalised, but close to 1


def test_taps_reject_tiny_sigma(orc):
    with pytest.raises(ValueError):
        orc.taps(0.5)  # (int)(2 sigma^2) == 0


def test_atan_accuracy(orc):
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-2, 2, 20000), rng.uniform(-1e4, 1e4, 20000), 10.0 ** rng.uniform(-30, 30, 5000),
                        -(10.0 ** rng.uniform(-30, 30, 5000)), [0.0, 1.0, -1.0, 1e38, -1e38]]).astype(f32)
    a = orc.atan(x)
    ref = np.arctan(x.astype(np.float64))
    ulp = np.abs(a.astype(np.float64) - ref) / np.spacing(np.abs(ref).astype(f32).clip(1e-38))
    assert float(ulp.max()) <= 1.4
    assert orc.atan(np.array([np.inf], dtype=f32))[0] == f32(math.pi / 2)


def _ulps(a, b):
    a = np.asarray(a, dtype=f32).view(np.int32).astype(np.int64)
    b = np.asarray(b, dtype=f32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


@pytest.mark.parametrize("eps", [0.2, 1.0])
def test_heaviside_and_dirac_portable_close_to_reference_double(orc, eps):
    rng = np.random.default_rng(1)
    phi = np.concatenate([rng.uniform(-3, 3, 20000), rng.uniform(-1e4, 1e4, 20000)]).astype(f32)
    # kernel.cu:259: float division, atan, double arithmetic (correctly rounded atan here)
    q = phi / f32(eps)
    a = np.arctan(q.astype(np.float64)).astype(f32).astype(np.float64)
    h_ref = (0.5 * (1.0 + (2.0 / math.pi) * a)).astype(f32)
    # 1 + (2/pi) atan cancels for large |phi/eps|, so H inherits the absolute
    # error of atan near +-pi/2 (0.5 * (2/pi) * 1.35 ulp(pi/2) plus rounding):
    # bounded in absolute terms, not in ulps of H.  The same holds for the
    # reference's own single-precision atan.
    assert float(np.abs(orc.heaviside(phi, eps, 0).astype(np.float64) - h_ref).max()) <= 1.2e-7
    assert int(_ulps(orc.heaviside(phi, eps, 1), h_ref).max()) <= 1
    # kernel.cu:276: float quotient with fma(phi, phi, eps*eps), then (1/pi) in double
    e2 = f32(eps) * f32(eps)
    den = (phi.astype(np.float64) * phi.astype(np.float64) + np.float64(e2)).astype(f32)  # fma(phi, phi, e2)
    dq = f32(eps) / den  # float division
    d_ref = ((1.0 / math.pi) * dq.astype(np.float64)).astype(f32)
    assert int(_ulps(orc.dirac(phi, eps, 0), d_ref).max()) <= 1
    assert int(_ulps(orc.dirac(phi, eps, 1), d_ref).max()) <= 1


def gradient_numpy(f):
    """kernel.cu:57-125: central differences, one-sided at the faces, x = 0
    reading the previous linear element (voxel 0 reads itself)."""
    L, H, W = f.shape
    flat = f.ravel()
    d = f.astype(np.float64)
    gx = np.empty_like(d)
    gx[:, :, 1:W - 1] = (d[:, :, 2:] - d[:, :, :-2]) / 2
    gx[:, :, W - 1] = (d[:, :, W - 1] - d[:, :, W - 2]) / 2
    idx = np.arange(f.size).reshape(f.shape)[:, :, 0].ravel()
    left = flat[np.maximum(idx - 1, 0)].astype(np.float64)
    gx[:, :, 0] = ((flat[idx + 1].astype(np.float64) - left) / 2).reshape(L, H)
    gy = np.empty_like(d)
    gy[:, 1:H - 1] = (d[:, 2:] - d[:, :-2]) / 2
    gy[:, 0] = (d[:, 1] - d[:, 0]) / 2
    gy[:, H - 1] = (d[:, H - 1] - d[:, H - 2]) / 2
    gz = np.empty_like(d)
    gz[1:L - 1] = (d[2:] - d[:-2]) / 2
    gz[0] = (d[1] - d[0]) / 2
    gz[L - 1] = (d[L - 1] - d[L - 2]) / 2
    return np.stack([gx, gy, gz]).astype(f32)


@pytest.mark.parametrize("shape", [(7, 6, 9), (2, 3, 2), (5, 11, 4)])
def test_gradient_boundary_rules(orc, shape):
    f = np.random.default_rng(2).normal(size=shape).astype(f32)
    assert np.array_equal(orc.gradient(f, boundary=0), gradient_numpy(f))
    g_clamp = orc.gradient(f, boundary=1)
    want = gradient_numpy(f)
    want[0][:, :, 0] = ((f[:, :, 1].astype(np.float64) - f[:, :, 0]) / 2).astype(f32)
    assert np.array_equal(g_clamp, want)


def blur_numpy(field, sigma):
    """kernel.cu:1000-1121 + 300-362 in float64: valid correlation along x,
    y, z with the unnormalised taps, embedded with border value 30."""
    g = taps_numpy(sigma).astype(np.float64)
    k = len(g)
    r = (k - 1) // 2
    L, H, W = field.shape
    out = np.full(field.shape, 30.0)
    if min(L, H, W) < k:
        return out
    a = field.astype(np.float64)
    ax = sum(g[t] * a[:, :, t:W - k + 1 + t] for t in range(k))
    ay = sum(g[t] * ax[:, t:H - k + 1 + t, :] for t in range(k))
    az = sum(g[t] * ay[t:L - k + 1 + t] for t in range(k))
    out[r:L - r, r:H - r, r:W - r] = az
    return out


@pytest.mark.parametrize("sigma,shape", [(1.5, (20, 23, 26)), (3.0, (30, 25, 40)), (3.0, (9, 40, 40))])
def test_blur_padded_matches_float64(orc, sigma, shape):
    f = np.random.default_rng(3).uniform(0, 255, size=shape).astype(f32)
    got = orc.blur_padded(f, sigma)
    want = blur_numpy(f, sigma)
    assert np.allclose(got, want, rtol=2e-6, atol=1e-4)
    border = want == 30.0
    assert np.array_equal(got[border], want[border].astype(f32))


def step_numpy(phi, img, sigma, eps, lam, mu, nu, dt):
    """One iteration of main.cpp:233-300 in float64."""
    phi = phi.astype(np.float64)
    I = img.astype(np.float64)
    H = 0.5 * (1 + (2 / math.pi) * np.arctan(phi / eps))
    g = gradient_numpy(phi.astype(f32)).astype(np.float64)
    mag = np.sqrt((g ** 2).sum(0))
    n = g / (mag + 1e-6)
    kap = sum(gradient_numpy(n[a].astype(f32))[a].astype(np.float64) for a in range(3))
    lap = sum(gradient_numpy(g[a].astype(f32))[a].astype(np.float64) for a in range(3))
    fo = blur_numpy(I * H, sigma) / blur_numpy(H, sigma)
    fi = blur_numpy(I * (1 - H), sigma) / blur_numpy(1 - H, sigma)
    eo, ei = (I - fo) ** 2, (I - fi) ** 2
    dh = (1 / math.pi) * eps / (eps ** 2 + phi ** 2)
    return phi - dh * lam * (eo - ei) * dt + nu * dt * dh * kap + mu * dt * (lap - kap)


def test_step_matches_float64_restatement(orc):
    from rsf_gb300 import synth

    img, phi0, _ = synth.make_small((26, 28, 30), n_tubes=4, seed=4)
    p = orc.params(sigma=2.0, eps=1.0, lambda1=1.0, mu=1.0, nu=65.025, dt=0.1)
    got = orc.step(phi0, img.astype(f32), p)
    want = step_numpy(phi0, img, 2.0, 1.0, 1.0, 1.0, 65.025, 0.1)
    scale = float(np.abs(want).max())
    # one iteration: the float32 path stays within 1e-5 of the float64 restatement
    assert float(np.abs(got - want).max()) <= 1e-5 * scale
    assert float((np.sign(got) == np.sign(want)).mean()) == 1.0


def test_f32_oracle_close_to_f64_twin(orc):
    from rsf_gb300 import synth

    img, phi0, _ = synth.make_small((32, 34, 36), n_tubes=4, seed=5)
    p = orc.params(sigma=2.0, eps=1.0, lambda1=1.0, mu=1.0, nu=65.025, dt=0.1)
    a = orc.evolve(phi0, img.astype(f32), p, 5)
    b = orc.evolve_f64(phi0, img.astype(f32), p, 5)
    assert float((np.sign(a) == np.sign(b)).mean()) >= 0.9999


def test_oracle_thread_count_invariant(orc):
    from rsf_gb300 import synth

    img, phi0, _ = synth.make_small((24, 26, 28), n_tubes=3, seed=6)
    p = orc.params(sigma=1.5, eps=0.2)
    a = orc.evolve(phi0, img.astype(f32), p, 3, threads=1)
    b = orc.evolve(phi0, img.astype(f32), p, 3, threads=4)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_lambda_split_reduces_to_single_e(orc):
    """lambda1 == lambda2 takes the reference's e*(Eout-Ein) form."""
    from rsf_gb300 import synth

    img, phi0, _ = synth.make_small((20, 22, 24), n_tubes=3, seed=7)
    a = orc.step(phi0, img.astype(f32), orc.params(sigma=1.5, lambda1=0.5, lambda2=0.5))
    b = orc.step(phi0, img.astype(f32), orc.params(sigma=1.5, lambda1=0.5, lambda2=0.5000001))
    assert float(np.abs(a - b).max()) < 1e-2 * float(np.abs(a).max())


def test_volume_smaller_than_kernel_is_all_border(orc):
    f = np.random.default_rng(8).uniform(0, 1, (9, 10, 11)).astype(f32)
    assert np.all(orc.blur_padded(f, 3.0) == 30.0)


def test_gaussian_data_term_matches_its_formula(orc):
    """The oracle's expanded Gaussian data term (data_term = 1) against the
    formula evaluated independently with NumPy in float64 from the oracle's
    own fits: e = I^2 K*1 - 2 I K*f + K*f^2 on the valid region, (I - 1)^2 on
    the border band; FP32 against FP64 within 1e-5 of max|e|."""
    from rsf_gb300 import synth

    img, phi0, _ = synth.make_small((26, 28, 30), n_tubes=3, seed=5)
    I = img.astype(np.float32)
    p = orc.params(sigma=1.5, eps=1.0, lambda1=1.0, mu=1.0, nu=65.025, dt=0.1, data_term=1)
    _, fields = orc.step(phi0, I, p, debug=True)
    fo, fi, eo, ei = (fields[j].astype(np.float64) for j in range(4))
    g = orc.taps(1.5).astype(np.float64)
    k, r = len(g), (len(g) - 1) // 2

    def blur_valid(f):
        out = f
        for axis in (2, 1, 0):
            n = out.shape[axis] - k + 1
            out = sum(g[t] * np.take(out, np.arange(t, t + n), axis=axis) for t in range(k))
        return out

    s3 = float(np.sum(g)) ** 3
    sl = tuple(slice(r, n - r) for n in I.shape)
    Iv = I.astype(np.float64)[sl]
    for f, e in ((fo, eo), (fi, ei)):
        want = Iv * Iv * s3 - 2.0 * Iv * blur_valid(f) + blur_valid(f * f)
        assert np.abs(e[sl] - want).max() <= 1e-5 * np.abs(want).max()
        border = np.ones(I.shape, bool)
        border[sl] = False
        assert np.array_equal(e[border], ((I.astype(np.float64) - 1.0) ** 2)[border])
    # the two data terms give different evolutions
    p0 = orc.params(sigma=1.5, eps=1.0, lambda1=1.0, mu=1.0, nu=65.025, dt=0.1, data_term=0)
    assert not np.array_equal(orc.evolve(phi0, I, p0, 1), orc.evolve(phi0, I, p, 1))


def test_gaussian_data_term_fp32_tracks_fp64(orc):
    from rsf_gb300 import synth

    img, phi0, _ = synth.make_small((30, 32, 34), n_tubes=3, seed=6)
    I = img.astype(np.float32)
    p = orc.params(sigma=3.0, eps=1.0, lambda1=1.0, lambda2=0.5, mu=1.0, nu=65.025, dt=0.1, data_term=1)
    a = orc.evolve(phi0, I, p, 2)
    b = orc.evolve_f64(phi0.astype(np.float64), I, p, 2)
    assert float(np.abs(a - b).max()) <= 1e-4 * float(np.abs(b).max())
    assert float((np.sign(a) == np.sign(b)).mean()) >= 0.9999
