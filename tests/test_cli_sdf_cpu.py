"""CPU checks of the initial level set (oracle) and of the rsf3d front end.

The signed distance restated in the oracle is compared with SciPy's exact
Euclidean distance transform; the command-line tool is checked for the
reference's option handling (CUDA_RSF/main.cpp:86-110) up to the point where
it needs a device.
"""
import subprocess

import numpy as np
import pytest

from conftest import PKG

CLI = PKG / "bin" / "rsf3d"


def _scipy_sdf(seed, thr):
    from scipy import ndimage

    m = seed > thr
    if m.all() or not m.any():
        L, H, W = seed.shape
        return np.full(seed.shape, (1.0 if m.all() else -1.0) * (W + H + L), dtype=np.float32)
    return np.where(m, ndimage.distance_transform_edt(m), -ndimage.distance_transform_edt(~m)).astype(np.float32)


def _blobs(shape, seed):
    from scipy import ndimage

    rng = np.random.default_rng(seed)
    return ndimage.uniform_filter((rng.random(shape) * 30).astype(np.float32), 3)


@pytest.mark.parametrize("shape", [(9, 11, 13), (1, 1, 7), (7, 1, 1), (1, 9, 1), (6, 7, 1), (12, 10, 14), (2, 3, 33)])
def test_oracle_sdf_equals_scipy_edt(orc, shape):
    seed = _blobs(shape, sum(shape))
    thr = float(np.median(seed))
    got = orc.signed_distance(seed, thr)
    assert np.array_equal(got.view(np.uint32), _scipy_sdf(seed, thr).view(np.uint32))


def test_oracle_sdf_one_class_fill_and_threshold_strictness(orc):
    seed = np.full((4, 5, 6), 13.0, dtype=np.float32)
    # seed == threshold is outside: the reference's sdf(seed - 13) sees 0 there
    assert np.all(orc.signed_distance(seed, 13.0) == -15.0)
    assert np.all(orc.signed_distance(seed, 12.5) == 15.0)
    seed[2, 2, 3] = 20.0
    phi = orc.signed_distance(seed, 13.0)
    assert phi[2, 2, 3] == 1.0
    assert phi[0, 0, 0] == -np.float32(np.sqrt(4 + 4 + 9))


def test_oracle_sdf_is_a_distance_field(orc):
    seed = _blobs((16, 18, 20), 3)
    phi = orc.signed_distance(seed, float(np.median(seed)))
    # 1-Lipschitz along each axis between voxels of one class
    for ax in range(3):
        d = np.abs(np.diff(phi.astype(np.float64), axis=ax))
        same = np.sign(np.take(phi, range(phi.shape[ax] - 1), axis=ax)) == np.sign(
            np.take(phi, range(1, phi.shape[ax]), axis=ax))
        assert d[same].max() <= 1.0 + 1e-6
    assert np.all(np.abs(phi) >= 1.0)


def _cli():
    from rsf_gb300 import build

    build.build()
    assert CLI.exists()
    return str(CLI)


def _run(*args):
    return subprocess.run([_cli(), *args], capture_output=True, text=True, timeout=60)


def test_cli_help_lists_reference_options_and_exits_1():
    r = _run("--help")
    assert r.returncode == 1
    for name in ("sigma", "t", "dt", "meu", "e", "v", "sigma2", "binary", "image", "ouput", "debug"):
        assert f"--{name} " in r.stdout or f"--{name}\n" in r.stdout
    assert "--sigma arg (=5)" in r.stdout and "--t arg (=30)" in r.stdout and "--ouput arg (=out.npy)" in r.stdout


@pytest.mark.parametrize("args,msg", [
    (["--s", "3"], "ambiguous"),
    (["--bogus", "1"], "unrecognised"),
    (["--sigma"], "needs a value"),
    (["--debug=1"], "takes no value"),
    (["-t", "3"], "unexpected argument"),
    (["--sigma", "x3"], "malformed"),
    (["--boundary", "wrap", "--image", "a", "--binary", "b"], "--boundary"),
    (["--t", "3"], "--image and --binary are required"),
])
def test_cli_usage_errors_exit_2(args, msg):
    r = _run(*args)
    assert r.returncode == 2, r.stderr
    assert msg in r.stderr


def test_cli_prefixes_and_output_alias_parse(tmp_path):
    # unambiguous prefixes resolve (--me -> --meu, --ou -> --ouput/--output);
    # the run then stops at the missing input file, before any device work
    r = _run("--me", "1", "--ou", str(tmp_path / "o.npy"), "--bin", str(tmp_path / "none.npy"), "--ima",
             str(tmp_path / "none2.npy"))
    assert r.returncode == 3 and "cannot open" in r.stderr


def test_cli_npy_reader_rejects_bad_files_and_shape_mismatch(tmp_path):
    img = tmp_path / "img.npy"
    seed = tmp_path / "seed.npy"
    np.save(img, np.zeros((4, 5, 6), dtype=np.uint8))
    np.save(seed, np.zeros((4, 5, 7), dtype=np.float32))
    r = _run("--image", str(img), "--binary", str(seed))
    assert r.returncode == 3 and "differ in shape" in r.stderr
    np.save(seed, np.zeros((4, 5), dtype=np.float32))
    r = _run("--image", str(img), "--binary", str(seed))
    assert r.returncode == 3 and "3-D" in r.stderr
    (tmp_path / "junk.npy").write_bytes(b"not an array")
    r = _run("--image", str(img), "--binary", str(tmp_path / "junk.npy"))
    assert r.returncode == 3 and "not a .npy" in r.stderr
    np.save(seed, np.zeros((4, 5, 6), dtype=np.complex64))
    r = _run("--image", str(img), "--binary", str(seed))
    assert r.returncode == 3 and "unsupported dtype" in r.stderr


def _raw_npy(header: str, version=1, data=b""):
    hdr = header.encode("latin1")
    if version == 1:
        return b"\x93NUMPY\x01\x00" + len(hdr).to_bytes(2, "little") + hdr + data
    return b"\x93NUMPY" + bytes([version, 0]) + len(hdr).to_bytes(4, "little") + hdr + data


@pytest.mark.parametrize("raw,msg", [
    (_raw_npy("{'descr': '<f4', 'fortran_order': False, 'shape': (4, x5, 6), }\n"), "malformed shape"),
    (_raw_npy("{'descr': '<f4', 'fortran_order': False, 'shape': (3000000000, 4, 4), }\n"), "extent too large"),
    (_raw_npy("{'descr': '<f4', 'fortran_order': False, 'shape': (2147483648, 2147483648, 2), }\n"),
     "array too large"),
    (b"\x93NUMPY\x02\x00" + (1 << 21).to_bytes(4, "little"), "header too long"),
    (_raw_npy("{'descr': '<f4', 'fortran_order': False, 'shape': (2, 2, 2), }\n", data=b"\0" * 12),
     "truncated data"),
])
def test_cli_npy_reader_rejects_malformed_headers(tmp_path, raw, msg):
    img = tmp_path / "img.npy"
    np.save(img, np.zeros((2, 2, 2), dtype=np.uint8))
    bad = tmp_path / "bad.npy"
    bad.write_bytes(raw)
    r = _run("--image", str(img), "--binary", str(bad))
    assert r.returncode == 3 and msg in r.stderr, r.stderr


@pytest.mark.parametrize("image,seed", [
    (np.zeros((4, 5, 6), np.uint8), np.asfortranarray(np.zeros((4, 5, 6), np.int16))),
    (np.zeros((1, 1, 4, 5, 6), np.float64), np.zeros((4, 5, 6), np.bool_)),
    (np.asfortranarray(np.ones((4, 5, 6), np.float32)), np.zeros((1, 4, 5, 6), np.uint16)),
])
def test_cli_npy_reader_accepts_layouts_and_numeric_types(tmp_path, image, seed):
    """Fortran order, leading size-1 axes and any integer, bool or float type
    load; the run then either evolves (with a GPU) or stops at the device
    (without one), never at the files."""
    np.save(tmp_path / "img.npy", image)
    np.save(tmp_path / "seed.npy", seed)
    out = tmp_path / "phi.npy"
    r = _run("--image", str(tmp_path / "img.npy"), "--binary", str(tmp_path / "seed.npy"), "--ouput", str(out),
             "--t", "1", "--sigma", "1", "--quiet")
    assert r.returncode in (0, 3), r.stderr
    if r.returncode == 0:
        assert np.load(out).shape == (4, 5, 6)
    else:
        assert str(tmp_path) not in r.stderr and "npy" not in r.stderr, r.stderr


_NPY_DUMP = r'''
#include <cstdio>
#include "npy_io.h"
// Loads argv[1] with the rsf3d reader; writes L H W is_u8 on stdout's first
// line, then saves the C-order data as float32 .npy to argv[2].
int main(int argc, char **argv) {
    rsf::NpyVolume v;
    std::string e = rsf::npy_load(argv[1], v);
    if (!e.empty()) { std::fprintf(stderr, "%s\n", e.c_str()); return 3; }
    std::vector<float> f(v.is_u8 ? v.u8.size() : 0);
    for (size_t i = 0; i < f.size(); i++) f[i] = (float)v.u8[i];
    e = rsf::npy_save_f32(argv[2], v.is_u8 ? f.data() : v.f32.data(), v.W, v.H, v.L);
    if (!e.empty()) { std::fprintf(stderr, "%s\n", e.c_str()); return 4; }
    std::printf("%lld %lld %lld %d\n", (long long)v.L, (long long)v.H, (long long)v.W, (int)v.is_u8);
    return 0;
}
'''


@pytest.fixture(scope="module")
def npy_dump(tmp_path_factory):
    d = tmp_path_factory.mktemp("npydump")
    (d / "main.cpp").write_text(_NPY_DUMP)
    exe = d / "npy_dump"
    csrc = PKG / "csrc"
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(csrc), str(d / "main.cpp"), str(csrc / "npy_io.cpp"),
                        "-o", str(exe)], capture_output=True, text=True, timeout=120)
    if r.returncode != 0:
        pytest.skip("g++ unavailable: " + r.stderr[-200:])
    return exe


@pytest.mark.parametrize("arr", [
    np.arange(4 * 5 * 6, dtype=np.uint8).reshape(4, 5, 6),
    np.asfortranarray(np.arange(4 * 5 * 6, dtype=np.int16).reshape(4, 5, 6) - 60),
    np.asfortranarray(np.arange(3 * 7 * 2, dtype=np.uint8).reshape(3, 7, 2)),
    np.linspace(-1, 1, 2 * 3 * 4).reshape(1, 1, 2, 3, 4),
    (np.arange(60).reshape(3, 4, 5) % 3 == 0),
    np.arange(60, dtype=np.uint32).reshape(5, 4, 3) * 1000,
])
def test_npy_reader_values_match_numpy(tmp_path, npy_dump, arr):
    """The rsf3d reader returns every value in C order (x fastest), also for
    Fortran-ordered files, and squeezes leading axes of length 1."""
    src, out = tmp_path / "in.npy", tmp_path / "out.npy"
    np.save(src, arr)
    r = subprocess.run([str(npy_dump), str(src), str(out)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    want = np.ascontiguousarray(arr.reshape(arr.shape[-3:]), dtype=np.float32)
    L, H, W, is_u8 = (int(v) for v in r.stdout.split())
    assert (L, H, W) == want.shape and is_u8 == (arr.dtype == np.uint8)
    assert np.array_equal(np.load(out), want)
