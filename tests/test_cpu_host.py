"""CPU tests: the C ABI library loads and exports every declared symbol, its
host-side helpers, the tiler, the synthetic generator and the multi-process
helpers (gloo, world size 2).  No device work."""
import ctypes
import os
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "rsf.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rsf_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(rsflib):
    syms = declared_symbols()
    assert "rsf_evolve" in syms and "rsf_evolve_batched" in syms and "rsf_status_string" in syms
    missing = [s for s in syms if not hasattr(rsflib, s)]
    assert not missing, missing


def test_abi_version_and_status_strings(rsflib):
    assert rsflib.rsf_abi_version() == 1
    for code in range(11):
        s = rsflib.rsf_status_string(code)
        assert s and s != b"unknown status"
    assert rsflib.rsf_status_string(99) == b"unknown status"


def test_params_default_are_reference_cli_defaults(rsflib):
    from rsf_gb300._lib import RsfParams

    p = RsfParams()
    assert rsflib.rsf_params_default(ctypes.byref(p)) == 0
    # CUDA_RSF/main.cpp:91-97 and kernel.cu:258
    vals = (p.sigma, p.dt, p.mu, p.lambda1, p.lambda2, p.nu, p.eps, p.sigma2)
    want = (5.0, 0.1, 1.0, 0.1, 0.1, 0.0001, 0.2, 0.0)
    assert np.allclose(vals, want) and p.boundary == 0 and p.arith == 0


@pytest.mark.parametrize("sigma", [0.75, 1.0, 2.5, 3.0, 4.0, 5.0, 10.0])
def test_taps_identical_to_oracle(rsflib, orc, sigma):
    from rsf_gb300 import gaussian_taps

    assert np.array_equal(gaussian_taps(sigma), orc.taps(sigma))


def test_taps_errors(rsflib):
    k = ctypes.c_int()
    assert rsflib.rsf_gaussian_taps(ctypes.c_float(0.0), None, 0, ctypes.byref(k)) == 1
    assert rsflib.rsf_gaussian_taps(ctypes.c_float(0.6), None, 0, ctypes.byref(k)) == 1
    assert rsflib.rsf_gaussian_taps(ctypes.c_float(40.0), None, 0, ctypes.byref(k)) == 4
    buf = (ctypes.c_float * 4)()
    assert rsflib.rsf_gaussian_taps(ctypes.c_float(3.0), buf, 4, ctypes.byref(k)) == 1
    assert b"too small" in rsflib.rsf_last_error()


def test_workspace_bytes_formula(rsflib):
    b = rsflib.rsf_workspace_bytes_for(1000, 2)
    assert b >= 1000 * 36


def test_null_arguments_are_rejected_without_device(rsflib):
    from rsf_gb300._lib import RsfParams

    p = RsfParams()
    rsflib.rsf_params_default(ctypes.byref(p))
    assert rsflib.rsf_evolve(None, ctypes.byref(p), None, 0, None, 8, 8, 8, 1, None) == 1
    assert rsflib.rsf_workspace_destroy(None) == 1
    assert rsflib.rsf_params_default(None) == 1


def test_workspace_create_reports_missing_device(rsflib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    assert rsflib.rsf_workspace_create(100, 1, ctypes.byref(h)) == 10  # RSF_ERR_NO_DEVICE
    assert b"no CUDA device" in rsflib.rsf_last_error()


# --------------------------------------------------------------------- tiling
def test_config2_tiles():
    from rsf_gb300 import tiling

    tiles = tiling.config2_tiles()
    assert len(tiles) == 48
    assert sum(t.voxels for t in tiles) == 1216 * 1216 * 640
    assert {t.shape[0] for t in tiles} == {64, 320, 256}
    assert {t.shape[1] for t in tiles} == {288, 320} and {t.shape[2] for t in tiles} == {288, 320}
    cover = np.zeros((512, 1024 // 16, 1024 // 16), dtype=np.int32)  # cores partition the volume
    for t in tiles:
        cover[t.clo[0]:t.chi[0], t.clo[1] // 16:t.chi[1] // 16, t.clo[2] // 16:t.chi[2] // 16] += 1
    assert np.all(cover == 1)


def test_plan_cut_reassemble_roundtrip():
    from rsf_gb300 import tiling

    vol = np.random.default_rng(0).normal(size=(37, 41, 29)).astype(np.float32)
    tiles = tiling.plan(vol.shape, (10, 16, 7), 3)
    parts = tiling.cut(vol, tiles)
    assert all(p.shape == t.shape for p, t in zip(parts, tiles))
    from oracle import reassembly

    assert np.array_equal(reassembly.reassemble_cores(vol.shape, tiles, parts), vol)


def test_blend_halves_matches_interpolating_volumes():
    """interpolating_volumes.py:10-40: concatenate the non-overlapping parts
    and blend the overlap with weights linspace(0, 1, overlap) along axis 1."""
    from rsf_gb300 import tiling

    rng = np.random.default_rng(1)
    a = rng.normal(size=(5, 30, 7)).astype(np.float32)
    b = rng.normal(size=(5, 25, 7)).astype(np.float32)
    ov = 6
    alpha = np.linspace(0, 1, ov)[None, :, None]
    want = np.concatenate((a[:, :-ov, :], (1 - alpha) * a[:, -ov:, :] + alpha * b[:, :ov, :], b[:, ov:, :]), axis=1)
    from oracle import reassembly

    assert np.allclose(reassembly.blend_halves(a, b, ov, axis=1), want)


def test_lpt_shards_balance_and_partition():
    from rsf_gb300 import tiling

    tiles = tiling.config2_tiles()
    for n in (1, 2, 3, 8):
        shards = tiling.lpt_shards(tiles, n)
        assert sorted(i for s in shards for i in s) == list(range(48))
        loads = [sum(tiles[i].voxels for i in s) for s in shards]
        assert max(loads) <= 1.2 * sum(loads) / n + max(t.voxels for t in tiles)


# ------------------------------------------------------------------ generator
def test_torch_signed_distance_equals_scipy_edt():
    import torch
    from scipy import ndimage

    from rsf_gb300 import synth

    rng = np.random.default_rng(2)
    m = ndimage.binary_opening(rng.random((24, 27, 25)) < 0.35)
    got = synth.signed_distance_torch(torch.from_numpy(m), 3.0).numpy()
    assert np.array_equal(got, synth.signed_distance(m, 3.0))


def test_generator_is_seeded_and_in_range():
    from rsf_gb300 import synth

    a = synth.make_small((20, 22, 24), n_tubes=3, seed=3)
    b = synth.make_small((20, 22, 24), n_tubes=3, seed=3)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    img, phi0, mask = a
    assert img.dtype == np.uint8 and phi0.dtype == np.float32 and mask.dtype == bool
    assert phi0.min() >= -3 and phi0.max() <= 3


# ------------------------------------------------------------- multi-process
def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from rsf_gb300 import dist as rd, tiling

    tiles = tiling.config2_tiles()
    mine = rd.shard(tiles, rank, world)
    total = rd.sum_over_ranks(len(mine))
    slowest = rd.max_over_ranks(10.0 + rank)
    out.put((rank, mine, total, slowest, rd.rank_info()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharding_and_timing_reduction():
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, t0, m0, i0), (r1, s1, t1, m1, i1) = res
    assert sorted(s0 + s1) == list(range(48)) and not set(s0) & set(s1)
    assert t0 == t1 == 48
    assert m0 == m1 == 11.0
    assert i0 == (2, 0, 0) and i1 == (2, 1, 1)


def test_grid_blend_of_two_tiles_is_the_reference_blend():
    from oracle import reassembly
    from rsf_gb300 import tiling

    tiles = [tiling.Tile((0, 0, 0), (6, 30, 5), (0, 0, 0), (6, 20, 5)),
             tiling.Tile((0, 10, 0), (6, 50, 5), (0, 20, 0), (6, 50, 5))]
    rng = np.random.default_rng(0)
    a, b = rng.standard_normal(tiles[0].shape), rng.standard_normal(tiles[1].shape)
    got = reassembly.blend_grid((6, 50, 5), tiles, [a, b])
    assert np.allclose(got, reassembly.blend_halves(a, b, 20, axis=1), rtol=0, atol=1e-12)


def test_grid_bounds_and_chunking():
    from rsf_gb300 import driver, tiling

    tiles = tiling.plan((40, 48, 56), ([0, 8, 30, 40], 16, [0, 20, 56]), 5)
    bz, by, bx = tiling.grid_bounds(tiles)
    assert bz == [0, 8, 30, 40] and by == [0, 16, 32, 48] and bx == [0, 20, 56]
    with pytest.raises(ValueError):
        tiling.grid_bounds(tiles[::-1])
    with pytest.raises(ValueError):
        tiling.grid_bounds(tiles[:-1])
    groups = driver.chunk_tiles(tiles, 20000)
    assert sorted(i for g in groups for i in g) == list(range(len(tiles)))
    for g in groups:
        assert len(g) == 1 or sum(tiles[i].voxels for i in g) <= 20000
        assert g == list(range(g[0], g[-1] + 1))


def test_autotuner_picks_the_fastest_owned_throughput():
    from rsf_gb300 import Params, autotune

    shape = (200, 300, 300)
    plans = autotune.candidate_plans(shape, 32, (64, 128, 256, 512))
    assert [c for c, _ in plans] == [64, 128, 256, 300]  # 512 clips to the largest extent
    # a fake device: time proportional to evolved voxels plus a per-tile cost
    res = autotune.tune_cores(shape, Params(sigma=3.0), 32, candidates=(64, 128, 256, 512),
                              timer=lambda tiles: sum(t.voxels for t in tiles) / 3e10 + 2e-5 * len(tiles))
    evolved = {c: sum(t.voxels for t in tiles) for c, tiles in plans}
    assert res.cores == 300 and evolved[300] < evolved[64]
    res2 = autotune.tune_cores(shape, Params(sigma=3.0), 32, candidates=(64, 128, 256, 512),
                               timer=lambda tiles: 1e-3 + 0.0 * len(tiles) if len(tiles) > 4 else 1.0)
    assert res2.cores in (64, 128)


def test_autotuner_level_set_is_smooth_and_bounded():
    import torch
    from rsf_gb300 import autotune

    phi = autotune.smooth_phi((20, 30, 40))
    assert phi.shape == (20, 30, 40) and phi.dtype == torch.float32 and phi.is_contiguous()
    assert float(phi.abs().max()) <= 3.0 and float(phi.min()) < 0.0 < float(phi.max())
    # neighbouring voxels differ by at most the field's Lipschitz bound
    steps = [phi.diff(dim=d).abs().max() for d in range(3)]
    assert max(float(s) for s in steps) <= 3.0 * 0.37 + 1e-6
    z, y, x = 5, 7, 11
    want = 3.0 * np.sin(0.37 * x) * np.sin(0.29 * y + 1.0) * np.sin(0.23 * z + 2.0)
    assert abs(float(phi[z, y, x]) - want) < 1e-5


def test_plan_properties_over_random_grids():
    """For random shapes, core sizes (int or explicit bounds) and halos: the
    cores partition the volume, every tile is its core grown by the halo and
    clipped at the faces, grid_bounds recovers the bounds, and cut followed
    by core reassembly is the identity."""
    from oracle import reassembly
    from rsf_gb300 import tiling

    rng = np.random.default_rng(123)
    for _ in range(40):
        shape = tuple(int(v) for v in rng.integers(1, 40, size=3))
        cores = []
        for n in shape:
            if rng.random() < 0.5:
                cores.append(int(rng.integers(1, n + 3)))
            else:
                cuts = sorted(set(int(v) for v in rng.integers(1, max(n, 2), size=int(rng.integers(0, 4)))))
                cores.append([0] + [c for c in cuts if 0 < c < n] + [n])
        halo = int(rng.integers(0, 6))
        tiles = tiling.plan(shape, tuple(cores), halo)
        owner = np.zeros(shape, dtype=np.int32)
        for t in tiles:
            owner[t.core_slices()] += 1
            for a in range(3):
                assert t.lo[a] == max(0, t.clo[a] - halo) and t.hi[a] == min(shape[a], t.chi[a] + halo)
                assert 0 <= t.lo[a] <= t.clo[a] < t.chi[a] <= t.hi[a] <= shape[a]
        assert np.all(owner == 1)
        bounds = tiling.grid_bounds(tiles)
        for a, n in enumerate(shape):
            want = list(range(0, n, cores[a])) + [n] if isinstance(cores[a], int) else cores[a]
            assert bounds[a] == want
        vol = rng.normal(size=shape).astype(np.float32)
        assert np.array_equal(reassembly.reassemble_cores(shape, tiles, tiling.cut(vol, tiles)), vol)


def test_plan_rejects_bounds_that_do_not_partition():
    from rsf_gb300 import tiling

    for bad in ([0, 5, 5, 10], [1, 10], [0, 12], [0, 7, 3, 10]):
        with pytest.raises(ValueError):
            tiling.plan((10, 10, 10), (bad, 5, 5), 2)


def test_launch_shape_autotuner_picks_the_fastest():
    from rsf_gb300 import autotune

    assert len(autotune.LAUNCH_CANDIDATES) == 12
    assert len(set(autotune.LAUNCH_CANDIDATES)) == 12
    times = {shape: 10.0 + i for i, shape in enumerate(autotune.LAUNCH_CANDIDATES)}
    fastest = autotune.LAUNCH_CANDIDATES[5]
    times[fastest] = 1.0
    best = autotune.pick_launch_shape(list(times.items()))
    assert (best.xpass_width, best.stencil_planes, best.z_tma) == fastest
    assert best.ms_per_iteration == 1.0 and len(best.table) == 12


def test_launch_shape_override_rejects_bad_values_without_device(rsflib):
    # a null workspace is rejected before any device work
    assert rsflib.rsf_workspace_set_launch_shape(None, 0, 0, -1) == 1


def test_batched_adjoint_rejects_bad_arguments_without_device(rsflib):
    """rsf_step_adjoint_batched checks its workspace and table before any
    device work: a null workspace or a null table is an invalid argument."""
    from rsf_gb300._lib import RsfAdjointSubvol, RsfParams

    p = RsfParams()
    assert rsflib.rsf_params_default(ctypes.byref(p)) == 0
    arr = (RsfAdjointSubvol * 1)()
    assert rsflib.rsf_step_adjoint_batched(None, ctypes.byref(p), 0, arr, 1, None, None) == 1
    assert "workspace" in rsflib.rsf_last_error().decode()


def _gather_worker(rank, world, port, q):
    import os

    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from rsf_gb300 import driver, tiling

    tiles = tiling.plan((20, 30, 26), 10, 3)
    shards = tiling.lpt_shards(tiles, world)
    parts = [None] * len(tiles)
    for i in shards[rank]:
        parts[i] = torch.full(tiles[i].shape, float(i))
    driver._gather_tiles(parts, tiles, shards, rank, "cpu")
    if rank == 0:
        ok = all(p is not None and p.shape == tiles[i].shape and bool((p == i).all()) for i, p in enumerate(parts))
        q.put((rank, ok, len(tiles)))
    else:
        q.put((rank, True, len(tiles)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_tile_gather_on_host():
    """The sharded driver's gather: every rank's evolved tiles reach rank 0
    in place, over gloo (the evolution itself needs no exchange)."""
    import socket

    import torch.multiprocessing as mp

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_gather_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] and res[0][2] == 2 * 3 * 3
