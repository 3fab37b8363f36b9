"""The whole-volume driver sharded over two ranks (two processes on this
GPU, gloo for the gather): each rank evolves its share of the tiles with no
exchange during the evolution, rank 0 stitches, and the volume equals the
single-process driver's bit for bit.  The two ranks' kernels never wait on
one another; only the host-side gather crosses ranks."""
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

SHAPE = (48, 72, 64)
PARAMS = dict(sigma=1.5, dt=0.1, mu=1.0, lambda1=1.0, lambda2=1.0, nu=65.025, eps=1.0)


def _volume():
    from rsf_gb300 import synth

    img, phi0, mask = synth.make_small(SHAPE, n_tubes=4, r_min=2.0, r_max=4.0, seed=17)
    seed = (mask.astype(np.uint8) * 200)
    return img, seed


def _rank(rank, world, port, q):
    import os
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    sys.path[:0] = [str(root), str(root / "paper-rsf-vesselseg_gb300")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    from rsf_gb300 import Params, driver

    dist.init_process_group("gloo", rank=rank, world_size=world)
    img, seed = _volume()
    out = driver.segment(img, seed, Params(**PARAMS), 6, cores=24, halo=12, device="cuda:0", distributed=True)
    q.put((rank, None if out is None else out.cpu().numpy()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_driver_equals_single_rank(cuda, rsflib):
    import torch.multiprocessing as mp

    from rsf_gb300 import Params, driver

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert res[1] is None
    img, seed = _volume()
    want = driver.segment(img, seed, Params(**PARAMS), 6, cores=24, halo=12, device="cuda:0").cpu().numpy()
    assert np.array_equal(res[0].view(np.uint32), want.view(np.uint32))
