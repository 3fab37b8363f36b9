"""Generates tests/golden/reference_kernels_*.npz: inputs and the outputs of
the reference's own kernels (CUDA_RSF/kernel.cu compiled unchanged,
oracle/_ref) for one and three iterations, so that the CPU tests can pin the
oracle to the reference without a GPU.

Run on a machine with a GPU, from the repository root, after
`python -c "import __graft_entry__ as g; g.build()"` in a checkout where the
reference sources were present at build time:

    python tests/golden/make_reference_goldens.py OUT_DIR
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "paper-rsf-vesselseg_gb300"))

CASES = {"s1": ((20, 22, 24), 1.0, 21), "s3": ((24, 26, 28), 3.0, 22)}
KEEP = ("H", "gx", "gy", "gz", "mag", "nx", "kappa", "lap", "I_ob", "HD_ob", "fout", "fin", "dh")


def main(out_dir: Path):
    import torch

    from oracle import ref_harness, rsf_oracle as orc
    from rsf_gb300 import synth

    rk = ref_harness.RefKernels()
    dev = torch.device("cuda:0")
    for tag, (shape, sigma, seed) in CASES.items():
        img, phi0, _ = synth.make_small(shape, n_tubes=4, r_min=1.5, r_max=4.0, seed=seed)
        L, H, W = shape
        im = torch.from_numpy(img.astype(np.float32).ravel()).to(dev)
        taps = torch.from_numpy(orc.taps(sigma)).to(dev)
        params = dict(sigma=sigma, e=1.0, dt=0.1, v=65.025, meu=1.0)
        phi = torch.from_numpy(phi0.ravel().copy()).to(dev)
        phi1, f = ref_harness.iteration(rk, phi, im, taps, W, H, L, **params)
        phi3, _ = ref_harness.evolve(rk, phi1, im, taps, W, H, L, 2, **params)
        arrays = {k: f[k].cpu().numpy().reshape(shape) for k in KEEP}
        arrays.update(phi0=phi0, image=img, phi1=phi1.cpu().numpy().reshape(shape),
                      phi3=phi3.cpu().numpy().reshape(shape), sigma=np.float32(sigma))
        path = out_dir / f"reference_kernels_{tag}.npz"
        np.savez_compressed(path, **arrays)
        print("wrote", path)


if __name__ == "__main__":
    main(Path(sys.argv[1] if len(sys.argv) > 1 else "."))
