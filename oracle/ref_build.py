"""Compiles the reference's own CUDA kernels (CUDA_RSF/kernel.cu, unchanged,
read where it lies in the reference checkout named by the environment
variable RSF_REFERENCE_ROOT, or by --reference-root) into a cubin for sm_103a
under oracle/_ref/, with the kernels' mangled entry names taken from ptxas's
report.  TEST INFRASTRUCTURE: only the reference cross-check uses it.  The
reference's host program (main.cpp) is not built: it needs Windows.h,
tiralib and Boost; oracle/ref_harness.py replays its iteration loop."""
from __future__ import annotations

import json
import os
import re
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
CUBIN = OUT / "kernel_sm103a.cubin"
NAMES = OUT / "kernels.json"
# The reference checkout's root; unset, the build recipe's mount point.
DEFAULT_REFERENCE_ROOT = "/root/reference"


def reference_kernel(root: str | None = None) -> Path:
    root = root or os.environ.get("RSF_REFERENCE_ROOT") or DEFAULT_REFERENCE_ROOT
    return Path(root) / "CUDA_RSF" / "kernel.cu"


def build_if_present(root: str | None = None) -> bool:
    """Builds the cubin when the reference sources are present; returns
    whether a cubin is available afterwards."""
    src = reference_kernel(root)
    if not src.exists():
        return CUBIN.exists() and NAMES.exists()
    if CUBIN.exists() and NAMES.exists() and CUBIN.stat().st_mtime >= src.stat().st_mtime:
        return True
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    OUT.mkdir(exist_ok=True)
    res = subprocess.run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-Xptxas", "-v",
                          str(src), "-o", str(CUBIN)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference kernel build failed:\n{res.stderr}")
    names = {}
    for m in re.findall(r"Compiling entry function '(_Z\d+([A-Za-z_]\w*?)P[^']*)'", res.stderr):
        mangled = m[0]
        plain = re.match(r"_Z(\d+)", mangled)
        n = int(plain.group(1))
        names[mangled[2 + len(plain.group(1)):2 + len(plain.group(1)) + n]] = mangled
    NAMES.write_text(json.dumps(names, indent=1, sort_keys=True))
    return True


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=None, help="root of the reference checkout")
    print(build_if_present(ap.parse_args().reference_root), CUBIN)
