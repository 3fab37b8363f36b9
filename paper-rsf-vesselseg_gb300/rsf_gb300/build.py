"""Builds librsf_gb300.so (sm_103a) and the `rsf3d` command-line tool in-tree.

nvcc compiles each translation unit in parallel; nothing is installed.  The
outputs land in paper-rsf-vesselseg_gb300/lib/ and paper-rsf-vesselseg_gb300/bin/.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parents[1]
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
INCLUDE = REPO_ROOT / "include"
LIB_DIR = PKG_ROOT / "lib"
BIN_DIR = PKG_ROOT / "bin"
BUILD_DIR = PKG_ROOT / "_build"
LIB_PATH = LIB_DIR / "librsf_gb300.so"
CLI_PATH = BIN_DIR / "rsf3d"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
                     "-I", str(INCLUDE), "-I", str(CSRC)]
# (source, object stem, extra defines): the per-family kernels are compiled
# once per tap specialisation so that the objects build in parallel.
CU_UNITS = ([(f"rsf_{fam}.cu", f"rsf_{fam}_k{k}", [f"-DRSF_K={k}"]) for fam in ("xpass", "ypass", "zpass")
             for k in (0, 21, 29, 35)]
            + [("rsf_ztpass.cu", f"rsf_ztpass_k{k}", [f"-DRSF_K={k}"]) for k in (21, 35)]
            + [("rsf_stencil.cu", "rsf_stencil", []), ("rsf_step.cu", "rsf_step", []),
               ("rsf_capi.cu", "rsf_capi", []), ("rsf_noalloc.cu", "rsf_noalloc", []),
               ("rsf_sdf.cu", "rsf_sdf", []), ("rsf_adjoint.cu", "rsf_adjoint", []),
               ("rsf_reassemble.cu", "rsf_reassemble", []), ("rsf_copy.cu", "rsf_copy", []),
               ("rsf_gauss.cu", "rsf_gauss", [])])
CLI_SOURCES = ["rsf_cli.cpp", "npy_io.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build librsf_gb300")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(map(str, cmd))}\n{res.stdout}\n{res.stderr}")
    return res


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> Path:
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    BIN_DIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    nv = nvcc()
    jobs = []
    objs = []
    for src, stem, defs in CU_UNITS:
        obj = BUILD_DIR / (stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            flags = NVCC_FLAGS + defs + (["-Xptxas", "-v"] if ptxas_info else [])
            jobs.append([nv, *flags, "-c", CSRC / src, "-o", obj])
    cli_objs = []
    for src in CLI_SOURCES:
        if not (CSRC / src).exists():
            continue
        obj = BUILD_DIR / (Path(src).stem + ".o")
        cli_objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
                         "-I", Path(nv).resolve().parents[1] / "include", "-c", CSRC / src, "-o", obj])
    outputs = []
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for res in ex.map(lambda c: _run(c, verbose), jobs):
            outputs.append(res)
    if ptxas_info:
        for res in outputs:
            print(res.stderr)
    if force or _stale(LIB_PATH, objs):
        _run([nv, *ARCH, "-shared", "-o", LIB_PATH, *objs, "-lcudart"], verbose)
    if cli_objs and (force or _stale(CLI_PATH, cli_objs + [LIB_PATH])):
        _run(["g++", "-o", CLI_PATH, *cli_objs, f"-L{LIB_DIR}", "-lrsf_gb300", "-Wl,-rpath,$ORIGIN/../lib",
              f"-L{Path(nv).resolve().parents[1] / 'lib64'}", "-lcudart"], verbose)
    return LIB_PATH


if __name__ == "__main__":
    import sys

    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
