"""Build the CUDA library libnatrix_gb300.so in-tree (natrix_gb300/_lib/).

nvcc compiles each translation unit for sm_103a in parallel and links one
shared library with the CUDA runtime linked statically, so the library has no
dependency beyond the driver.  The solver units use -fmad=false: the kernels
rely on every product and sum rounding separately (bit-exact FP32 parity with
the reference shader arithmetic).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_lib"
LIB = OUT / "libnatrix_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
          "-I", str(HERE.parent / "include")]
# translation unit -> extra flags
UNITS = {
    "solver_kernels.cu": ["-fmad=false"],
    "jacobi_tma.cu": ["-fmad=false"],
    "capi.cu": [],
    "noalloc.cu": ["-fmad=false"],
    "particles.cu": ["-fmad=false"],
    "batch.cu": ["-fmad=false"],
    "render.cu": ["-fmad=false"],
    "unet_conv.cu": [],
    "unet_kernels.cu": [],
    "unet_wgrad.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(srcs, target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(p.stat().st_mtime > t for p in srcs)


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list((HERE.parent / "include").glob("*.h"))
    objs = []
    jobs = []
    for unit, flags in UNITS.items():
        src = CSRC / unit
        obj = OUT / (src.stem + ".o")
        objs.append(obj)
        if force or _stale([src, *headers, Path(__file__)], obj):
            cmd = [nvcc(), *ARCH, *COMMON, *flags, "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg, file=sys.stderr)
    if force or jobs or _stale(objs, LIB):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIB), *map(str, objs)]
        run(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
