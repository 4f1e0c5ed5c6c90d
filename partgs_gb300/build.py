"""Builds libsgr.so in-tree (partgs_gb300/_lib/) with nvcc for sm_103a.

The translation units compile in parallel; the library links the CUDA runtime
as a shared object so that it shares the process's runtime with PyTorch.
Nothing is rebuilt when the library is newer than every source.
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
INCLUDE = HERE.parent / "include"
OUT = HERE / "_lib"
LIB = OUT / "libsgr.so"
SOURCES = ["sgr_api.cu", "sgr_forward.cu", "sgr_blend.cu", "sgr_binning.cu", "sgr_backward.cu", "sgr_bind.cu",
           "sgr_loss.cu", "sgr_adam.cu", "sgr_mlp.cu", "sgr_activate.cu",
           "sgr_eval.cu", "sgr_sq.cu", "sgr_densify.cu", "sgr_sort.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the surfel rasteriser needs the CUDA toolkit to build")
    return cand


def cuda_lib_dir() -> str:
    root = Path(nvcc()).resolve().parent.parent
    for cand in (root / "lib64", root / "lib", root / "targets" / "sbsa-linux" / "lib",
                 root / "targets" / "x86_64-linux" / "lib"):
        if (cand / "libcudart.so").exists() or (cand / "libcudart.so.13").exists():
            return str(cand)
    return str(root / "lib64")


def common_flags(extra=()):
    return ["-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
            f"-I{INCLUDE}", *extra]


def _inputs():
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _inputs())


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
    if not force and up_to_date():
        return LIB
    OUT.mkdir(exist_ok=True)
    cc = nvcc()
    flags = common_flags(extra_flags)

    def compile_one(src: str):
        obj = OUT / (Path(src).stem + ".o")
        cmd = [cc, *flags, "-c", str(CSRC / src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = OUT / "libsgr.so.tmp"
    cmd = [cc, "-shared", *ARCH, "-cudart", "shared", "-o", str(tmp), *map(str, objs),
           "-Xlinker", f"-rpath={cuda_lib_dir()}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libsgr.so failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                 extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else ())
    print(path)
