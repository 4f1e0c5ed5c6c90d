"""Recipe that compiles the reference surfel rasterisers (plain and part) into
``oracle/_ref/`` as a parity and timing oracle.

TEST / MEASUREMENT INFRASTRUCTURE ONLY: tests, ``smoke()`` and ``bench.py``'s
reference-CUDA measurement import what this builds; the product library never
does.

Two steps, so that the build can run where the reference tree is absent:

1. ``stage(ref_root)`` copies, unmodified, the files the reference's own
   extension is made of (``submodules/diff-surfel-rasterization{,_part}/``:
   ``cuda_rasterizer/*``, ``rasterize_points.{cu,h}``, ``ext.cpp`` and the
   package ``__init__.py``) into the git-ignored ``oracle/_ref/src/``.
   Nothing under ``oracle/_ref/`` is committed.
2. ``build()`` compiles the staged sources with nvcc / g++ directly (no
   setuptools, no ninja) against PyTorch's headers and the project-written
   glm subset in ``oracle/glm/``: ``-O3``, no fast-math, sm_103a, as the
   reference's ``setup.py`` lists the sources
   (``submodules/diff-surfel-rasterization/setup.py:18-30``).  The CUDA
   sources are compiled with ``-include cstdint``: ``rasterizer_impl.h`` uses
   ``uint32_t`` without including ``<cstdint>``, which GCC 13's standard
   headers no longer pull in for it.  Each variant
   becomes a package ``oracle/_ref/<variant>/<package>/`` holding the
   reference's ``__init__.py`` and its ``_C`` extension module.

``load(variant)`` imports that package under a private module name
(``ref_plain`` / ``ref_part``), so it can sit beside the product's own
``diff_surfel_rasterization`` modules in one process.

    python oracle/ref_build.py [--ref /path/to/PartGS] [--force]
"""
from __future__ import annotations

import importlib.util
import os
import shutil
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SRC = OUT / "src"
GLM = HERE / "glm"

VARIANTS = {
    "plain": ("diff-surfel-rasterization", "diff_surfel_rasterization"),
    "part": ("diff-surfel-rasterization_part", "diff_surfel_rasterization_part"),
}
# the extension's sources in the reference's setup.py order
CU_SOURCES = ["cuda_rasterizer/rasterizer_impl.cu", "cuda_rasterizer/forward.cu", "cuda_rasterizer/backward.cu",
              "rasterize_points.cu"]
CPP_SOURCES = ["ext.cpp"]
HEADERS = ["cuda_rasterizer/auxiliary.h", "cuda_rasterizer/backward.h", "cuda_rasterizer/config.h",
           "cuda_rasterizer/forward.h", "cuda_rasterizer/rasterizer.h", "cuda_rasterizer/rasterizer_impl.h",
           "rasterize_points.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def staged(variant: str) -> bool:
    d, pkg = VARIANTS[variant]
    root = SRC / d
    return all((root / f).exists() for f in CU_SOURCES + CPP_SOURCES + HEADERS + [f"{pkg}/__init__.py"])


def stage(ref_root: str | os.PathLike) -> None:
    """Copy the reference extension's sources, unmodified, into oracle/_ref/src."""
    ref_root = Path(ref_root)
    for variant, (d, pkg) in VARIANTS.items():
        src = ref_root / "submodules" / d
        if not src.is_dir():
            raise FileNotFoundError(f"reference rasteriser sources not found at {src}")
        for f in CU_SOURCES + CPP_SOURCES + HEADERS + [f"{pkg}/__init__.py"]:
            dst = SRC / d / f
            dst.parent.mkdir(parents=True, exist_ok=True)
            shutil.copyfile(src / f, dst)


def _so_name() -> str:
    return "_C" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so")


def product(variant: str) -> Path:
    d, pkg = VARIANTS[variant]
    return OUT / variant / pkg / _so_name()


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found")
    return cand


def _torch_flags():
    import torch
    troot = Path(torch.__file__).resolve().parent
    inc = [troot / "include", troot / "include" / "torch" / "csrc" / "api" / "include"]
    abi = int(getattr(torch._C, "_GLIBCXX_USE_CXX11_ABI", True))
    defs = ["-DTORCH_API_INCLUDE_EXTENSION_H", "-DTORCH_EXTENSION_NAME=_C", f"-D_GLIBCXX_USE_CXX11_ABI={abi}"]
    return [f"-I{p}" for p in inc] + [f"-I{sysconfig.get_paths()['include']}"] + defs, troot / "lib"


def _cuda_root() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _cuda_lib_dir() -> Path:
    root = _cuda_root()
    for cand in (root / "lib64", root / "lib", root / "targets" / "sbsa-linux" / "lib",
                 root / "targets" / "x86_64-linux" / "lib"):
        if (cand / "libcudart.so").exists():
            return cand
    return root / "lib64"


def up_to_date(variant: str) -> bool:
    p = product(variant)
    if not p.exists():
        return False
    d, _ = VARIANTS[variant]
    t = p.stat().st_mtime
    inputs = [SRC / d / f for f in CU_SOURCES + CPP_SOURCES + HEADERS] + [GLM / "glm" / "glm.hpp"]
    return all(f.exists() and f.stat().st_mtime <= t for f in inputs)


def build(force: bool = False, verbose: bool = False) -> dict:
    """Compile every staged variant that is out of date; returns {variant: path}."""
    todo = [v for v in VARIANTS if staged(v) and (force or not up_to_date(v))]
    built = {v: product(v) for v in VARIANTS if staged(v)}
    if not todo:
        return built
    tflags, tlib = _torch_flags()
    nvcc = _nvcc()
    cuda_inc = _cuda_root() / "include"
    jobs = []
    for v in todo:
        d, pkg = VARIANTS[v]
        root = SRC / d
        obj_dir = OUT / "obj" / v
        obj_dir.mkdir(parents=True, exist_ok=True)
        for s in CU_SOURCES:
            obj = obj_dir / (Path(s).stem + ".o")
            cmd = [nvcc, "-O3", "-std=c++17", *ARCH, "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                   "-D__CUDA_NO_HALF_OPERATORS__", "-D__CUDA_NO_HALF_CONVERSIONS__",
                   "-D__CUDA_NO_BFLOAT16_CONVERSIONS__", "-D__CUDA_NO_HALF2_OPERATORS__",
                   "-include", "cstdint", f"-I{GLM}", f"-I{root}", *tflags, "-c", str(root / s), "-o", str(obj)]
            jobs.append((v, obj, cmd))
        for s in CPP_SOURCES:
            obj = obj_dir / (Path(s).stem + ".o")
            cmd = ["g++", "-O3", "-std=c++17", "-fPIC", f"-I{root}", f"-I{cuda_inc}", *tflags,
                   "-c", str(root / s), "-o", str(obj)]
            jobs.append((v, obj, cmd))

    def run(job):
        v, obj, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference build ({v}) failed on {obj.name}:\n{' '.join(cmd)}\n{r.stderr[-4000:]}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    for v in todo:
        d, pkg = VARIANTS[v]
        pkg_dir = OUT / v / pkg
        pkg_dir.mkdir(parents=True, exist_ok=True)
        shutil.copyfile(SRC / d / pkg / "__init__.py", pkg_dir / "__init__.py")
        objs = [str(OUT / "obj" / v / (Path(s).stem + ".o")) for s in CU_SOURCES + CPP_SOURCES]
        tmp = pkg_dir / (_so_name() + ".tmp")
        cmd = ["g++", "-shared", "-o", str(tmp), *objs, f"-L{tlib}", f"-L{_cuda_lib_dir()}",
               "-lc10", "-ltorch", "-ltorch_cpu", "-ltorch_python", "-lc10_cuda", "-ltorch_cuda", "-lcudart",
               f"-Wl,-rpath,{tlib}", f"-Wl,-rpath,{_cuda_lib_dir()}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference link ({v}) failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, product(v))
    return built


_LOADED = {}


def available(variant: str) -> bool:
    return product(variant).exists()


def load(variant: str):
    """Import the built reference package of ``variant`` ("plain" or "part")
    as module ``ref_<variant>``; raises ImportError when it was not built."""
    if variant in _LOADED:
        return _LOADED[variant]
    d, pkg = VARIANTS[variant]
    pkg_dir = OUT / variant / pkg
    if not product(variant).exists():
        raise ImportError(f"reference rasteriser ({variant}) not built: run oracle/ref_build.py")
    import torch  # noqa: F401  (the extension links against torch's libraries)
    name = f"ref_{variant}"
    spec = importlib.util.spec_from_file_location(name, pkg_dir / "__init__.py",
                                                  submodule_search_locations=[str(pkg_dir)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    _LOADED[variant] = mod
    return mod


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("PARTGS_REFERENCE"),
                    help="root of a PartGS checkout to stage the sources from")
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", action="store_true")
    a = ap.parse_args(argv)
    if a.ref:
        stage(a.ref)
    if not all(staged(v) for v in VARIANTS):
        raise SystemExit("reference sources are not staged: pass --ref <PartGS checkout>")
    for v, p in build(force=a.force, verbose=a.v).items():
        print(v, p)


if __name__ == "__main__":
    main()
