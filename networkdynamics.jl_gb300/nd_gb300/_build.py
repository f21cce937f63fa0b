"""In-tree build of the native libraries.

* ``lib/libnd_b200.so``    — the CUDA library behind the C ABI of ``include/nd_gb300.h``,
  compiled for sm_103a only (``-gencode arch=compute_103a,code=sm_103a``).
* ``lib/libnd_graphgen.so`` — host-only seeded graph generators.

Translation units are compiled in parallel and relinked only when a source or header is
newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent                      # networkdynamics.jl_gb300/
REPO = ROOT.parent
CSRC = ROOT / "csrc"
INCLUDE = REPO / "include"
LIB_DIR = PKG_DIR / "lib"
OBJ_DIR = ROOT / "_build"

CUDA_LIB = LIB_DIR / "libnd_b200.so"
GRAPHGEN_LIB = LIB_DIR / "libnd_graphgen.so"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def _newest(paths) -> float:
    return max((p.stat().st_mtime for p in paths), default=0.0)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def build_cuda_library(force: bool = False, verbose: bool = False) -> Path:
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    if (not force and CUDA_LIB.exists()
            and CUDA_LIB.stat().st_mtime >= _newest(sources + headers + [Path(__file__)])):
        return CUDA_LIB
    nvcc = _nvcc()

    def compile_one(src: Path) -> Path:
        obj = OBJ_DIR / (src.stem + ".o")
        cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
        r = _run(cmd)
        if verbose and (r.stderr.strip()):
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(sources), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_one, sources))
    tmp = CUDA_LIB.with_suffix(".so.tmp")
    _run([nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
    os.replace(tmp, CUDA_LIB)
    return CUDA_LIB


def build_graphgen_library(force: bool = False) -> Path:
    src = CSRC / "nd_graphgen.cpp"
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    if not force and GRAPHGEN_LIB.exists() and GRAPHGEN_LIB.stat().st_mtime >= src.stat().st_mtime:
        return GRAPHGEN_LIB
    tmp = GRAPHGEN_LIB.with_suffix(".so.tmp")
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", str(src), "-o", str(tmp)])
    os.replace(tmp, GRAPHGEN_LIB)
    return GRAPHGEN_LIB


def build_all(force: bool = False, verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_cuda_library, force, verbose)
        f2 = ex.submit(build_graphgen_library, force)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all(force=True, verbose=True)
    print("built", CUDA_LIB, GRAPHGEN_LIB)
