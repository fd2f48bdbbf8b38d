"""In-tree build of the native libraries (no CMake, no torch extension machinery).

* ``_build/libsubsweep_gpu.so``  — the sweep library behind include/subsweep_gpu.h:
  sweep_fp64.cu (compiled with -fmad=false so FP64 expressions round as the Rust
  reference's do), sweep_mixed.cu (FMA allowed) and the C++ host runtime, plus the GPU
  Voronoi producer voronoi_gpu.cu (-fmad=false, as the host producer).
* ``_build/libsubsweep_grid.so`` — host grid producers (Voronoi / cartesian CSR).

Both are compiled for sm_103a only.  Sources are rebuilt when newer than the output.
"""
from __future__ import annotations

import os
import pathlib
import subprocess
import concurrent.futures as cf

HERE = pathlib.Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
ROOT = HERE.parent

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: host-side FP64 (geometry checks, direction normalisation) must not
# fuse multiply-adds either; aarch64 g++ contracts by default.
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]

GPU_LIB = BUILD / "libsubsweep_gpu.so"
GRID_LIB = BUILD / "libsubsweep_grid.so"

_HEADERS = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [CSRC / "direction_bins.inc",
                                                                     ROOT / "include" / "subsweep_gpu.h"]


def _stale(out: pathlib.Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(pathlib.Path(d).stat().st_mtime > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(str(c) for c in cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _nvcc_obj(src: pathlib.Path, fmad: bool, verbose: bool, extra=()):
    obj = BUILD / (src.stem + ".o")
    if _stale(obj, [src] + _HEADERS):
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", f"-fmad={'true' if fmad else 'false'}",
               "-c", src, "-o", obj, *extra]
        _run(cmd, verbose)
    return obj


def build(verbose: bool = False) -> dict:
    """Compile every native library; returns their paths."""
    BUILD.mkdir(exist_ok=True)
    jobs = [
        (CSRC / "sweep_fp64.cu", False),
        (CSRC / "sweep_mixed.cu", True),
        (CSRC / "sweep_host.cpp", True),
        (CSRC / "sweep_noalloc.cu", True),
        (CSRC / "voronoi_gpu.cu", False),
    ]
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        futs = [ex.submit(_nvcc_obj, src, fmad, verbose) for src, fmad in jobs]
        grid_fut = None
        if _stale(GRID_LIB, [CSRC / "grid_host.cpp", CSRC / "grid_host.h"]):
            grid_fut = ex.submit(_run, [CXX, *HOST_FLAGS, "-O3", "-shared", "-o", GRID_LIB,
                                        CSRC / "grid_host.cpp", "-lpthread"], verbose)
        objs = [f.result() for f in futs]
        if grid_fut is not None:
            grid_fut.result()
    if _stale(GPU_LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", GPU_LIB, *objs, "-lcudart"], verbose)
    return {"gpu": GPU_LIB, "grid": GRID_LIB}


if __name__ == "__main__":
    print(build(verbose=True))
