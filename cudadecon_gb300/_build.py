"""Build the in-tree CUDA library ``lib/libcudaDecon.so`` for sm_103a.

Each translation unit is compiled by nvcc in parallel into ``_build/`` and
then linked; a unit is recompiled only when its source or any header in
``csrc/`` is newer than its object.
"""

from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OBJDIR = PKG / "_build"
LIBDIR = PKG / "lib"
LIBNAME = "libcudaDecon.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(INCLUDE)]
SOURCES = ["decon_kernels.cu", "decon_x_fwd.cu", "decon_x_ratio.cu", "decon_x_update.cu", "decon_x_tc.cu", "decon_y.cu", "decon_z.cu", "geometry.cu", "affine.cu", "accel.cu", "accel_noalloc.cu", "abi.cu", "otf_make.cu", "wiener.cu", "tiles.cu", "otf_io.cpp"]


# the generated units of the x-pass plans (gen_plans.py)
SOURCES += sorted(p.name for p in CSRC.glob("decon_x_gen_*.cu"))


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: str, hmt: float, verbose: bool) -> Path:
    s = CSRC / src
    o = OBJDIR / (s.stem + ".o")
    if o.exists() and o.stat().st_mtime >= max(s.stat().st_mtime, hmt):
        return o
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return o


def build(verbose: bool = False, force: bool = False) -> Path:
    OBJDIR.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    if force:
        for o in OBJDIR.glob("*.o"):
            o.unlink()
    hmt = _headers_mtime()
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, hmt, verbose), SOURCES))
    out = lib_path()
    newest = max(o.stat().st_mtime for o in objs)
    if force or not out.exists() or out.stat().st_mtime < newest:
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(out), *map(str, objs), "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    print(build(verbose=True))
