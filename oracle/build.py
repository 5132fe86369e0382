"""ORACLE build recipe — test infrastructure only.

* geom_oracle.c -> oracle/_build/libgeom_oracle.so, with -ffp-contract=off (so
  the compiler adds no fused multiply-adds beyond the explicit fma() calls;
  gcc on aarch64 would otherwise contract).
* The reference's makeOTF (src/radialft_interface.cpp) with stand-ins for
  FFTW and libtiff (oracle/shim/) into oracle/_ref/libradialft_ref.so, only
  where the reference is present (it generates the OTF fixtures).
* The reference's own CUDA kernels, compiled from its sources where they lie
  (src/{RLgpuImpl,geometryTransform,camcor}.cu of the reference checkout, with
  its Buffers/ headers) to PTX in oracle/_ref/ — only where the reference is
  present.  The checkout is taken from the CDX_REFERENCE_DIR environment
  variable or the --reference argument, by default /root/reference.  The PTX travels with the repository to the GPU machine, where
  ref_runner.cu (our launcher, driver API + cuFFT) is compiled against it into
  oracle/_ref/libref_runner.so.  Nothing here reads the PTX; it is loaded with
  cuModuleLoad.
"""

from __future__ import annotations

import argparse
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"


def build_geom() -> Path:
    src = HERE / "geom_oracle.c"
    out = OUT / "libgeom_oracle.so"
    if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    OUT.mkdir(exist_ok=True)
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           str(src), "-o", str(out), "-lm"]
    subprocess.run(cmd, check=True)
    return out


REF_SRC = Path(os.environ.get("CDX_REFERENCE_DIR", "/root/reference")) / "src"
REF_OUT = HERE / "_ref"
REF_UNITS = ["RLgpuImpl", "geometryTransform", "camcor"]


def _nvcc() -> str:
    p = Path("/usr/local/cuda/bin/nvcc")
    return str(p) if p.exists() else "nvcc"


def build_ref_ptx() -> bool:
    """Compile the reference's kernels to PTX (only where the reference exists)."""
    if not (REF_SRC / "RLgpuImpl.cu").exists():
        return all((REF_OUT / f"{u}.ptx").exists() for u in REF_UNITS)
    REF_OUT.mkdir(exist_ok=True)
    for u in REF_UNITS:
        src, out = REF_SRC / f"{u}.cu", REF_OUT / f"{u}.ptx"
        if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
            continue
        cmd = [_nvcc(), "-ptx", "-arch=compute_103a", "-std=c++17", f"-I{REF_SRC}",
               f"-I{REF_SRC / 'Buffers'}", str(src), "-o", str(out)]
        subprocess.run(cmd, check=True)
    return True


def build_ref_runner() -> Path | None:
    """Compile our launcher of the reference kernels (needs the PTX and cuFFT)."""
    if not all((REF_OUT / f"{u}.ptx").exists() for u in REF_UNITS):
        return None
    src, out = HERE / "ref_runner.cu", REF_OUT / "libref_runner.so"
    if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
        return out
    cmd = [_nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", str(src), "-o",
           str(out), "-lcuda", "-lcufft"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print("reference runner not built:", r.stderr[-2000:])
        return None
    return out


SHIM = HERE / "shim"


def build_radialft_ref() -> Path | None:
    """The reference's makeOTF (src/radialft_interface.cpp, compiled where it
    lies) with the FFTW and libtiff stand-ins of oracle/shim/, into
    oracle/_ref/libradialft_ref.so; only where the reference is present."""
    src = REF_SRC / "radialft_interface.cpp"
    if not src.exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "libradialft_ref.so"
    deps = [src, SHIM / "fftw_shim.cpp", SHIM / "tiff_capture.cpp", SHIM / "fftw3.h",
            SHIM / "tiffio.h"]
    if out.exists() and out.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return out
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-Dcimg_display=0", f"-I{SHIM}",
           f"-I{REF_SRC}", str(src), str(SHIM / "fftw_shim.cpp"), str(SHIM / "tiff_capture.cpp"),
           "-o", str(out), "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        print("reference makeOTF not built:", r.stderr[-2000:])
        return None
    return out


def build_all() -> None:
    build_geom()
    try:
        build_radialft_ref()
    except (subprocess.CalledProcessError, OSError) as e:
        print("reference makeOTF not built:", e)
    try:
        if build_ref_ptx():
            build_ref_runner()
    except (subprocess.CalledProcessError, OSError) as e:
        print("reference kernels not built:", e)


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", help="reference checkout (its src/ holds the .cu sources)")
    a = ap.parse_args()
    if a.reference:
        REF_SRC = Path(a.reference) / "src"
    build_all()
    print("ok")
