"""ORACLE build recipe — test infrastructure only.

Compiles the C restatement geom_oracle.c into oracle/_build/libgeom_oracle.so
with -ffp-contract=off (so the compiler adds no fused multiply-adds beyond
the explicit fma() calls; gcc on aarch64 would otherwise contract).
"""

from __future__ import annotations

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


def build_all() -> None:
    build_geom()


if __name__ == "__main__":
    build_all()
    print("ok")
