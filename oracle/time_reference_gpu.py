"""ORACLE -- test infrastructure only: times the reference's own RL iteration
on the GPU (its kernels from src/RLgpuImpl.cu compiled here, with cuFFT, in the
order of RichardsonLucy_GPU's loop, src/RL-Biggs-Andrews.cpp:282-367; run by
oracle/ref_runner.cu) on the stage-scan decon grid, for comparison with the
library's iteration.  Setup (allocations, cuFFT plans, OTF array) is removed
by timing 5 and 20 iterations and taking the difference.

    python oracle/time_reference_gpu.py      (needs a GPU and oracle/_ref built)
"""

import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

from cudadecon_gb300 import synth  # noqa: E402
from oracle import ref_kernels as RK  # noqa: E402


def main(shape=(100, 256, 756), reps=2):
    import torch
    ok, why = RK.available()
    if not ok:
        print("reference build unavailable:", why)
        return 1
    nz, ny, nx = shape
    rng = np.random.default_rng(1)
    X0 = (100 + rng.gamma(2, 40, shape)).astype(np.float32)
    tab = synth.gaussian_otf_table(129, 64, 1.3, 3.0)
    best = {}
    for _ in range(reps):
        for n in (5, 20):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            RK.rl_iterations(X0, X0, tab, (0.3, 0.3, 0.5), n)
            torch.cuda.synchronize()
            best[n] = min(best.get(n, 1e9), time.perf_counter() - t0)
    it = (best[20] - best[5]) / 15
    print(f"reference RL iteration (its kernels + cuFFT) on {nz}x{ny}x{nx}: "
          f"{it * 1e3:.3f} ms/iteration, {nz * ny * nx / it / 1e9:.2f} G voxel-iter/s "
          f"(5 it {best[5] * 1e3:.1f} ms, 20 it {best[20] * 1e3:.1f} ms)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
