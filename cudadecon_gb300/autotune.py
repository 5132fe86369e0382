"""Autotuner of the generated compile-time FFT plans.

Every length of the batched workloads' ranges has a few candidate plans
(gen_plans.candidates): radix order, pencil batch (y rows, z columns or x
row pairs per block), register budget and stage-layout padding.  Plans are compile-time types,
so the tuner builds the library once per candidate column (column k =
candidate k of every length, candidate 0 where a length has fewer) in a
scratch copy of the package, runs one synthetic stack per length through cdx_RL_device with the
per-pass timers (cdx_profile_*) on this GPU, and keeps, per axis and length,
the candidate with the shortest pass time: x = forward + ratio + update
passes, y = the four y passes, z = the two z passes of an iteration.  A
candidate replaces candidate 0 only when it is faster by more than the
margin (timing noise).  The choices and the measured times are written to
tuned_plans.json, then gen_plans.py regenerates the plan sources from it;
rebuild the library afterwards.

    python cudadecon_gb300/autotune.py [--columns N] [--margin 0.02]
                                       [--workdir DIR] [--no-apply]

The stack of probe i has z, y and x lengths zs[i % nz], ys[i % ny] and
xs[i % nx], so every length is timed at least once on its axis; every
column times the same stacks.
"""

from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent

# pass indices of cdx_profile_read (abi.cu: x_fwd_predict, y_fwd, z_otf,
# y_inv, x_ratio_fwd, y_fwd2, z_otf_conj, y_inv2, x_inv_update)
AXIS_PASSES = {"x": (0, 4, 8), "y": (1, 3, 5, 7), "z": (2, 6)}
ITERS = 10


def probe_shapes(lens: dict[str, list[int]]) -> list[tuple[int, int, int]]:
    n = max(len(v) for v in lens.values())
    zs, ys, xs = lens["z"], lens["y"], lens["x"]
    return [(zs[i % len(zs)], ys[i % len(ys)], xs[i % len(xs)]) for i in range(n)]


def axis_times(shapes, pass_ms, lens) -> dict[str, dict[int, float]]:
    """Per axis and length: the summed pass time (ms per iteration) of that
    axis's passes over the probe stacks with that length on the axis."""
    out: dict[str, dict[int, float]] = {a: {} for a in AXIS_PASSES}
    for (nz, ny, nx), pm in zip(shapes, pass_ms):
        for axis, L in (("x", nx), ("y", ny), ("z", nz)):
            if L in lens[axis]:
                out[axis][L] = out[axis].get(L, 0.0) + sum(pm[i] for i in AXIS_PASSES[axis])
    return out


def select(times_by_column: list[dict[str, dict[int, float]]], cands, margin: float) -> dict:
    """Fastest candidate per axis and length.  times_by_column[k][axis][L]
    is column k's time; cands(axis, L) the candidate list.  Candidate 0 is
    kept unless another beats it by more than margin (relative)."""
    res: dict = {}
    for axis in AXIS_PASSES:
        res[axis] = {}
        lens = sorted(set().union(*(t[axis].keys() for t in times_by_column)))
        for L in lens:
            c = cands(axis, L)
            ms = {}
            for k, t in enumerate(times_by_column):
                if L in t[axis] and k < len(c):
                    ms[k] = t[axis][L]
            if 0 not in ms:
                continue
            best = min(ms, key=ms.get)
            if ms[best] > ms[0] * (1.0 - margin):
                best = 0
            rad, batch, regx, pads = c[best]
            res[axis][str(L)] = {"radices": rad, "batch": batch, "regx": regx, "pads": pads,
                                 "candidate": best,
                                 "ms": {str(k): round(v, 5) for k, v in ms.items()}}
    return res


# ---------------------------------------------------------------- GPU side
def run_probe(shapes, out_path: Path) -> None:
    """Time each probe stack (runs in a subprocess whose cudadecon_gb300 is
    the scratch copy under test)."""
    import ctypes

    import torch

    import cudadecon_gb300 as cdx
    from cudadecon_gb300 import synth

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    L = cdx.lib()
    stream = torch.cuda.Stream(device=dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    td = tempfile.TemporaryDirectory()
    otf = Path(td.name) / "otf.tif"
    synth.write_otf(otf, synth.gaussian_otf_table(129, 64, 1.5, 4.0))
    rows = []
    for shape in shapes:
        nz, ny, nx = shape
        gen = torch.Generator(device=dev)
        gen.manual_seed(nz * 1000003 + ny * 1009 + nx)
        lam = 100.0 + 3000.0 * (torch.rand(shape, generator=gen, device=dev) < 2e-4).float()
        raw = torch.poisson(lam, generator=gen).clamp_(0, 65535).to(torch.int32).to(torch.uint16)
        cdx.rl_init(shape, otf, dr=0.104, dz=0.3, dr_psf=0.104, dz_psf=0.3)
        grid = list(cdx.decon_grid())
        out = torch.empty(cdx.output_shape(), dtype=torch.float32, device=dev)

        def call():
            if L.cdx_RL_device(ctypes.c_void_p(raw.data_ptr()), nx, ny, nz,
                               ctypes.c_void_p(out.data_ptr()), None, 100.0, False, False, ITERS,
                               0, 0, 0, 0.0, False, False, sp) != 1:
                raise RuntimeError(L.cdx_last_error().decode())

        with torch.cuda.stream(stream):
            call()
            call()
            L.cdx_profile_enable(1)
            call()
            call()
        stream.synchronize()
        pm = (ctypes.c_double * 9)()
        pn = (ctypes.c_longlong * 9)()
        it_ms = ctypes.c_double(0)
        it_n = ctypes.c_longlong(0)
        L.cdx_profile_read(pm, pn, 9, ctypes.byref(it_ms), ctypes.byref(it_n))
        L.cdx_profile_enable(0)
        rows.append({"shape": list(shape), "grid": grid,
                     "pass_ms": [pm[i] / max(pn[i], 1) for i in range(9)]})
        cdx.rl_cleanup()
        del raw, out
    td.cleanup()
    out_path.write_text(json.dumps({"device": torch.cuda.get_device_name(0), "rows": rows}))


def scratch_copy(dst: Path) -> Path:
    """Copy the package sources and the public header into dst."""
    if dst.exists():
        shutil.rmtree(dst)
    ign = shutil.ignore_patterns("lib", "_build", "__pycache__", "*.so", "*.o")
    shutil.copytree(PKG, dst / PKG.name, ignore=ign)
    shutil.copytree(ROOT / "include", dst / "include")
    return dst


def tune(columns: int, margin: float, workdir: Path, apply: bool) -> dict:
    sys.path.insert(0, str(PKG))
    import gen_plans as G

    lens = G.lengths()
    shapes = probe_shapes(lens)
    times = []
    device = None
    for k in range(columns):
        root = scratch_copy(workdir / f"column{k}")
        env = dict(os.environ, PYTHONPATH=str(root))
        py = sys.executable
        res = root / "probe.json"
        (root / "shapes.json").write_text(json.dumps(shapes))
        try:
            subprocess.run([py, str(root / PKG.name / "gen_plans.py"), "--column", str(k)],
                           check=True, env=env)
            subprocess.run([py, "-c", "import cudadecon_gb300 as c; c.build()"], check=True,
                           env=env, cwd=str(root))
            subprocess.run([py, str(root / PKG.name / "autotune.py"), "--probe",
                            str(root / "shapes.json"), str(res)], check=True, env=env,
                           cwd=str(root))
        except subprocess.CalledProcessError as e:
            # a column that does not build or run is left out: its lengths
            # keep the candidates of the other columns
            print(f"column {k}: left out ({e})", flush=True)
            times.append({a: {} for a in AXIS_PASSES})
            continue
        d = json.loads(res.read_text())
        device = d["device"]
        t = axis_times([tuple(r["shape"]) for r in d["rows"]], [r["pass_ms"] for r in d["rows"]],
                       lens)
        times.append(t)
        tot = sum(sum(v.values()) for v in t.values())
        print(f"column {k}: {len(d['rows'])} stacks, {tot:.3f} ms of pass time per iteration",
              flush=True)
    chosen = select(times, G.candidates, margin)
    chosen = {"device": device, "columns": columns, "margin": margin,
              "iterations_per_call": ITERS, **chosen}
    G.TUNED.write_text(json.dumps(chosen, indent=1) + "\n")
    for axis in AXIS_PASSES:
        moved = sum(1 for v in chosen[axis].values() if v["candidate"] != 0)
        print(f"{axis}: {moved} of {len(chosen[axis])} lengths take a candidate other than 0")
    if apply:
        G.generate()
    return chosen


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--columns", type=int, default=None,
                    help="candidate columns to build and time (default: all)")
    ap.add_argument("--margin", type=float, default=0.02)
    ap.add_argument("--workdir", type=Path, default=None)
    ap.add_argument("--no-apply", action="store_true",
                    help="write tuned_plans.json without regenerating the sources")
    ap.add_argument("--probe", nargs=2, metavar=("SHAPES", "OUT"), help=argparse.SUPPRESS)
    a = ap.parse_args()
    if a.probe:
        sys.path.insert(0, str(ROOT))
        run_probe([tuple(s) for s in json.loads(Path(a.probe[0]).read_text())], Path(a.probe[1]))
        return 0
    sys.path.insert(0, str(PKG))
    import gen_plans as G
    cols = a.columns or G.N_COLUMNS
    with tempfile.TemporaryDirectory() as td:
        tune(cols, a.margin, a.workdir or Path(td), not a.no_apply)
    return 0


if __name__ == "__main__":
    sys.exit(main())
