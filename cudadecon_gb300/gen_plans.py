"""Generate the compile-time FFT plans for every 2,3,5,7-smooth length of
the batched workloads' stack sizes that the hand-tuned registry in
csrc/static_plans.cuh does not already hold: x in [128, 1024], y in
[128, 512], z in [32, 160].

Writes csrc/static_plans_gen.cuh (the plan lists), csrc/x_gen_dispatch.h
(the dispatch of the x passes) and csrc/decon_x_gen_<k>.cu (the x-pass
kernels of the generated x lengths, spread over several units so that the
build compiles them in parallel).

Each length has a short list of candidate plans (radix order, pencil batch
-- rows, row pairs or columns per block -- the register budget behind the
launch bounds, and for three-radix row plans the padding of the layouts
between the stages); candidate 0 is the heuristic choice:

  y, z : the most balanced pair of radices of at most 32 points (in
         registers), larger radix first; three radices when no such pair
         exists (343 = 7*7*7).  y blocks take 2048 // L rows, z blocks 16
         columns.  Candidates: half the rows (or 8 columns), the reversed
         radix order, twice the rows (or 32 columns) where the block stays
         within 1024 threads, 16 more registers per thread, and three
         radices (the most balanced triple) with the full and half batch:
         an unbalanced pair such as 125 = 25*5 leaves most threads idle in
         its large-radix stage.
  x    : the most balanced three radices, smallest last (the fused epilogues
         of the x passes run in the last stage, which then has a thread for
         every butterfly), with the generic engine's row pairs per block.
         Candidates: half the row pairs, the two larger radices swapped, the
         most balanced two-radix plan where its padded middle array fits the
         tile, 16 more registers per thread, a quarter of the row pairs, and
         the swapped radices with half the row pairs.

Padding (x and y plans of three radices): each layout between two stages
can get one float2 of padding after every B, with B in PAD_CHOICES picked
by a model of the shared-memory bank conflicts of the stage that writes it
and the stage that reads it (smem_pads); one candidate per length carries
the model's padding where the model finds one.

autotune.py times the candidates on the GPU and records the fastest per
axis and length in tuned_plans.json, which this script then follows.

    python cudadecon_gb300/gen_plans.py               (tuned, else candidate 0)
    python cudadecon_gb300/gen_plans.py --column k    (candidate k everywhere,
                                                       for the tuning builds)
"""

from __future__ import annotations

import argparse
import functools
import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "csrc" / "static_plans_gen.cuh"
XDISPATCH = HERE / "csrc" / "x_gen_dispatch.h"
TUNED = HERE / "tuned_plans.json"
X_UNITS = 12
N_COLUMNS = 8
REGX = 16
PAD_CHOICES = (0, 16, 32, 64, 128)
PAD_MIN_GAIN = 0.7

REGISTERED = {32, 64, 100, 128, 256, 512, 756, 1024, 1620}
X_RANGE = (128, 1024)
Y_RANGE = (128, 512)
Z_RANGE = (32, 160)
Z_COLS = 16
MAX_THREADS = 1024


def smooth(n: int) -> bool:
    for p in (2, 3, 5, 7):
        while n % p == 0:
            n //= p
    return n == 1


def lengths() -> dict[str, list[int]]:
    def rng(r):
        return [n for n in range(r[0], r[1] + 1) if smooth(n) and n not in REGISTERED]
    return {"x": rng(X_RANGE), "y": rng(Y_RANGE), "z": rng(Z_RANGE)}


def radices2(L: int) -> list[int] | None:
    """The most balanced pair of radices <= 32 (larger first), or None."""
    best = None
    for a in range(2, 33):
        b, r = divmod(L, a)
        if r == 0 and 2 <= b <= 32 and (best is None or max(a, b) < max(best)):
            best = (max(a, b), min(a, b))
    return list(best) if best else None


def radices3(L: int) -> list[int]:
    """The most balanced triple of radices <= 32, in descending order."""
    best = None
    for a in range(2, 33):
        if L % a:
            continue
        for b in range(2, 33):
            c, r = divmod(L // a, b)
            if (L // a) % b == 0 and 2 <= c <= 32:
                t = sorted((a, b, c), reverse=True)
                key = (t[0], -t[2])
                if best is None or key < best[0]:
                    best = (key, t)
    if best is None:
        raise ValueError(f"no three-radix plan for {L}")
    return best[1]


def radices(L: int) -> list[int]:
    """y/z plans: a pair where one exists, else three radices."""
    return radices2(L) or radices3(L)


def x_pairs(nx: int) -> int:
    """Row pairs per x tile of the generic engine (x_pairs, decon_common.cuh)."""
    p = min(8, 8192 // nx)
    if nx >= 512:
        p = min(p, 4)
    return max(p, 1)


def threads(L: int, rad: list[int], batch: int) -> int:
    """Threads of a block (splan_threads, fft_static.cuh)."""
    t = batch * (L // min(rad))
    return (t + 31) // 32 * 32


def spad_size(n: int) -> int:
    return n + (n >> 4) + 1


def x_fits(L: int, rad: list[int], P: int) -> bool:
    """A two-radix plan's padded middle array must fit the padded row tile
    the x launchers allocate (splan_rows_fit, fft_static.cuh)."""
    if threads(L, rad, P) > MAX_THREADS:
        return False
    if len(rad) == 2:
        return P * rad[1] * (rad[0] + 1) <= spad_size(P * L)
    return True


def _wavefronts64(addr: np.ndarray) -> int:
    """Shared-memory wavefronts of 8-byte accesses: addr (..., 32) float2
    indices of one warp's threads (-1: inactive); each half-warp is one
    request whose wavefronts are the most distinct words on one bank."""
    a = addr.reshape(-1, 16)
    act = np.concatenate([a >= 0, a >= 0], axis=1)
    words = np.where(act, np.concatenate([2 * a, 2 * a + 1], axis=1), -1)
    words.sort(axis=1)
    uniq = np.ones_like(words, dtype=bool)
    uniq[:, 1:] = words[:, 1:] != words[:, :-1]
    uniq &= words >= 0
    g = np.broadcast_to(np.arange(words.shape[0])[:, None], words.shape)
    cnt = np.zeros((words.shape[0], 32), dtype=np.int64)
    np.add.at(cnt, (g[uniq], words[uniq] % 32), 1)
    return int(cnt.max(axis=1).sum())


def _wavefronts128(addr: np.ndarray) -> int:
    """Wavefronts of 16-byte accesses: addr (..., 32) float4 indices (-1:
    inactive); each quarter-warp is one request."""
    a = addr.reshape(-1, 8)
    act = np.concatenate([a >= 0] * 4, axis=1)
    words = np.where(act, np.concatenate([4 * a + i for i in range(4)], axis=1), -1)
    words.sort(axis=1)
    uniq = np.ones_like(words, dtype=bool)
    uniq[:, 1:] = words[:, 1:] != words[:, :-1]
    uniq &= words >= 0
    g = np.broadcast_to(np.arange(words.shape[0])[:, None], words.shape)
    cnt = np.zeros((words.shape[0], 32), dtype=np.int64)
    np.add.at(cnt, (g[uniq], words[uniq] % 32), 1)
    return int(cnt.max(axis=1).sum())


def boundary_wavefronts(L: int, rad: list[int], V: int, s: int, B: int) -> int:
    """Wavefronts of the stores of stage s and the loads of stage s + 1 of a
    row plan (sstage in fft_static.cuh: thread b owns butterfly j of vector
    v; loads at j + r L/Q, stores at (j - k) Q + k + r Ns with k = j mod
    Ns) through the layout padded every B float2s.  The first stage's stores
    into the natural layout (B = 0) go out as 16-byte pairs when its radix is
    even (sstage's pair path)."""
    T = threads(L, rad, V)
    b = np.arange(T)
    ns = int(np.prod(rad[:s])) if s else 1
    tot = 0
    for kind, Q, nsk in (("st", rad[s], ns), ("ld", rad[s + 1], ns * rad[s])):
        LR = L // Q
        v, j = np.divmod(b, LR)
        if kind == "st" and nsk == 1 and Q % 2 == 0 and B == 0:
            r2 = np.arange(0, Q, 2)[:, None]
            t = (v[None, :] * L + j[None, :] * Q + r2) // 2
            t = np.where(b[None, :] < V * LR, t, -1)
            tot += _wavefronts128(t.reshape(len(r2), -1, 32))
            continue
        r = np.arange(Q)[:, None]
        if kind == "ld":
            e = j[None, :] + r * LR
        else:
            k = j % nsk
            e = ((j - k) * Q + k)[None, :] + r * nsk
        t = v[None, :] * L + e
        if B:
            t = t + t // B
        t = np.where(b[None, :] < V * LR, t, -1)
        tot += _wavefronts64(t.reshape(Q, -1, 32))
    return tot


def smem_pads(L: int, rad: list[int], V: int) -> list[int]:
    """Padding periods (powers of two: the padded index is a shift and an
    add) of the two layouts between the stages of a three-radix row plan:
    per boundary the fewest modelled wavefronts, kept where they save a
    quarter of that boundary's, and none at all unless the plan's two
    boundaries together drop below PAD_MIN_GAIN of the natural layout's.
    Measured on the GB300 against float2 stores in the natural layout:
    plans whose model dropped below half ran 5-13% faster padded (radix 8
    first, B = 16); those between 0.58 and 0.97 ran up to 8% slower.  The
    first stage now stores 16-byte pairs into the natural layout, which
    removes most of what the padding did, so the padded plan is one
    candidate among the others for the tuner to measure."""
    return list(_smem_pads(L, tuple(rad), V))


@functools.lru_cache(maxsize=None)
def _smem_pads(L: int, rad: tuple[int, ...], V: int) -> tuple[int, int]:
    if len(rad) != 3:
        return (0, 0)
    nat = [boundary_wavefronts(L, list(rad), V, s, 0) for s in range(2)]
    pads, cost = [], []
    for s in range(2):
        c = {B: boundary_wavefronts(L, list(rad), V, s, B) for B in PAD_CHOICES}
        best = min(c, key=lambda B: (c[B], B))
        if c[best] > 0.75 * nat[s]:
            best = 0
        pads.append(best)
        cost.append(c[best])
    # the padded index costs instructions of its own: pad only where the
    # model removes more than PAD_MIN_GAIN of the two boundaries' wavefronts
    if sum(cost) > PAD_MIN_GAIN * sum(nat):
        return (0, 0)
    return tuple(pads)


def candidates(axis: str, L: int) -> list[tuple[list[int], int, int, list[int]]]:
    """Candidate (radices, batch, extra registers, paddings) of one length,
    candidate 0 first."""
    out: list[tuple[list[int], int, int, list[int]]] = []

    def add(rad, b, rx=0, padded=False):
        rad = list(rad)
        if axis == "x" and not x_fits(L, rad, b):
            return
        if axis != "x" and threads(L, rad, b) > MAX_THREADS:
            return
        pads = smem_pads(L, rad, b) if padded and axis != "z" else [0, 0]
        if padded and pads == [0, 0]:
            return
        c = (rad, b, rx, pads)
        if c not in out:
            out.append(c)

    if axis == "x":
        base, P = radices3(L), x_pairs(L)
        swapped = [base[1], base[0], base[2]]
        add(base, P)
        add(base, max(1, P // 2))
        add(swapped, P)
        pair = radices2(L)
        if pair:
            add(pair, P)
        add(base, P, REGX)
        add(base, max(1, P // 4))
        add(swapped, max(1, P // 2))
        add(base, max(1, P // 2), padded=True)
    else:
        base = radices(L)
        b = max(1, 2048 // L) if axis == "y" else Z_COLS
        add(base, b)
        add(base, max(1, b // 2))
        add(list(reversed(base)), b)
        add(base, 2 * b)
        add(base, b, REGX)
        if len(base) == 2:
            try:
                tri = radices3(L)
            except ValueError:
                tri = None
            if tri:
                add(tri, b)
                add(tri, max(1, b // 2))
                add(tri, b, padded=True)
    assert out, f"no plan within {MAX_THREADS} threads for {axis} length {L}"
    return out


def choose(axis: str, L: int, column: int | None,
           tuned: dict) -> tuple[list[int], int, int, list[int]]:
    c = candidates(axis, L)
    if column is not None:
        return c[column] if column < len(c) else c[0]
    t = tuned.get(axis, {}).get(str(L))
    if t:
        pick = (t["radices"], t["batch"], t.get("regx", 0), t.get("pads", [0, 0]))
        if pick in c:
            return pick
    return c[0]


def x_units(xs: list[int], xplans: dict) -> None:
    units = [xs[k::X_UNITS] for k in range(X_UNITS)]
    kinds = {
        "fwd": ("const float* X, float* Xm1, const float* lam, int predict, float2* S",
                "x_fwd_go", "g, fx.gxdev, X, Xm1, lam, predict, S, PP"),
        "ratio": ("float2* S, const float* raw, float eps",
                  "x_ratio_go", "g, fx.gxdev, S, raw, eps, PP"),
        "update": ("const float2* S, const float* Y, float* Xout, float* G, int dots, RLWork& w, "
                   "float* lam_next, float eps",
                   "x_update_go", "g, fx.gxdev, S, Y, Xout, G, dots, w, lam_next, eps, PP"),
    }
    decl, disp = [], []
    for kind, (args, go, call) in kinds.items():
        sig = f"(const Geom& g, const FftLen& fx, {args}, cudaStream_t st, bool* done)"
        for k in range(X_UNITS):
            decl.append(f"int xgen_{kind}_{k}{sig};")
        names = [a.split()[-1].lstrip("*&") for a in args.split(", ")]
        fwdargs = ", ".join(["g", "fx"] + names + ["st", "done"])
        body = "\n".join(f"  if ((rc = xgen_{kind}_{k}({fwdargs})) || *done) return rc;"
                         for k in range(X_UNITS))
        disp.append(f"inline int xgen_{kind}{sig} {{\n  int rc = 0;\n  *done = false;\n{body}\n"
                    f"  return 0;\n}}")
    XDISPATCH.write_text(
        "// Generated by cudadecon_gb300/gen_plans.py (do not edit): dispatch of the\n"
        "// x passes of the generated x lengths to the units decon_x_gen_<k>.cu.\n"
        "// Each function sets *done when its length has a generated plan.\n"
        "#pragma once\n\n#include \"kernels.h\"\n\nnamespace cdx {\n\n" + "\n".join(decl) +
        "\n\n" + "\n\n".join(disp) + "\n\n}  // namespace cdx\n")
    for k, lens in enumerate(units):
        out = ["// Generated by cudadecon_gb300/gen_plans.py (do not edit): x-pass kernels",
               f"// of the generated x lengths {', '.join(map(str, lens))}.",
               '#include "decon_x_kernels.cuh"', '#include "x_gen_dispatch.h"', "",
               "namespace cdx {", ""]
        for kind, (args, go, call) in kinds.items():
            out.append(f"int xgen_{kind}_{k}(const Geom& g, const FftLen& fx, {args}, "
                       f"cudaStream_t st, bool* done) {{")
            out.append("  switch (g.nx) {")
            for L in lens:
                _, P, rx, (b0, b1) = xplans[L]
                c = call.replace("PP", str(P))
                out.append(f"    case {L}:")
                out.append("      *done = true;")
                out.append(f"      return {go}<StaticRunner<SPX{L}, {P}, false, false, {rx}, {b0}, "
                           f"{b1}>>({c}, splan_threads<SPX{L}, {P}>(), st);")
            out += ["    default:", "      return 0;", "  }", "}", ""]
        out += ["}  // namespace cdx", ""]
        (HERE / "csrc" / f"decon_x_gen_{k}.cu").write_text("\n".join(out))


def generate(column: int | None = None) -> dict:
    """Write the generated sources; returns the chosen plans per axis."""
    tuned = json.loads(TUNED.read_text()) if column is None and TUNED.exists() else {}
    lens = lengths()
    plans = {a: {L: choose(a, L, column, tuned) for L in lens[a]} for a in lens}
    src = "tuned_plans.json" if tuned else ("candidate column %d" % column if column is not None
                                             else "candidate 0")
    lines = [
        "// Generated by cudadecon_gb300/gen_plans.py (do not edit): compile-time",
        "// plans for the 2,3,5,7-smooth x lengths in [128, 1024], y lengths in",
        "// [128, 512] and z lengths in [32, 160] outside the hand-tuned registry of",
        "// static_plans.cuh; x plans are types SPX<L>, z plans SPZ<L>, y plans",
        f"// SP<L>.  Plans from {src}.",
        "#pragma once",
        "",
    ]

    def block(name, items):
        return [f"#define {name}(F) \\"] + [f"  F({i}) \\" for i in items] + [""]

    lines += block("CDX_GEN_SPLANS", [f"{L}, {', '.join(map(str, c[0]))}"
                                      for L, c in plans["y"].items()])
    lines += block("CDX_GEN_Z_SPLANS", [f"{L}, {', '.join(map(str, c[0]))}"
                                        for L, c in plans["z"].items()])
    lines += block("CDX_GEN_X_SPLANS", [f"{L}, {', '.join(map(str, c[0]))}"
                                        for L, c in plans["x"].items()])
    lines += block("CDX_GEN_X_PAIRS", [f"{L}, {c[1]}" for L, c in plans["x"].items()])
    lines += block("CDX_GEN_Y_PLANS", [f"{L}, {c[1]}, {c[2]}, {c[3][0]}, {c[3][1]}"
                                       for L, c in plans["y"].items()])
    lines += block("CDX_GEN_Z_PLANS", [f"{L}, {c[1]}, {c[2]}" for L, c in plans["z"].items()])
    OUT.write_text("\n".join(lines) + "\n")
    x_units(lens["x"], plans["x"])
    return plans


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--column", type=int, default=None,
                    help="use candidate COLUMN for every length (tuning builds)")
    a = ap.parse_args()
    plans = generate(a.column)
    print(f"{OUT}: {len(plans['y'])} y, {len(plans['z'])} z and {len(plans['x'])} x plans")


if __name__ == "__main__":
    main()
