"""Generate the compile-time FFT plans for every 2,3,5,7-smooth length of
the batched workloads' stack sizes that the hand-tuned registry in
csrc/static_plans.cuh does not already hold: x in [128, 1024], y in
[128, 512], z in [32, 160].

Writes csrc/static_plans_gen.cuh (the plan lists), csrc/x_gen_dispatch.h
(the dispatch of the x passes) and csrc/decon_x_gen_<k>.cu (the x-pass
kernels of the generated x lengths, spread over several units so that the
build compiles them in parallel).

Plan choice: y and z: two radices of at most 32 points each (in
registers), the most balanced pair, larger radix first; three radices when
no such pair exists (343 = 7*7*7).  x: three radices, the most balanced
triple, smallest last (the fused epilogues of the x passes run in the last
stage, which then has a thread for every butterfly).  Tiles: y passes take
2048 // L rows per block, z passes 16 columns, x passes the generic engine's
row pairs (so the dot-product partials keep their size).  The z pass of
these lengths is compiled for radially averaged OTFs; a full 3D OTF takes
the generic engine.

    python cudadecon_gb300/gen_plans.py     (rewrites the generated files)
"""

from __future__ import annotations

from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "csrc" / "static_plans_gen.cuh"
XDISPATCH = HERE / "csrc" / "x_gen_dispatch.h"
X_UNITS = 12

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


def radices(L: int) -> list[int]:
    best = None
    for a in range(2, 33):
        b, r = divmod(L, a)
        if r == 0 and 2 <= b <= 32 and (best is None or max(a, b) < max(best)):
            best = (max(a, b), min(a, b))
    if best:
        return list(best)
    best3 = None
    for a in range(2, 33):
        if L % a:
            continue
        for b in range(2, 33):
            c, r = divmod(L // a, b)
            if (L // a) % b == 0 and 2 <= c <= 32:
                t = sorted((a, b, c), reverse=True)
                if best3 is None or t[0] < best3[0]:
                    best3 = t
    if best3 is None:
        raise ValueError(f"no plan of radices <= 32 for {L}")
    return best3


def radices3(L: int) -> list[int]:
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


def x_pairs(nx: int) -> int:
    """Row pairs per x tile of the generic engine (x_pairs, decon_common.cuh)."""
    p = min(8, 8192 // nx)
    if nx >= 512:
        p = min(p, 4)
    return max(p, 1)


def x_units(xs: list[int]) -> None:
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
                P = x_pairs(L)
                c = call.replace("PP", str(P))
                out.append(f"    case {L}:")
                out.append("      *done = true;")
                out.append(f"      return {go}<StaticRunner<SPX{L}, {P}, false>>({c}, "
                           f"splan_threads<SPX{L}, {P}>(), st);")
            out += ["    default:", "      return 0;", "  }", "}", ""]
        out += ["}  // namespace cdx", ""]
        (HERE / "csrc" / f"decon_x_gen_{k}.cu").write_text("\n".join(out))


def main() -> None:
    xs = [n for n in range(X_RANGE[0], X_RANGE[1] + 1) if smooth(n) and n not in REGISTERED]
    ys = [n for n in range(Y_RANGE[0], Y_RANGE[1] + 1) if smooth(n) and n not in REGISTERED]
    zs = [n for n in range(Z_RANGE[0], Z_RANGE[1] + 1) if smooth(n) and n not in REGISTERED]
    plans = {}
    for L in sorted(set(ys) | set(zs)):
        plans[L] = radices(L)
    # x lengths have plans of their own (SPX<L>, three radices)
    xplans = {L: radices3(L) for L in xs}
    for L in xs:
        assert x_pairs(L) * L // min(xplans[L]) <= MAX_THREADS, L
    yv = {L: max(1, 2048 // L) for L in ys}
    for L in ys:
        assert yv[L] * L // min(plans[L]) <= MAX_THREADS, L
    for L in zs:
        assert Z_COLS * L // min(plans[L]) <= MAX_THREADS, L
    lines = [
        "// Generated by cudadecon_gb300/gen_plans.py (do not edit): compile-time",
        "// plans for the 2,3,5,7-smooth x lengths in [128, 1024], y lengths in",
        "// [128, 512] and z lengths in [32, 160] outside the hand-tuned registry of",
        "// static_plans.cuh (x plans are types of their own, SPX<L>).",
        "#pragma once",
        "",
        "#define CDX_GEN_SPLANS(F) \\",
    ]
    lines += [f"  F({L}, {', '.join(map(str, r))}) \\" for L, r in plans.items()]
    lines += ["", "#define CDX_GEN_X_SPLANS(F) \\"]
    lines += [f"  F({L}, {', '.join(map(str, r))}) \\" for L, r in xplans.items()]
    lines += ["", "#define CDX_GEN_Y_PLANS(F) \\"]
    lines += [f"  F({L}, {yv[L]}) \\" for L in ys]
    lines += ["", "#define CDX_GEN_Z_PLANS(F) \\"]
    lines += [f"  F({L}, {Z_COLS}) \\" for L in zs]
    lines += [""]
    OUT.write_text("\n".join(lines) + "\n")
    x_units(xs)
    print(f"{OUT}: {len(plans)} y/z plans ({len(ys)} y, {len(zs)} z lengths), {len(xplans)} x plans")


if __name__ == "__main__":
    main()
