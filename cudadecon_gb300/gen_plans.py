"""Generate csrc/static_plans_gen.cuh: compile-time FFT plans for every
2,3,5,7-smooth length of the y range [128, 512] and the z range [32, 160]
(the batched workloads' stack sizes) that the hand-tuned registry in
csrc/static_plans.cuh does not already hold.

Plan choice: two radices of at most 32 points each (in registers), the most
balanced pair, larger radix first; three radices when no such pair exists
(343 = 7*7*7).  Tiles: y passes take 2048 // L rows per block, z passes 16
columns, as the registered plans do.  The y and z kernels of these lengths
then run as compile-time plans (the z pass for radially averaged OTFs; a
full 3D OTF still takes the generic engine).

    python cudadecon_gb300/gen_plans.py     (rewrites the header)
"""

from __future__ import annotations

from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "csrc" / "static_plans_gen.cuh"

REGISTERED = {32, 64, 100, 128, 256, 512, 756, 1024, 1620}
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


def main() -> None:
    ys = [n for n in range(Y_RANGE[0], Y_RANGE[1] + 1) if smooth(n) and n not in REGISTERED]
    zs = [n for n in range(Z_RANGE[0], Z_RANGE[1] + 1) if smooth(n) and n not in REGISTERED]
    plans = {}
    for L in sorted(set(ys) | set(zs)):
        plans[L] = radices(L)
    yv = {L: max(1, 2048 // L) for L in ys}
    for L in ys:
        assert yv[L] * L // min(plans[L]) <= MAX_THREADS, L
    for L in zs:
        assert Z_COLS * L // min(plans[L]) <= MAX_THREADS, L
    lines = [
        "// Generated by cudadecon_gb300/gen_plans.py (do not edit): compile-time",
        "// plans for the 2,3,5,7-smooth y lengths in [128, 512] and z lengths in",
        "// [32, 160] outside the hand-tuned registry of static_plans.cuh.",
        "#pragma once",
        "",
        "#define CDX_GEN_SPLANS(F) \\",
    ]
    lines += [f"  F({L}, {', '.join(map(str, r))}) \\" for L, r in plans.items()]
    lines += ["", "#define CDX_GEN_Y_PLANS(F) \\"]
    lines += [f"  F({L}, {yv[L]}) \\" for L in ys]
    lines += ["", "#define CDX_GEN_Z_PLANS(F) \\"]
    lines += [f"  F({L}, {Z_COLS}) \\" for L in zs]
    lines += [""]
    OUT.write_text("\n".join(lines) + "\n")
    print(f"{OUT}: {len(plans)} plans ({len(ys)} y, {len(zs)} z lengths)")


if __name__ == "__main__":
    main()
