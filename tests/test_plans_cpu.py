"""The generated compile-time plans and their autotuner, on the CPU.

* Every candidate plan of every length multiplies out to the length, keeps
  its radices within 32 points and its block within 1024 threads, and a
  two-radix x plan's padded middle array fits the row tile.
* Candidate 0 is the heuristic choice (the plan used without tuning).
* The committed generated sources are what gen_plans.py writes from the
  committed tuned_plans.json (or candidate 0 without one).
* The tuner's probe stacks cover every length on its axis, and its selection
  keeps candidate 0 unless another is faster by more than the margin.
"""

import json
import math
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "cudadecon_gb300"
sys.path.insert(0, str(PKG))
import autotune as T  # noqa: E402
import gen_plans as G  # noqa: E402


def test_candidates_are_valid_plans():
    lens = G.lengths()
    assert len(lens["x"]) == 86 and len(lens["y"]) == 51 and len(lens["z"]) == 33
    for axis, ls in lens.items():
        for L in ls:
            c = G.candidates(axis, L)
            assert c, (axis, L)
            for rad, batch, regx, pads in c:
                assert regx in (0, G.REGX)
                assert all(b in G.PAD_CHOICES for b in pads)
                assert pads == [0, 0] or (len(rad) == 3 and axis != "z")
                assert math.prod(rad) == L and max(rad) <= 32 and min(rad) >= 2
                assert batch >= 1 and G.threads(L, rad, batch) <= G.MAX_THREADS
                if axis == "x":
                    assert G.x_fits(L, rad, batch)
            assert len({(tuple(r), b, x, tuple(p)) for r, b, x, p in c}) == len(c)
            assert len(c) <= G.N_COLUMNS


def test_candidate_zero_is_the_heuristic():
    for L in G.lengths()["x"]:
        r = G.radices3(L)
        assert G.candidates("x", L)[0] == (r, G.x_pairs(L), 0, [0, 0])
        r = G.candidates("x", L)[0][0]
        assert r == sorted(r, reverse=True)
    for L in G.lengths()["y"]:
        r, V = G.radices(L), max(1, 2048 // L)
        assert G.candidates("y", L)[0] == (r, V, 0, [0, 0])
    for L in G.lengths()["z"]:
        assert G.candidates("z", L)[0] == (G.radices(L), G.Z_COLS, 0, [0, 0])


def test_choose_follows_a_tuned_table_only_for_known_candidates():
    L = 600
    c = G.candidates("x", L)
    assert len(c) > 1
    tuned = {"x": {"600": {"radices": c[1][0], "batch": c[1][1], "regx": c[1][2],
                           "pads": c[1][3]}}}
    assert G.choose("x", L, None, tuned) == c[1]
    bogus = {"x": {"600": {"radices": [600], "batch": 1}}}
    assert G.choose("x", L, None, bogus) == c[0]
    assert G.choose("x", L, 99, {}) == c[0]


def test_committed_sources_match_the_generator(tmp_path, monkeypatch):
    (tmp_path / "csrc").mkdir()
    monkeypatch.setattr(G, "HERE", tmp_path)
    monkeypatch.setattr(G, "OUT", tmp_path / "csrc" / "static_plans_gen.cuh")
    monkeypatch.setattr(G, "XDISPATCH", tmp_path / "csrc" / "x_gen_dispatch.h")
    if (PKG / "tuned_plans.json").exists():
        (tmp_path / "tuned_plans.json").write_text((PKG / "tuned_plans.json").read_text())
    monkeypatch.setattr(G, "TUNED", tmp_path / "tuned_plans.json")
    G.generate()
    names = ["static_plans_gen.cuh", "x_gen_dispatch.h"] + \
        [f"decon_x_gen_{k}.cu" for k in range(G.X_UNITS)]
    for n in names:
        assert (tmp_path / "csrc" / n).read_text() == (PKG / "csrc" / n).read_text(), n


def test_bank_model_counts_known_patterns():
    # 16 threads at stride 10 float2s: two threads per bank pair -> 2
    # wavefronts per half-warp; stride 1 -> 1
    a = np.arange(32) * 10
    assert G._wavefronts64(a.reshape(1, 32)) == 4
    assert G._wavefronts64(np.arange(32).reshape(1, 32)) == 2
    assert G._wavefronts64(np.full((1, 32), -1)) == 0
    # 1008 = 12*12*7 after its first stage: 16-byte pairs at stride 6 float4s
    # still meet twice on a bank; padding every 48 lowers the model further
    nat = G.boundary_wavefronts(1008, [12, 12, 7], 4, 0, 0)
    pad = G.boundary_wavefronts(1008, [12, 12, 7], 4, 0, 48)
    assert pad < 0.8 * nat
    # radix 8 first: even as 16-byte pairs its stride-8 stores put four
    # threads of a quarter-warp on a bank; padding every 16 halves that
    assert G.boundary_wavefronts(392, [8, 7, 7], 8, 0, 16) < \
        0.6 * G.boundary_wavefronts(392, [8, 7, 7], 8, 0, 0)
    assert G.smem_pads(392, [8, 7, 7], 8) == [16, 0]
    assert G.smem_pads(600, [10, 10, 6], 4) == [0, 0]
    assert G.smem_pads(600, [24, 25], 4) == [0, 0]
    # 16-byte pairs at stride 5 float4s: conflict-free
    assert G._wavefronts128((np.arange(32) * 5).reshape(1, 32)) == 4


def test_probe_shapes_cover_every_length():
    lens = G.lengths()
    shapes = T.probe_shapes(lens)
    assert len(shapes) == max(len(v) for v in lens.values())
    for i, axis in enumerate("zyx"):
        assert {s[i] for s in shapes} == set(lens[axis])


def test_select_keeps_candidate_zero_within_the_margin():
    lens = {"x": [600], "y": [320], "z": [120]}
    shapes = [(120, 320, 600)]
    base = [0.07, 0.03, 0.05, 0.03, 0.11, 0.03, 0.05, 0.03, 0.10]
    faster_x = list(base)
    faster_x[4] = 0.08            # column 1: x ratio 30 us faster
    slower_y = list(base)
    slower_y[1] = 0.0299          # column 2: y within the margin
    cols = [T.axis_times(shapes, [pm], lens) for pm in (base, faster_x, slower_y)]
    assert cols[0]["x"][600] == pytest.approx(0.07 + 0.11 + 0.10)
    assert cols[0]["y"][320] == pytest.approx(0.12)
    sel = T.select(cols, G.candidates, 0.02)
    assert sel["x"]["600"]["candidate"] == 1
    got = sel["x"]["600"]
    assert (got["radices"], got["batch"], got["regx"], got["pads"]) == G.candidates("x", 600)[1]
    assert sel["y"]["320"]["candidate"] == 0
    assert sel["z"]["120"]["candidate"] == 0
    json.dumps(sel)


def test_select_ignores_a_column_left_out():
    """A tuning column that failed to build or run contributes no times;
    the others still decide."""
    lens = {"x": [600], "y": [320], "z": [120]}
    shapes = [(120, 320, 600)]
    base = [0.07, 0.03, 0.05, 0.03, 0.11, 0.03, 0.05, 0.03, 0.10]
    faster = list(base)
    faster[4] = 0.08
    cols = [T.axis_times(shapes, [base], lens), {a: {} for a in T.AXIS_PASSES},
            T.axis_times(shapes, [faster], lens)]
    sel = T.select(cols, G.candidates, 0.02)
    assert sel["x"]["600"]["candidate"] == 2
    assert "1" not in sel["x"]["600"]["ms"]
