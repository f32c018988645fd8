"""Generates the golden fixtures in tests/golden/ from the reference's own
CPU solver.

Run in a container where the reference sources are present:

    python tests/golden/make_golden.py [REFERENCE_SRC_DIR]

It builds oracle/_ref/d4ref (oracle/Makefile `ref` target: the reference's
src/Piece.cpp, Shape.cpp, Group.cpp, known1.cpp, known2.cpp compiled where
they lie, plus oracle/ref_driver.cpp) and records, for a fixed list of
seeded problems, the reference's solve_count, its full solve() list (type and
step grids, in the reference's order) when small, and solve(single = true).
It also records the reference's polyomino catalogues.  Nothing here runs on
the GPU machine: the fixtures are committed.
"""
from __future__ import annotations

import json
import os
import random
import subprocess
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO / "d4-pieces_gb300"))
sys.path.insert(0, str(REPO))

from d4gb.problem import (FULL_D4, ROTATIONS, Problem, canonical, cells_to_shape,  # noqa: E402
                          merge_pieces)
from oracle import pyoracle  # noqa: E402

OUT = Path(__file__).resolve().parent
MAX_LISTED = 600        # store every solution when there are at most this many
TIMEOUT_S = 8.0


def run_ref(p: Problem, mode: str) -> str:
    lines = [f"{p.width} {p.height} {p.sym} {mode}", " ".join(str(r) for r in p.rows),
             str(len(p.shapes))] + [f"{s} {c}" for s, c in zip(p.shapes, p.counts)]
    r = subprocess.run([str(pyoracle.REF_BIN)], input="\n".join(lines) + "\n",
                       capture_output=True, text=True, timeout=TIMEOUT_S, check=True)
    return r.stdout


def enc(grid) -> str:
    """Compact grid text: one character per cell, chr(48 + value + 1)."""
    return "".join(chr(49 + v) for v in grid)


def parse_solutions(out: str, cells: int):
    lines = out.strip().splitlines()
    n = int(lines[0].split()[1])
    sols = []
    for ln in lines[1:]:
        v = [int(x) for x in ln.split()]
        sols.append((v[:cells], v[cells:2 * cells]))
    return n, sols


def rand_piece(rng: random.Random, size: int) -> int:
    cells = {(0, 0)}
    while len(cells) < size:
        r, c = rng.choice(sorted(cells))
        dr, dc = rng.choice(((0, 1), (0, -1), (1, 0), (-1, 0)))
        cells.add((r + dr, c + dc))
    return canonical(cells_to_shape(cells))


def random_case(rng: random.Random, idx: int) -> Problem:
    W = rng.randint(2, 8)
    H = rng.randint(2, 8 if rng.random() < 0.8 else 11)
    rows = [(1 << W) - 1] * H
    for _ in range(rng.randint(0, 3)):
        h = rng.randrange(W * H)
        rows[h // W] &= ~(1 << (h % W))
    area = sum(bin(r).count("1") for r in rows)
    shapes = []
    while area > 0:
        s = min(area, rng.randint(1, 5))
        shapes.append(rand_piece(rng, s))
        area -= s
    # a few spare pieces make sub-multiset tilings possible
    for _ in range(rng.randint(0, 2)):
        shapes.append(rand_piece(rng, rng.randint(1, 4)))
    types, counts = merge_pieces(shapes)
    sym = rng.choice([FULL_D4, FULL_D4, FULL_D4, ROTATIONS, 0b00000001, 0b00001001, 0b00000011])
    return Problem(W, H, rows, types, counts, sym, name=f"random#{idx}")


def fixed_cases(cat) -> list:
    p5 = cat["free"][5]
    rows = [0xFF] * 8
    rows[3] &= ~0x18 & 0xFF
    rows[4] &= ~0x18 & 0xFF
    ring = Problem(8, 8, rows, p5, [1] * 12, FULL_D4, name="pentomino ring 8x8-2x2")
    # 5x6 board with the six 5-cell pieces that tile it in many ways
    rect = Problem(6, 5, [0x3F] * 5, p5[:8], [1] * 8, FULL_D4, name="5x6 pentomino subset")
    # one-sided tetrominoes on a 4x7 board (C4 only)
    os4 = cat["onesided"][4]
    c4 = Problem(7, 4, [0x7F] * 4, os4, [1] * len(os4), ROTATIONS, name="one-sided tetrominoes 4x7")
    # tall narrow board that needs Shape<11>
    tall = Problem(3, 10, [0x7] * 10, p5, [1] * 12, FULL_D4, name="3x10 pentominoes")
    # dominoes on 4x4 (multiplicity 8)
    dom = Problem(4, 4, [0xF] * 4, [3], [8], FULL_D4, name="dominoes 4x4")
    # L-trominoes with holes
    trom = Problem(6, 6, [0x3F, 0x3F, 0x3B, 0x3F, 0x3F, 0x1F], [259], [11], FULL_D4,
                   name="L-trominoes 6x6 minus 2")
    return [ring, rect, c4, tall, dom, trom]


def main() -> None:
    ref_src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("D4_REFERENCE_SRC", "")
    if not ref_src:
        sys.exit("usage: make_golden.py <reference src dir> (or set D4_REFERENCE_SRC)")
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "ref", f"REF={ref_src}"], check=True)
    cat_out = run_ref(Problem(1, 1, [1], [], [], FULL_D4), "catalogue")
    cat = {"free": {}, "onesided": {}}
    for ln in cat_out.strip().splitlines():
        kind, m, *vals = ln.split()
        cat[kind][int(m)] = [int(v) for v in vals]
    (OUT / "catalogue.json").write_text(json.dumps(cat, indent=0) + "\n")

    rng = random.Random(20241203)
    probs = fixed_cases(cat)
    while len(probs) < 70:
        probs.append(random_case(rng, len(probs)))

    cases = []
    for p in probs:
        try:
            cnt = int(run_ref(p, "count").split()[1])
        except subprocess.TimeoutExpired:
            print("skip (timeout)", p.name)
            continue
        case = {"name": p.name, "width": p.width, "height": p.height, "rows": p.rows,
                "shapes": p.shapes, "counts": p.counts, "sym": p.sym, "count": cnt}
        cells = p.width * p.height
        if cnt <= MAX_LISTED:
            n, sols = parse_solutions(run_ref(p, "all"), cells)
            assert n == cnt
            case["solutions"] = [[enc(t), enc(s)] for t, s in sols]
        n1, one = parse_solutions(run_ref(p, "one"), cells)
        case["first"] = [enc(one[0][0]), enc(one[0][1])] if n1 else None
        cases.append(case)
        print(f"{p.name:32s} {p.width}x{p.height} sym={p.sym:#04x} count={cnt}")
    (OUT / "cases.json").write_text(json.dumps({
        "generator": "tests/golden/make_golden.py",
        "grid_encoding": "one char per cell (row-major), chr(49 + value); value -1 = not on the board",
        "cases": cases}, indent=0) + "\n")
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
