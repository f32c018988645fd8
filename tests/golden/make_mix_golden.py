"""Pins larger instances of the batched mix with the CPU oracle.

The batched-mix tests compare the engine with the oracle on instances the
oracle finishes at once; this script runs the oracle's exact row DP (the
memory-lean variant, pinned to the reference's solver by the golden cases
in tests/test_oracle.py) on larger instances of the same distribution --
`d4gb.problem.batched_mix(2024, 8192)`, the instances of 40..96 cells in
index order -- and keeps those it finishes within a time bound, writing
`tests/golden/mix_large.json` (instance index, board, pieces, tiling count,
distinct states per row).  `tests/test_gpu_batch.py` compares batched counts
with it.

Usage: python tests/golden/make_mix_golden.py [threads] [max_cases] [max_seconds]
"""
from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO / "d4-pieces_gb300"))
sys.path.insert(0, str(REPO))

from d4gb.problem import batched_mix  # noqa: E402
from oracle import pyoracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "mix_large.json"


def main() -> None:
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    max_cases = int(sys.argv[2]) if len(sys.argv) > 2 else 24
    max_seconds = float(sys.argv[3]) if len(sys.argv) > 3 else 20.0
    pyoracle.build()
    cases = []
    for idx, p in enumerate(batched_mix(2024, 8192)):
        if len(cases) >= max_cases:
            break
        if not 40 <= p.cells <= 96:
            continue
        # The probe run bounds the time: the full DP runs only if the first
        # rows' frontier stays small.
        r = pyoracle.rowdp(p, threads=threads, max_seconds=max_seconds,
                           max_children=50_000_000)
        if r["levels_done"] < p.height:
            continue
        t = time.time()
        full = pyoracle.rowdp_lean(p, threads=threads)
        cases.append({"index": idx, "name": p.name, "width": p.width, "height": p.height,
                      "rows": p.rows, "shapes": p.shapes, "counts": p.counts, "sym": p.sym,
                      "cells": p.cells, "count": full["count"],
                      "level_sizes": full["level_sizes"],
                      "oracle_seconds": round(time.time() - t, 2)})
        print(f"#{idx} {p.name} {p.cells} cells: {full['count']} tilings, "
              f"{sum(full['level_sizes'])} states", flush=True)
    OUT.write_text(json.dumps({"generator": "oracle or_rowdp_lean", "seed": 2024,
                               "cases": cases}, indent=1) + "\n")
    print(f"wrote {OUT} ({len(cases)} cases)")


if __name__ == "__main__":
    main()
