"""Pins the large enumerations' counts with the CPU oracle.

Runs the oracle's exact row DP (the memory-lean variant, which keeps only
each row's distinct states) on the 8x15 single large enumeration
(`d4gb.problem.single_large(3)`: 3 seeded holes, 24 piece copies of 4-6
cells) and on the 8x10 medium board, and writes `tests/golden/large.json`:
the tiling count, the distinct states after every row and the children
produced per row.  The oracle's DP is pinned to the reference's own solver by
`tests/test_oracle.py` on every golden case; the GPU tests then compare the
engine's count and per-row frontier sizes with this file.

Usage: python tests/golden/make_large_golden.py [threads]
(the 8x15 run needs about 25 GB of host memory and some minutes on 8 cores).
"""
from __future__ import annotations

import json
import os
import platform
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO / "d4-pieces_gb300"))
sys.path.insert(0, str(REPO))

from d4gb.problem import medium_board, single_large  # noqa: E402
from oracle import pyoracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "large.json"


def main() -> None:
    threads = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    pyoracle.build()
    cases = []
    for name, p in (("medium 8x10 seed 77", medium_board(77)),
                    ("single large 8x15 seed 3", single_large(3))):
        t = time.time()
        r = pyoracle.rowdp_lean(p, threads=threads)
        print(f"{name}: {r['count']} tilings, peak {max(r['level_sizes'])} states, "
              f"{r['seconds']:.1f} s", flush=True)
        cases.append({
            "name": name,
            "width": p.width, "height": p.height, "rows": p.rows,
            "shapes": p.shapes, "counts": p.counts, "sym": p.sym,
            "count": r["count"],
            "level_sizes": r["level_sizes"],
            "raw_sizes": r["raw_sizes"],
            "oracle_seconds": round(r["seconds"], 1),
            "oracle_threads": threads,
            "host": f"{platform.machine()} x {os.cpu_count()}",
            "wall_s": round(time.time() - t, 1),
        })
    OUT.write_text(json.dumps({"generator": "oracle or_rowdp_lean", "cases": cases},
                              indent=1) + "\n")
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
