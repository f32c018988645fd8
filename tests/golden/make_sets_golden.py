"""Generates tests/golden/sets.json: piece-set (Sets mode) golden vectors
from the reference's own CPU solver.

Run in a container where the reference sources are present:

    python tests/golden/make_sets_golden.py

For every board below, every multiset of the board's pieces within their
counts that covers the board's cells is passed to the reference's
solve_count (oracle/_ref/d4ref, built from the reference's sources by
oracle/Makefile); the multisets with at least one tiling are recorded with
their counts, sorted by copies.  Boards: the configurations of a small board
family (free 2-4-cell pieces, each at most once) and the golden cases whose
piece counts exceed their board's area.  Nothing here runs on the GPU
machine: the fixture is committed.
"""
from __future__ import annotations

import itertools
import json
import subprocess
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(REPO / "d4-pieces_gb300"))
sys.path.insert(0, str(REPO))

from d4gb import family as F  # noqa: E402
from d4gb.problem import Problem  # noqa: E402
from oracle import pyoracle  # noqa: E402

OUT = Path(__file__).resolve().parent
FAMILY = "\naaab....\naaab....\nccdd....\nccdd....\n"


def ref_count(p: Problem) -> int:
    return int(pyoracle.ref_run(p, "count").split()[1])


def ref_sets(p: Problem):
    areas = [bin(v).count("1") for v in p.shapes]
    out = []
    for copies in itertools.product(*[range(k + 1) for k in p.counts]):
        if sum(a * k for a, k in zip(areas, copies)) != p.cells:
            continue
        n = ref_count(Problem(p.width, p.height, p.rows, p.shapes, list(copies), p.sym))
        if n:
            out.append([list(copies), n])
    return sorted(out)


def main() -> None:
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "ref"], check=True)
    cat = json.loads((OUT / "catalogue.json").read_text())["free"]
    shapes = cat["2"] + cat["3"] + cat["4"]
    fam = F.BoardFamily.from_text(FAMILY)
    boards = []
    for m in sorted(set(fam.configs())):
        p = F.board_problem(m, shapes, [1] * len(shapes))
        boards.append({"name": f"family {m:#x}", "width": p.width, "height": p.height,
                       "rows": p.rows, "shapes": p.shapes, "counts": p.counts, "sym": p.sym,
                       "sets": ref_sets(p)})
    for c in json.loads((OUT / "cases.json").read_text())["cases"]:
        p = Problem(c["width"], c["height"], c["rows"], c["shapes"], c["counts"], c["sym"])
        n_multisets = 1
        for k in c["counts"]:
            n_multisets *= k + 1
        if c["width"] > 8 or p.piece_area <= p.cells or n_multisets > 4096 or \
                not 0 < c["count"] < 10 ** 6:
            continue
        boards.append({"name": c["name"], "width": p.width, "height": p.height, "rows": p.rows,
                       "shapes": p.shapes, "counts": p.counts, "sym": p.sym,
                       "sets": ref_sets(p)})
    (OUT / "sets.json").write_text(json.dumps({
        "generator": "tests/golden/make_sets_golden.py",
        "family": FAMILY, "family_pieces": "free 2-4-cell pieces, catalogue order, 1 each",
        "boards": boards}, separators=(",", ":")) + "\n")
    print(len(boards), "boards,", sum(len(b["sets"]) for b in boards), "sets")


if __name__ == "__main__":
    main()
