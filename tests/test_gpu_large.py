"""The large enumerations against the oracle's pinned results.

tests/golden/large.json holds the oracle's exact row DP (memory-lean
variant, pinned to the reference's solver on every golden case by
tests/test_oracle.py) on the 8x15 single large enumeration and the 8x10
medium board: tiling counts and the distinct states after every row.  The
engine must reproduce both exactly, and a mirrored board must give the same
count (all 8 transforms allowed).
"""
import json

import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

LARGE = {c["name"]: c for c in json.loads((GOLDEN / "large.json").read_text())["cases"]}


@pytest.fixture(scope="module")
def E(engine):
    if engine.device_count() == 0:
        pytest.fail("no CUDA device visible")
    return engine


def problem(c, rows=None):
    from d4gb.problem import Problem

    return Problem(c["width"], c["height"], list(rows or c["rows"]), c["shapes"], c["counts"],
                   c["sym"], name=c["name"])


def run(E, p):
    f = E.Frow(p.shapes, p.counts, p.sym, p.width, device=0)
    s = E.CudaSearcher(f, rows=p.rows)
    s.run()
    return s.count(), s.level_sizes()


@pytest.mark.parametrize("name", sorted(LARGE))
def test_count_and_rows_match_oracle(E, name):
    c = LARGE[name]
    count, sizes = run(E, problem(c))
    assert count == c["count"]
    assert sizes == c["level_sizes"]


def test_single_large_mirror_has_same_count(E):
    c = LARGE["single large 8x15 seed 3"]
    count, _ = run(E, problem(c, rows=c["rows"][::-1]))
    assert count == c["count"]
