"""d4e_count_noalloc: counting without any device allocation.

Callers that cannot call cudaMalloc (a process with a device-memory budget
fixed at start-up, or one running under its own pool allocator) use this
entry point; all its device buffers live in a static array inside the
library.  Here it is called through the C ABI and compared, exactly (integer
counts), with the allocating searcher path on the same puzzles, twice in a row
per puzzle: the second call must not be affected by what the first call left
in the shared array.  The file sorts last so that a run stopping at the first
failure has already run every other test; it also passes alone in a fresh
process.
"""
import pytest

from conftest import case_problem, load_cases

pytestmark = pytest.mark.gpu

CASES = {c["name"]: c for c in load_cases()}
NAMES = ["pentomino ring 8x8-2x2", "random#33", "3x10 pentominoes", "random#19",
         "L-trominoes 6x6 minus 2"]


@pytest.fixture(scope="module")
def E(engine):
    if engine.device_count() == 0:
        pytest.fail("no CUDA device visible")
    return engine


def searcher_count(E, p):
    f = E.Frow(p.shapes, p.counts, p.sym, p.width, device=0)
    s = E.CudaSearcher(f, rows=p.rows)
    s.run()
    return s.count(), s.stats()["states_out"]


@pytest.mark.parametrize("name", NAMES)
def test_noalloc_matches_searcher_twice(E, name):
    p = case_problem(CASES[name])
    want_count, want_states = searcher_count(E, p)
    assert want_count == CASES[name]["count"]
    first = E.count_noalloc(p)
    second = E.count_noalloc(p)
    assert first == (want_count, want_states)
    assert second == (want_count, want_states)


def test_noalloc_alternating_puzzles(E):
    """Back-to-back calls on different puzzles: each result is that
    puzzle's own, whatever the previous call left in the array."""
    a = case_problem(CASES["pentomino ring 8x8-2x2"])
    b = case_problem(CASES["random#33"])
    want_a, want_b = searcher_count(E, a), searcher_count(E, b)
    for _ in range(2):
        assert E.count_noalloc(a) == want_a
        assert E.count_noalloc(b) == want_b


def wide_table_problems(E):
    """8-wide puzzles whose columns hold more than 64 placements, so their
    candidate filters take 2 or 4 words per bitset: the largest tables the
    array has to hold (the 35 hexominoes: 214 placements at column 3)."""
    from d4gb.problem import Problem, single_large

    hexo = E.catalogue(6)
    sl = single_large(3)
    return [
        Problem(8, 3, [0xFF] * 3, hexo, [1] * len(hexo), 0xFF, name="35 hexominoes 8x3"),
        Problem(8, 4, [0xFF] * 4, sl.shapes, [1] * len(sl.shapes), 0xFF,
                name="13 types of the 8x15 set, 8x4"),
        Problem(8, 5, [0xFF, 0xFF, 0xE7, 0xFF, 0xFF], sl.shapes, [1] * len(sl.shapes), 0xFF,
                name="13 types of the 8x15 set, 8x5 minus 2"),
    ]


@pytest.mark.parametrize("which", [0, 1, 2])
def test_noalloc_wide_placement_tables(E, oracle, which):
    """Multi-word candidate filters fit the array and leave the frontier
    buffers after them intact: the count and the states equal the
    searcher's and the oracle's, on two calls in a row."""
    p = wide_table_problems(E)[which]
    f = E.Frow(p.shapes, p.counts, p.sym, p.width, device=None)
    assert max(f.placements(c) for c in range(p.width)) > 64
    want = searcher_count(E, p)
    ref = oracle.rowdp(p, threads=4)
    assert want == (ref["count"], sum(ref["level_sizes"]))
    assert E.count_noalloc(p) == want
    assert E.count_noalloc(p) == want


def test_noalloc_rejects_frontier_beyond_capacity(E):
    from d4gb.problem import medium_board

    big = medium_board(77)          # a row of 18.2M states: beyond the array
    with pytest.raises(E.D4Error) as e:
        E.count_noalloc(big)
    assert e.value.code == -4 and "scratch capacity" in str(e.value)
    ring = case_problem(CASES["pentomino ring 8x8-2x2"])
    assert E.count_noalloc(ring) == searcher_count(E, ring)
