"""GPU parity: the engine (through its C ABI) against the reference's golden
vectors and the CPU oracle.  Integer work, so every comparison is exact."""
import numpy as np
import pytest

from conftest import case_problem, decode_grid, load_cases

pytestmark = pytest.mark.gpu

CASES = [c for c in load_cases() if c["width"] <= 8]


@pytest.fixture(scope="module")
def E(engine):
    if engine.device_count() == 0:
        pytest.fail("no CUDA device visible")
    return engine


def gpu_count(E, p, keep_levels=False):
    f = E.Frow(p.shapes, p.counts, p.sym, p.width, device=0)
    s = E.CudaSearcher(f, rows=p.rows, keep_levels=keep_levels)
    s.run()
    return s, s.count()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_count_matches_reference(E, case):
    p = case_problem(case)
    _, n = gpu_count(E, p)
    assert n == case["count"]


@pytest.mark.parametrize("case", CASES[:24], ids=[c["name"] for c in CASES[:24]])
def test_level_sizes_match_oracle_rowdp(E, oracle, case):
    p = case_problem(case)
    s, n = gpu_count(E, p)
    ref = oracle.rowdp(p, threads=2)
    got = s.level_sizes()
    # the engine stops early once a frontier is empty
    assert got == ref["level_sizes"][: len(got)]
    assert all(v == 0 for v in ref["level_sizes"][len(got):])
    assert n == ref["count"]


def test_reference_style_empty_area_searcher(E):
    ring = next(c for c in CASES if c["name"].startswith("pentomino ring"))
    p = case_problem(ring)
    f = E.Frow(p.shapes, p.counts, p.sym, 8, device=0)
    s = E.CudaSearcher(f, empty_area=p.empty_area())
    heights = []
    while s.get_height():
        heights.append(s.get_height())
        assert s.size() >= 1
        assert s.next_size() >= 1
        s.search_GPU()
    assert heights == list(range(8, 0, -1))
    assert s.count() == 520
    st = s.stats()
    assert st["rows"] == 8 and st["states_out"] == 961612


def test_bucket_sizes_partition_the_frontier(E):
    ring = next(c for c in CASES if c["name"].startswith("pentomino ring"))
    p = case_problem(ring)
    f = E.Frow(p.shapes, p.counts, p.sym, 8, device=0)
    s = E.CudaSearcher(f, empty_area=p.empty_area())
    s.search_GPU()
    s.search_GPU()
    total = s.size()
    assert sum(s.size(b) for b in range(256)) == total


LISTED = [c for c in CASES if "solutions" in c and c["count"] > 0]


@pytest.mark.parametrize("case", LISTED, ids=[c["name"] for c in LISTED])
def test_solution_sets_match_reference(E, case):
    p = case_problem(case)
    s, n = gpu_count(E, p, keep_levels=True)
    assert n == case["count"]
    tg, sg = s.solutions(n + 5)
    assert len(tg) == n
    got = {(a.tobytes(), b.tobytes()) for a, b in zip(tg, sg)}
    want = {(decode_grid(t, p.width, p.height).tobytes(), decode_grid(st, p.width, p.height).tobytes())
            for t, st in case["solutions"]}
    assert got == want


def test_pentomino_ring_canonical_65(E, oracle):
    ring = next(c for c in CASES if c["name"].startswith("pentomino ring"))
    p = case_problem(ring)
    s, n = gpu_count(E, p, keep_levels=True)
    tg, _ = s.solutions(1000)
    assert n == len(tg) == 520
    canon = {E.canonical_grid(p, g).tobytes() for g in tg}
    assert len(canon) == 65
    want = {oracle.canonical_grid(p, decode_grid(t, 8, 8)).tobytes() for t, _ in ring["solutions"]}
    assert canon == want


ONE = [c for c in CASES if c["first"] is not None]


@pytest.mark.parametrize("case", ONE[:30], ids=[c["name"] for c in ONE[:30]])
def test_solve_one_is_a_valid_tiling(E, oracle, case):
    p = case_problem(case)
    s, n = gpu_count(E, p, keep_levels=True)
    tg, sg = s.solutions(1, single=True)
    assert len(tg) == 1
    types, masks = oracle.grid_to_placements(p, tg[0], sg[0])
    assert oracle.check_tiling(p, types, masks)


def test_unsolvable_instances_report_zero(E):
    from d4gb.problem import Problem

    # 5 cells, only a domino and a tromino-sized area mismatch
    p = Problem(5, 1, [0x1F], [3], [1], 0xFF)
    assert gpu_count(E, p)[1] == 0
    # a board with no cells is tiled exactly once (by nothing)
    p = Problem(4, 3, [0, 0, 0], [3], [2], 0xFF)
    assert gpu_count(E, p)[1] == 1


def test_batch_equals_alone(E):
    """Each instance's count is the same alone (sequential, one launch
    sequence per puzzle) and in the mixed batch (one launch pair per row for
    all puzzles)."""
    probs = [case_problem(c) for c in CASES if c["count"] < 10 ** 6][:40]
    want = [c["count"] for c in CASES if c["count"] < 10 ** 6][:40]
    mixed, st_m = E.batch_count(probs)
    alone, st_a = E.batch_count(probs, sequential=True)
    assert mixed == want
    assert alone == want
    assert st_m["expand_launches"] < st_a["expand_launches"]


def test_batched_mix_matches_oracle(E, oracle):
    """Batched-mix instances small enough for the CPU row DP (<= 36 cells)
    against the oracle, counted in one mixed batch."""
    from d4gb.problem import batched_mix

    probs = [p for p in batched_mix(5, 400) if p.cells <= 36][:24]
    assert len(probs) >= 8
    got, _ = E.batch_count(probs)
    for p, g in zip(probs, got):
        assert g == oracle.rowdp(p, threads=4)["count"], p.name


def test_batched_mix_flip_invariance(E):
    """Batched-mix instances beyond the CPU oracle's reach (37..48 cells):
    each count equals its mirrored board's count (all 8 transforms allowed),
    in one batch of 2 x 32 puzzles."""
    from d4gb.problem import Problem, batched_mix

    probs = [p for p in batched_mix(9, 600) if 37 <= p.cells <= 48][:32]
    flipped = [Problem(p.width, p.height, p.rows[::-1], p.shapes, p.counts, p.sym) for p in probs]
    got, _ = E.batch_count(probs + flipped)
    assert got[:32] == got[32:]


def test_d4_invariance_on_tall_board(E):
    """Size-independent property: a board and its mirror images have the same
    number of tilings when all 8 transforms are allowed (8 x 10 board, 16
    random 4..6-cell pieces of exactly the board's area)."""
    from d4gb.problem import Problem, medium_board

    p = medium_board(77)
    rows, types, counts = p.rows, p.shapes, p.counts
    n = gpu_count(E, p)[1]
    flip_y = Problem(8, 10, rows[::-1], types, counts, 0xFF)
    flip_x = Problem(8, 10, [int(f"{r:08b}"[::-1], 2) for r in rows], types, counts, 0xFF)
    assert gpu_count(E, flip_y)[1] == n
    assert gpu_count(E, flip_x)[1] == n
    assert n == 4952290238   # computed once by the oracle's row DP (237 s on 8 threads)


def test_width_one_to_eight(E, oracle):
    from d4gb.problem import Problem

    for w in range(1, 9):
        p = Problem(w, 6, [(1 << w) - 1] * 6, [1, 3, 7, 259], [6, 4, 2, 2], 0xFF)
        want = oracle.rowdp(p, threads=2)["count"]
        assert gpu_count(E, p)[1] == want, w


def test_many_copies_and_limits(E, oracle):
    from d4gb.problem import Problem

    p = Problem(8, 5, [0xFF] * 5, [3], [20], 0xFF)     # dominoes, 20 copies
    assert gpu_count(E, p)[1] == oracle.rowdp(p)["count"]
    p = Problem(8, 5, [0xFF] * 5, [1, 3], [20, 20], 0xFF)  # 40 copies
    assert gpu_count(E, p)[1] == oracle.rowdp(p)["count"]
    p = Problem(8, 8, [0xFF] * 8, [1, 3], [40, 12], 0xFF)  # 52 copies (6 + 4 counter bits)
    assert gpu_count(E, p)[1] == oracle.rowdp(p)["count"]
    with pytest.raises(E.D4Error) as e:
        E.Frow([1, 3] * 11, [3] * 22, 0xFF, 8, device=0)
    assert e.value.code == -4


def test_cpp_facade_reference_loop(E):
    """The reference's caller loop (Searcher::step) through the C++ facade."""
    import subprocess

    from d4gb import build

    r = subprocess.run([str(build.EXAMPLE_PATH), "0xFFFFFFE7E7FFFFFF", "5", "5"],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().splitlines()[-1] == "count 520"
    assert r.stdout.count("height=") == 8
