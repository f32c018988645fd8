"""The CPU oracle against the reference's own golden vectors (CPU only).

tests/golden/cases.json was produced by the reference's solver compiled from
its sources (tests/golden/make_golden.py); this pins the C restatement in
oracle/ before it is trusted as the GPU checker.
"""
import pytest

from conftest import case_problem, decode_grid, load_cases

CASES = load_cases()
SMALL = [c for c in CASES if c["count"] <= 20000]


@pytest.mark.parametrize("case", SMALL, ids=[c["name"] for c in SMALL])
def test_backtracker_count_matches_reference(oracle, case):
    p = case_problem(case)
    assert oracle.solve_count(p) == case["count"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_rowdp_count_matches_reference(oracle, case):
    p = case_problem(case)
    r = oracle.rowdp(p, threads=2)
    assert r["levels_done"] == p.height
    assert r["count"] == case["count"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_lean_rowdp_matches_reference_and_rowdp(oracle, case):
    """The memory-lean DP (used to pin the 8x15 enumeration) gives the
    reference's count and the same per-row frontier sizes as the stored-
    children DP."""
    p = case_problem(case)
    lean = oracle.rowdp_lean(p, threads=3)
    full = oracle.rowdp(p, threads=2)
    assert lean["count"] == case["count"]
    assert lean["level_sizes"] == full["level_sizes"]


LISTED = [c for c in CASES if "solutions" in c]


@pytest.mark.parametrize("case", LISTED, ids=[c["name"] for c in LISTED])
def test_solution_lists_match_reference_order(oracle, case):
    p = case_problem(case)
    n, tg, sg = oracle.solve(p, single=False, max_solutions=max(case["count"], 1))
    assert n == case["count"]
    for k, (t, s) in enumerate(case["solutions"]):
        assert (tg[k] == decode_grid(t, p.width, p.height)).all(), k
        assert (sg[k] == decode_grid(s, p.width, p.height)).all(), k


FIRST = [c for c in CASES if c["first"] is not None and c["count"] <= 20000]


@pytest.mark.parametrize("case", FIRST, ids=[c["name"] for c in FIRST])
def test_solve_one_matches_reference(oracle, case):
    p = case_problem(case)
    n, tg, sg = oracle.solve(p, single=True, max_solutions=1)
    assert n == 1
    assert (tg[0] == decode_grid(case["first"][0], p.width, p.height)).all()
    assert (sg[0] == decode_grid(case["first"][1], p.width, p.height)).all()
    types, masks = oracle.grid_to_placements(p, tg[0], sg[0])
    assert oracle.check_tiling(p, types, masks)


def test_pentomino_ring_canonical_classes(oracle):
    ring = next(c for c in CASES if c["name"].startswith("pentomino ring"))
    p = case_problem(ring)
    assert ring["count"] == 520
    grids = [decode_grid(t, p.width, p.height) for t, _ in ring["solutions"]]
    assert len(oracle.canonical_set(p, grids)) == 65


def test_rowdp_threads_agree(oracle):
    big = max((c for c in CASES if c["width"] * c["height"] <= 40), key=lambda c: c["count"])
    p = case_problem(big)
    a = oracle.rowdp(p, threads=1)
    b = oracle.rowdp(p, threads=4)
    assert a["count"] == b["count"] == big["count"]
    assert a["level_sizes"] == b["level_sizes"]


def test_check_tiling_rejects_bad_covers(oracle):
    ring = next(c for c in CASES if c["name"].startswith("pentomino ring"))
    p = case_problem(ring)
    t, s = ring["solutions"][0]
    types, masks = oracle.grid_to_placements(p, decode_grid(t, 8, 8), decode_grid(s, 8, 8))
    assert oracle.check_tiling(p, types, masks)
    assert not oracle.check_tiling(p, types[:-1], masks[:-1])          # board not covered
    assert not oracle.check_tiling(p, types + types[:1], masks + masks[:1])  # overlap
    swapped = list(types)
    swapped[0], swapped[1] = swapped[1], swapped[0]
    if swapped != types:
        assert not oracle.check_tiling(p, swapped, masks)              # wrong shapes


def test_oracle_piece_sets_match_reference_fixture(oracle):
    """Every multiset within the counts of the fixture's boards: the oracle's
    count equals the reference solver's (tests/golden/sets.json, generated by
    tests/golden/make_sets_golden.py from the reference's solve_count)."""
    import itertools
    import json

    from conftest import GOLDEN
    from d4gb.problem import Problem

    data = json.loads((GOLDEN / "sets.json").read_text())
    assert len(data["boards"]) >= 200
    for b in data["boards"]:
        p = Problem(b["width"], b["height"], b["rows"], b["shapes"], b["counts"], b["sym"])
        areas = [bin(v).count("1") for v in p.shapes]
        got = []
        for copies in itertools.product(*[range(k + 1) for k in p.counts]):
            if sum(a * k for a, k in zip(areas, copies)) != p.cells:
                continue
            n = oracle.solve_count(Problem(p.width, p.height, p.rows, p.shapes, list(copies),
                                           p.sym))
            if n:
                got.append([list(copies), n])
        assert sorted(got) == b["sets"], b["name"]
