"""Partitioned de-duplication (children appended into hash buckets, each
bucket merged in shared memory) gives the same frontiers, counts and
solve-one results as direct hash-table inserts."""
import pytest

from conftest import case_problem, load_cases

pytestmark = pytest.mark.gpu

CASES = [c for c in load_cases() if c["width"] <= 8 and c["width"] * c["height"] <= 512]


@pytest.fixture(scope="module")
def E(engine):
    if engine.device_count() == 0:
        pytest.fail("no CUDA device visible")
    return engine


def run(E, p, dedup):
    f = E.Frow(p.shapes, p.counts, p.sym, p.width, device=0)
    s = E.CudaSearcher(f, rows=p.rows, dedup=dedup)
    s.run()
    return s.count(), s.level_sizes(), s.stats()


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_partitioned_counts_and_levels(E, case):
    p = case_problem(case)
    n_p, lv_p, st = run(E, p, "partitioned")
    n_d, lv_d, _ = run(E, p, "direct")
    assert n_p == n_d == case["count"]
    assert lv_p == lv_d
    if st["record_bytes"] == 16 and p.height >= 3 and lv_d[0] > 0:
        assert st["partitioned"] > 0, st


def test_partitioned_medium_board(E):
    from d4gb.problem import medium_board

    p = medium_board(77)
    n, lv, st = run(E, p, "partitioned")
    assert n == 4952290238
    assert st["partitioned"] >= 5, st
    assert st["partition_fallbacks"] == 0, st


def test_partitioned_batches(E, oracle):
    from d4gb.problem import batched_mix

    probs = [p for p in batched_mix(11, 400) if p.cells <= 60][:48]
    direct, _ = E.batch_run(probs, dedup="direct")
    part, st = E.batch_run(probs, dedup="partitioned")
    assert [r["count"] for r in part] == [r["count"] for r in direct]
    assert st["partitioned"] > 0
    one, _ = E.batch_run(probs, mode=E.MODE_SOLVE_ONE, beam=256, dedup="partitioned")
    one_d, _ = E.batch_run(probs, mode=E.MODE_SOLVE_ONE, beam=256, dedup="direct")
    for p, r, rd, c in zip(probs, one, one_d, direct):
        assert r["found"] == (1 if c["count"] > 0 else 0), p.name
        if r["found"]:
            # Same witnesses, same sampling: the same tiling either way.
            assert (r["grid"] == rd["grid"]).all() and (r["steps"] == rd["steps"]).all()
            types, masks = oracle.grid_to_placements(p, r["grid"], r["steps"])
            assert oracle.check_tiling(p, types, masks)
