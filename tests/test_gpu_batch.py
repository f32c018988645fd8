"""Batches through d4e_batch_run: counting and solve-one, memory pressure,
per-instance failures, and results that do not depend on the batch.

Counts are compared exactly with the reference's golden counts and the
oracle; solve-one tilings are checked by the oracle's independent cover
check (any valid tiling is a correct answer), and must be identical alone
and batched."""
import json

import numpy as np
import pytest

from conftest import GOLDEN, case_problem, load_cases

pytestmark = pytest.mark.gpu

CASES = [c for c in load_cases() if c["width"] <= 8 and c["width"] * c["height"] <= 512]
SMALL = [c for c in CASES if c["count"] < 10 ** 6]
# Larger instances of the batched mix (40-71 cells), pinned by the oracle's
# exact row DP (tests/golden/make_mix_golden.py).
MIX_LARGE = json.loads((GOLDEN / "mix_large.json").read_text())["cases"]


@pytest.fixture(scope="module")
def E(engine):
    if engine.device_count() == 0:
        pytest.fail("no CUDA device visible")
    return engine


def assert_valid(oracle, p, r):
    types, masks = oracle.grid_to_placements(p, r["grid"], r["steps"])
    assert oracle.check_tiling(p, types, masks), p.name


@pytest.mark.parametrize("wide", [False, True])
def test_batch_counts_match_oracle_on_larger_mix_instances(E, wide):
    probs = [case_problem(c) for c in MIX_LARGE]
    res, _ = E.batch_run(probs, wide_keys=wide)
    assert [r["status"] for r in res] == [0] * len(probs)
    assert [r["count"] for r in res] == [c["count"] for c in MIX_LARGE]


def test_searcher_rows_match_oracle_on_larger_mix_instances(E):
    for c in MIX_LARGE:
        p = case_problem(c)
        f = E.Frow(p.shapes, p.counts, p.sym, p.width, device=0)
        s = E.CudaSearcher(f, rows=p.rows)
        s.run()
        assert (s.count(), s.level_sizes()) == (c["count"], c["level_sizes"]), c["name"]


def test_batch_run_counts_match_reference(E):
    probs = [case_problem(c) for c in SMALL]
    res, st = E.batch_run(probs)
    assert [r["status"] for r in res] == [0] * len(probs)
    assert [r["count"] for r in res] == [c["count"] for c in SMALL]
    assert [r["tag"] for r in res] == list(range(len(probs)))


def test_wide_keys_give_the_same_counts(E):
    probs = [case_problem(c) for c in SMALL]
    res, st = E.batch_run(probs, wide_keys=True)
    assert st["record_bytes"] == 24
    assert [r["count"] for r in res] == [c["count"] for c in SMALL]


@pytest.mark.parametrize("beam", [0, 64])
@pytest.mark.parametrize("wide", [False, True])
def test_solve_one_found_and_valid(E, oracle, beam, wide):
    """found == (count > 0) for every golden case; every tiling passes the
    oracle's cover check.  beam=64 samples rows (wider restarts when a sample
    dies out), beam=0 is exact."""
    probs = [case_problem(c) for c in CASES if c["count"] < 10 ** 9]
    want = [c["count"] for c in CASES if c["count"] < 10 ** 9]
    res, st = E.batch_run(probs, mode=E.MODE_SOLVE_ONE, beam=beam, wide_keys=wide)
    for p, r, n in zip(probs, res, want):
        assert r["status"] == 0, (p.name, r)
        assert r["found"] == (1 if n > 0 else 0), p.name
        if r["found"]:
            assert_valid(oracle, p, r)


def test_solve_one_same_alone_and_batched(E):
    probs = [case_problem(c) for c in CASES if 0 < c["count"] < 10 ** 9]
    batched, _ = E.batch_run(probs, mode=E.MODE_SOLVE_ONE, beam=256)
    alone, _ = E.batch_run(probs, mode=E.MODE_SOLVE_ONE, beam=256, sequential=True)
    for p, a, b in zip(probs, alone, batched):
        assert a["found"] and b["found"], p.name
        assert np.array_equal(a["grid"], b["grid"]), p.name
        assert np.array_equal(a["steps"], b["steps"]), p.name


def test_solve_one_mix_cover_check(E, oracle):
    """Batched-mix instances (width 5..8, height 5..12, 0..4 holes), solve-one
    with sampled rows; every reported tiling passes the cover check, and an
    instance reported unsolvable is confirmed by the exact count."""
    from d4gb.problem import batched_mix

    probs = [p for p in batched_mix(11, 300) if p.cells <= 40][:64]
    res, st = E.batch_run(probs, mode=E.MODE_SOLVE_ONE, beam=128)
    counts, _ = E.batch_run(probs)
    for p, r, c in zip(probs, res, counts):
        assert r["status"] == 0, p.name
        assert r["found"] == (1 if c["count"] > 0 else 0), p.name
        if r["found"]:
            assert_valid(oracle, p, r)


def test_memory_budget_pauses_and_groups(E):
    """Under a small device budget the batch runs in groups and instances
    wait for memory; every count still equals the instance's count alone."""
    from d4gb.problem import batched_mix

    probs = [p for p in batched_mix(21, 400) if 50 <= p.cells <= 60][:24]
    alone, st_a = E.batch_run(probs, sequential=True)
    # Room for the largest instance alone (frontiers + table at load 0.5,
    # with headroom), far less than all of them at once.
    budget = (64 << 20) + 8 * st_a["peak_frontier"] * 48
    tight, st = E.batch_run(probs, memory_budget=budget)
    assert [r["status"] for r in tight] == [0] * len(probs)
    assert [r["count"] for r in tight] == [r["count"] for r in alone]
    assert st["paused"] + st["splits"] > 0, st


def test_frontier_limit_fails_only_that_instance(E):
    probs = [case_problem(c) for c in SMALL]
    sizes = []
    for p in probs:
        f = E.Frow(p.shapes, p.counts, p.sym, p.width, device=0)
        s = E.CudaSearcher(f, rows=p.rows)
        s.run()
        sizes.append(max(s.level_sizes() or [1]))
    limit = sorted(sizes)[len(sizes) // 2]
    res, st = E.batch_run(probs, max_states=limit)
    for c, r, peak in zip(SMALL, res, sizes):
        if peak > limit:
            assert r["status"] == E.D4E_ERR_UNSUPPORTED, c["name"]
        else:
            assert r["status"] == 0 and r["count"] == c["count"], c["name"]
    assert st["failed"] == sum(1 for s in sizes if s > limit)


def test_kept_memory_reuse_and_release(E):
    """An ended engine's pool is reused by the next one; releasing it
    changes no result."""
    probs = [case_problem(c) for c in SMALL]
    want = [c["count"] for c in SMALL]
    for release in (False, False, True, False):
        if release:
            E.release_cached_memory()
        res, _ = E.batch_run(probs)
        assert [r["count"] for r in res] == want
