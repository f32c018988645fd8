"""Batched solution listing (d4e_batch_solutions): every tiling of many
boards from one batch, against the reference's own solution lists in the
golden vectors (the tilings and their placement order, as sets)."""
import numpy as np
import pytest

from conftest import case_problem, decode_grid, load_cases

pytestmark = pytest.mark.gpu

LISTED = [c for c in load_cases()
          if c["width"] <= 8 and "solutions" in c and c["count"] > 0]


@pytest.fixture(scope="module")
def E(engine):
    if engine.device_count() == 0:
        pytest.fail("no CUDA device visible")
    return engine


def golden_set(c):
    w, h = c["width"], c["height"]
    return {(decode_grid(t, w, h).tobytes(), decode_grid(s, w, h).astype(np.int16).tobytes())
            for t, s in c["solutions"]}


def listed_set(tg, sg):
    return {(a.tobytes(), b.tobytes()) for a, b in zip(tg, sg)}


@pytest.mark.parametrize("flags", [{}, {"wide_keys": True}, {"sequential": True}],
                         ids=["packed", "wide", "sequential"])
def test_batch_lists_every_tiling(E, flags):
    probs = [case_problem(c) for c in LISTED]
    out, res, st = E.batch_solutions(probs, **flags)
    for c, (tg, sg), r in zip(LISTED, out, res):
        assert r["status"] == 0 and r["count"] == c["count"], c["name"]
        assert len(tg) == c["count"], c["name"]
        assert listed_set(tg, sg) == golden_set(c), c["name"]


def test_batch_listing_limits(E):
    """max_per_instance caps each board's list (distinct tilings of the
    golden set); max_total too small for the batch is grown by the binding."""
    probs = [case_problem(c) for c in LISTED]
    out, res, _ = E.batch_solutions(probs, max_per_instance=7, max_total=5)
    for c, (tg, sg), r in zip(LISTED, out, res):
        assert r["count"] == c["count"]
        assert len(tg) == min(7, c["count"])
        got = listed_set(tg, sg)
        assert len(got) == len(tg) and got <= golden_set(c), c["name"]


def test_batch_listing_unsolvable_and_mixed(E):
    """Boards without a tiling list nothing and do not disturb the others."""
    from d4gb.problem import Problem

    none = Problem(3, 3, [7, 7, 7], [0x3], [4], 0xFF)   # 9 cells, dominoes: no tiling
    ring = case_problem(LISTED[0])
    out, res, _ = E.batch_solutions([none, ring, none])
    assert [r["count"] for r in res] == [0, LISTED[0]["count"], 0]
    assert len(out[0][0]) == 0 and len(out[2][0]) == 0
    assert listed_set(*out[1]) == golden_set(LISTED[0])
