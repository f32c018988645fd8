"""Host-side helpers of bench.py on CPU: the latency summary, the seeded
arrival stream of the serving sections and the listing section's boards."""
import pytest


def test_latency_summary_counts_cut_requests():
    import bench

    done = [1.0, 2.0, 3.0, 4.0]
    s = bench._latency_summary(done, [])
    assert s["p50"] == s["p50_completed"] and s["p99"] == 4.0
    # requests cut at the deadline count with the time they had waited
    s = bench._latency_summary(done, [100.0, 200.0])
    assert s["p99"] == 200.0 and s["p99_completed"] == 4.0
    assert bench._latency_summary([], [])["p50"] is None


def test_arrivals_are_seeded_and_poisson(engine):
    import bench

    a1, p1, m1 = bench._arrivals(200.0, 10.0, 4242)
    a2, p2, m2 = bench._arrivals(200.0, 10.0, 4242)
    assert a1 == a2 and m1 == m2 and [p.rows for p in p1] == [p.rows for p in p2]
    assert len(a1) == 2000 and all(x < y for x, y in zip(a1, a1[1:]))
    assert abs(a1[-1] - 10.0) < 1.0                      # mean gap 1 / rate
    share = sum(1 for m in m1 if m == engine.MODE_SOLVE_ONE) / len(m1)
    assert 0.65 < share < 0.75                          # 70 % solve-one


def test_listing_section_boards():
    import bench
    from d4gb.problem import batched_mix

    probs = [p for p in batched_mix(bench.BATCHED_SEED, 16 * bench.LIST_INSTANCES)
             if p.cells <= bench.LIST_MAX_CELLS][: bench.LIST_INSTANCES]
    assert len(probs) == bench.LIST_INSTANCES
    assert all(p.cells <= bench.LIST_MAX_CELLS for p in probs)
