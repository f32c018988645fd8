"""The launch autotuner (replacing the reference's KSizing::optimize): it
measures launch plans on a real row, never changes results, and is cached
per process."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E(engine):
    if engine.device_count() == 0:
        pytest.fail("no CUDA device visible")
    return engine


def test_autotune_keeps_counts_and_caches(E):
    from d4gb.problem import medium_board

    p = medium_board(77)   # rows of 10^5..10^7 states: the tuner measures one
    E.autotune_clear()
    f = E.Frow(p.shapes, p.counts, p.sym, p.width, device=0)
    s = E.CudaSearcher(f, rows=p.rows, autotune=True)
    s.run()
    st = s.stats()
    assert s.count() == 4952290238
    assert st["tune_ms"] > 0
    assert st["tuned_chunk_cap"] in (256, 512, 1024, 2048)
    assert st["tuned_chunks_per_warp"] in (4, 8, 16)
    assert 0.3 <= st["tuned_load"] <= 0.75
    # The dedup tile plan: blocks per SM x shared-memory ring depth.
    assert (st["tuned_compact_ctas"], st["tuned_compact_stages"]) in ((2, 3), (2, 2), (1, 6))
    again = E.CudaSearcher(f, rows=p.rows, autotune=True)
    again.run()
    assert again.count() == 4952290238
    st2 = again.stats()
    assert st2["tune_ms"] == 0          # plan taken from the process cache
    assert st2["tuned_chunk_cap"] == st["tuned_chunk_cap"]
    assert st2["tuned_compact_stages"] == st["tuned_compact_stages"]


def test_autotuned_batch_equals_plain(E):
    from d4gb.problem import batched_mix

    probs = [p for p in batched_mix(21, 400) if 50 <= p.cells <= 64][:32]
    a, _ = E.batch_run(probs)
    b, st = E.batch_run(probs, autotune=True)
    assert [r["count"] for r in a] == [r["count"] for r in b]
