"""The serving loop (d4e_server_*): requests admitted while others run share
the device, and every result is the same as the request run alone."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E(engine):
    if engine.device_count() == 0:
        pytest.fail("no CUDA device visible")
    return engine


def mix_requests(n, seed):
    from d4gb.problem import batched_mix

    probs = [p for p in batched_mix(seed, 6 * n) if p.cells <= 64][:n]
    modes = [1 if (i * 7) % 10 < 7 else 0 for i in range(len(probs))]   # 70% solve-one
    return probs, modes


def alone_results(E, probs, modes, beam):
    out = []
    for p, m in zip(probs, modes):
        r, _ = E.batch_run([p], mode=m, sequential=True, beam=beam)
        out.append(r[0])
    return out


def same(a, b):
    if a["status"] != b["status"] or a["count"] != b["count"] or a["found"] != b["found"]:
        return False
    if a["found"]:
        return np.array_equal(a["grid"], b["grid"]) and np.array_equal(a["steps"], b["steps"])
    return True


def test_server_results_equal_alone(E, oracle):
    probs, modes = mix_requests(48, 31)
    beam = 128
    want = alone_results(E, probs, modes, beam)
    srv = E.Server(beam=beam)
    try:
        # Staggered arrivals: some requests join while others are running.
        for i, (p, m) in enumerate(zip(probs, modes)):
            srv.submit(p, m, i)
            if i % 8 == 7:
                time.sleep(0.002)
        srv.drain(300)
        got = {r["tag"]: r for r in srv.poll(1000)}
        st = srv.stats()
    finally:
        srv.close()
    assert sorted(got) == list(range(len(probs)))
    for i, p in enumerate(probs):
        assert same(got[i], want[i]), (p.name, got[i], want[i])
        if got[i]["found"]:
            types, masks = oracle.grid_to_placements(p, got[i]["grid"], got[i]["steps"])
            assert oracle.check_tiling(p, types, masks)
    assert st["completed"] == len(probs)
    assert st["peak_active"] > 1     # requests overlapped on the device
    assert st["moved"] > 0           # some outgrew the fast lane and restarted
    assert all(got[i]["latency_ms"] >= got[i]["queued_ms"] >= 0 for i in got)


def test_server_small_budget_queues_requests(E):
    """A budget smaller than the projected bytes of all requests admits them
    in turns; results are unchanged."""
    probs, modes = mix_requests(16, 41)
    modes = [0] * len(probs)
    want = alone_results(E, probs, modes, 0)
    srv = E.Server(memory_budget=64 << 20)
    try:
        for i, p in enumerate(probs):
            srv.submit(p, 0, i)
        srv.drain(300)
        got = {r["tag"]: r for r in srv.poll(1000)}
    finally:
        srv.close()
    for i in range(len(probs)):
        assert same(got[i], want[i])


def test_server_rejects_bad_requests_without_stopping(E):
    from d4gb.problem import Problem

    srv = E.Server()
    try:
        bad = Problem(8, 2, [0xFF, 0xFF], [0], [1], 0xFF)    # empty piece shape
        good = Problem(4, 2, [0xF, 0xF], [0x3], [4], 0xFF)    # 2x4 by dominoes: 5
        srv.submit(bad, 0, 1)
        srv.submit(good, 0, 2)
        srv.drain(60)
        got = {r["tag"]: r for r in srv.poll(10)}
    finally:
        srv.close()
    assert got[1]["status"] != 0
    assert got[2]["status"] == 0 and got[2]["count"] == 5


def test_server_preempted_rows_keep_results(E, oracle):
    """Small requests arriving while the 8x15 enumeration runs in the slow
    lane preempt its k_expand launches (warps stop taking chunks, the row
    resumes later): the enumeration still gives the oracle's pinned count,
    and every small request its result alone."""
    import json

    from conftest import GOLDEN
    from d4gb.problem import Problem

    c = next(c for c in json.loads((GOLDEN / "large.json").read_text())["cases"]
             if c["name"].startswith("single large"))
    big = Problem(c["width"], c["height"], list(c["rows"]), c["shapes"], c["counts"], c["sym"],
                  name=c["name"])
    probs, modes = mix_requests(40, 57)
    beam = 128
    want = alone_results(E, probs, modes, beam)
    srv = E.Server(beam=beam)
    try:
        srv.submit(big, 0, 1000)
        t0 = time.time()
        while srv.stats()["moved"] == 0 and time.time() - t0 < 60:
            time.sleep(0.005)
        time.sleep(0.05)
        for i, (p, m) in enumerate(zip(probs, modes)):
            srv.submit(p, m, i)
            time.sleep(0.01)
        srv.drain(600)
        got = {r["tag"]: r for r in srv.poll(1000)}
        st = srv.stats()
    finally:
        srv.close()
    assert got[1000]["status"] == 0 and got[1000]["count"] == int(c["count"])
    for i, p in enumerate(probs):
        assert same(got[i], want[i]), (p.name, got[i], want[i])
    assert st["preemptions"] > 0
