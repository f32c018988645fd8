"""Piece-set mode (d4e_batch_sets) and the board-family driver.

A piece set is the multiset of copies a tiling uses; the engine keeps the
final row's states, whose copy counters are exactly those multisets.  Every
reported set is checked against the oracle: its number of tilings equals the
oracle's count with that set as the piece counts, and on the small families
the whole list equals the oracle's exhaustive search over all multisets.
The sum over a board's sets equals its counting-mode result (the
reference's golden counts)."""
import itertools
import json

import pytest

from conftest import GOLDEN, case_problem, load_cases

pytestmark = pytest.mark.gpu

CASES = [c for c in load_cases() if c["width"] <= 8]
FAMILY = "\naaab....\naaab....\nccdd....\nccdd....\n"


@pytest.fixture(scope="module")
def E(engine):
    if engine.device_count() == 0:
        pytest.fail("no CUDA device visible")
    return engine


@pytest.fixture(scope="module")
def free():
    raw = json.loads((GOLDEN / "catalogue.json").read_text())
    return {int(m): v for m, v in raw["free"].items()}


def oracle_sets(oracle, p, area_only=None):
    """Every multiset within p.counts (covering area_only cells, when given)
    with a non-zero oracle count, in the engine's order (sorted copies)."""
    areas = [bin(v).count("1") for v in p.shapes]
    cells = p.cells if area_only is None else area_only
    out = []
    for copies in itertools.product(*[range(k + 1) for k in p.counts]):
        if sum(a * k for a, k in zip(areas, copies)) != cells:
            continue
        q = type(p)(p.width, p.height, p.rows, p.shapes, list(copies), p.sym)
        n = oracle.solve_count(q)
        if n:
            out.append((tuple(copies), n))
    return sorted(out)


def test_ring_is_one_set(E):
    ring = next(c for c in CASES if c["name"].startswith("pentomino ring"))
    sets, res, st = E.batch_sets([case_problem(ring)])
    assert res[0]["status"] == 0
    assert res[0]["found"] == 1 and res[0]["count"] == 520
    assert sets == [[((1,) * 12, 520)]]


@pytest.mark.parametrize("wide", [False, True])
def test_golden_cases_sets_sum_to_counts(E, oracle, wide):
    probs = [case_problem(c) for c in CASES]
    sets, res, _ = E.batch_sets(probs, wide_keys=wide)
    for c, p, s, r in zip(CASES, probs, sets, res):
        assert r["status"] == 0, c["name"]
        assert sum(t for _, t in s) == c["count"] == r["count"], c["name"]
        assert r["found"] == len(s)
        assert [x for x, _ in s] == sorted(x for x, _ in s)
        areas = [bin(v).count("1") for v in p.shapes]
        for copies, t in s:
            assert t > 0
            assert all(0 <= k <= m for k, m in zip(copies, p.counts)), c["name"]
            assert sum(a * k for a, k in zip(areas, copies)) == p.cells, c["name"]
            if c["count"] < 10 ** 6:
                q = type(p)(p.width, p.height, p.rows, p.shapes, list(copies), p.sym)
                assert oracle.solve_count(q) == t, (c["name"], copies)


SMALL = [c for c in CASES if 0 < c["count"] < 10 ** 6 and
         sum(1 for _ in itertools.product(*[range(k + 1) for k in c["counts"]])) <= 4096]


@pytest.mark.parametrize("case", SMALL, ids=[c["name"] for c in SMALL])
def test_sets_equal_exhaustive_oracle(E, oracle, case):
    p = case_problem(case)
    sets, res, _ = E.batch_sets([p])
    assert sets[0] == oracle_sets(oracle, p)


def test_alone_and_batched_identical(E):
    probs = [case_problem(c) for c in CASES]
    a, _, _ = E.batch_sets(probs, sequential=True)
    b, _, _ = E.batch_sets(probs)
    assert a == b


def test_max_sets_retry(E):
    probs = [case_problem(c) for c in CASES]
    full, _, _ = E.batch_sets(probs)
    small, _, _ = E.batch_sets(probs, max_sets=1)
    assert small == full


@pytest.mark.parametrize("copies", [1, 2])
def test_family_matches_exhaustive_oracle(E, oracle, free, copies):
    from d4gb import family as F

    fam = F.BoardFamily.from_text(FAMILY)
    shapes = free[2] + free[3] + free[4]
    per_config, ledger = F.tiling_sets(fam, shapes, [copies] * len(shapes))
    assert set(per_config) == set(fam.configs())
    want_ledger = {}
    for m in fam.configs():
        p = F.board_problem(m, shapes, [copies] * len(shapes))
        want = oracle_sets(oracle, p, fam.left)
        assert per_config[m] == want, hex(m)
        assert sum(t for _, t in want) == oracle.solve_count(p)
        for c, _ in want:
            want_ledger[c] = want_ledger.get(c, 0) + 1
    assert ledger == want_ledger


@pytest.mark.parametrize("rotations_only", [False, True])
def test_family_ledger_ranks(E, oracle, rotations_only):
    """The AtomicCount ledger: Naming rank -> configurations tiled."""
    from d4gb import family as F

    fam = F.BoardFamily.from_text(FAMILY)
    run = F.family_ledger(fam, 2, 4, 3, 5, rotations_only=rotations_only)
    sym = 0b01101001 if rotations_only else 0xFF
    want = {}
    for m in fam.configs():
        for r in range(run.naming.size()):
            chosen = run.naming.resolve(r)
            if not 3 <= sum(len(x) for x in chosen) <= 5:
                continue
            counts = []
            for d, x in enumerate(chosen):
                counts += [1 if i in x else 0 for i in range(run.naming.sizes[2 + d])]
            p = F.board_problem(m, run.shapes, counts, sym)
            if oracle.solve_count(p):
                want[r] = want.get(r, 0) + 1
    assert run.ledger == want
    assert run.unsolved(fam) == [m for m in fam.configs() if not run.per_config[m]]


def test_cpp_family_driver_matches_python(E, tmp_path):
    """The C++ facade's AtomicCount run (example_family) and the Python
    driver give the same ledger and the same ZERO-count boards."""
    import os
    import subprocess

    from d4gb import build
    from d4gb import family as F

    text = FAMILY + "\n"
    f = tmp_path / "family.txt"
    f.write_text(text)
    env = {k: v for k, v in os.environ.items() if k not in ("S", "C")}
    r = subprocess.run([str(build.FAMILY_EXAMPLE_PATH), str(f), "2", "4", "0", "64"],
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    fam = F.BoardFamily.from_text(text)
    run = F.family_ledger(fam, 2, 4, 0, 64)
    ranked, total, weighted = (int(x) for x in lines[-1].split()[1:])
    assert ranked == len(run.ledger)
    assert total == sum(run.ledger.values())
    assert weighted == sum((k + 1) * v for k, v in run.ledger.items())
    # the C++ facade visits configurations in the reference's region order
    zero = [int(x.split()[-1], 16) for x in lines if x.startswith("ZERO-count board")]
    assert sorted(zero) == sorted(run.unsolved(fam))
    assert f"number of pieces combinations: {run.naming.size()}" in lines


@pytest.mark.parametrize("kind", ["fb", "fB"])
def test_cpp_family_ledger_file(E, tmp_path, kind):
    """The FileBit / FileByte run of the C++ facade: the file holds, for
    every configuration, exactly the ranks the Python driver finds for that
    board, and a second run resumes with nothing left to do."""
    import os
    import subprocess

    import numpy as np

    from d4gb import build
    from d4gb import family as F

    text = FAMILY + "\n"
    f = tmp_path / "family.txt"
    f.write_text(text)
    path = tmp_path / "ledger.bin"
    env = {k: v for k, v in os.environ.items() if k != "C"}
    env["S"] = kind
    args = [str(build.FAMILY_EXAMPLE_PATH), str(f), "2", "4", "0", "64", str(path)]
    first = subprocess.run(args, capture_output=True, text=True, timeout=300, env=env)
    assert first.returncode == 0, first.stderr
    fam = F.BoardFamily.from_text(text)
    run = F.family_ledger(fam, 2, 4, 0, 64)
    desc, tiled, logged = F.read_ledger_file(path, fam.count, run.naming.size(),
                                             "byte" if kind == "fB" else "bit")
    assert sorted(desc[:, 0].tolist()) == sorted(fam.configs())
    assert (desc[:, 2] > 0).all()
    assert tiled.tolist() == [run.ledger.get(r, 0) for r in range(run.naming.size())]
    sizes = [run.naming.sizes[m] for m in range(2, 5)]
    per_board = run.per_config
    for i, m in enumerate(desc[:, 0].tolist()):
        ranks = set()
        for copies, _ in per_board[m]:
            chosen, at = [], 0
            for n in sizes:
                chosen.append([j for j in range(n) if copies[at + j]])
                at += n
            ranks.add(run.naming.name(chosen))
        assert set(np.nonzero(logged[:, i])[0].tolist()) == ranks, hex(m)
        assert desc[i, 1] == len(ranks)
    again = subprocess.run(args, capture_output=True, text=True, timeout=300, env=env)
    assert again.returncode == 0, again.stderr
    assert f"{fam.count}/{fam.count} configs were previously solved; solved now 0 in 0 batches" \
        in again.stdout
    assert again.stdout.splitlines()[-1] == first.stdout.splitlines()[-1]


def test_sets_match_reference_fixture(E):
    """The engine's piece sets equal the reference solver's, board by board
    (tests/golden/sets.json: a board family's configurations and the golden
    cases with more pieces than cells)."""
    from d4gb.problem import Problem

    data = json.loads((GOLDEN / "sets.json").read_text())
    probs = [Problem(b["width"], b["height"], b["rows"], b["shapes"], b["counts"], b["sym"])
             for b in data["boards"]]
    sets, res, _ = E.batch_sets(probs)
    for b, s, r in zip(data["boards"], sets, res):
        assert r["status"] == 0, b["name"]
        assert [[list(c), t] for c, t in s] == b["sets"], b["name"]
