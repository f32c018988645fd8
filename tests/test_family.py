"""Board-family text parsing, configuration enumeration and combination
ranks (host logic, no GPU).

Parsing follows the reference's Shape / Board text rules
(src/Shape.hpp:49-77, src/board.hpp:15-38); ranks follow its Naming
(src/naming.cpp:34-90, src/naming.inl:6-72) and are checked here as a
bijection onto 0..size-1 whose size matches a brute-force count."""
import itertools

import pytest

from d4gb import family as F


def test_shape_text_rules():
    assert F.parse_shape("#.#\n.#.") == 0b101 | (0b010 << 8)
    # a leading newline is skipped; '*', '1', '@', '#', 'X', '%' are cells;
    # ' ', '0', '.', '-', '_' are holes; anything else is ignored
    assert F.parse_shape("\n*1@#X%") == 0b111111
    assert F.parse_shape(" 0.-_#") == 1 << 5
    assert F.parse_shape("#?!#") == 0b11
    # a row longer than the width runs on into the next row's bits
    assert F.parse_shape("#########") == (1 << 9) - 1
    assert F.parse_shape("#\n#", width=11) == 1 | (1 << 11)


def test_board_regions_and_configs():
    fam = F.BoardFamily.from_text("\naaab....\naaab....\nccdd....\nccdd....\n")
    assert fam.names == ["a", "b", "c", "d"]
    assert fam.base == 0x0F0F0F0F
    assert fam.regions == [0x707, 0x808, 0x3030000, 0xC0C0000]
    assert fam.count == 6 * 2 * 4 * 4 == 192
    assert fam.left == 12
    cfgs = list(fam.configs())
    assert len(cfgs) == len(set(cfgs)) == 192
    for m in cfgs:
        assert m & ~fam.base == 0
        for r in fam.regions:
            assert bin(r & ~m).count("1") == 1


def test_base_marks_belong_to_every_region():
    # as in the reference, a non-letter cell mark is kept in every region's
    # text, so it belongs to each region as well as to the base
    fam = F.BoardFamily.from_text("a#\nb#")
    assert fam.base == 0b11 | (0b11 << 8)
    assert fam.regions == [0b11 | (0b10 << 8), 0b10 | (0b11 << 8)]
    cfgs = list(fam.configs())
    assert len(cfgs) == fam.count == 9
    # picking the shared cell twice leaves three cells, not two
    assert (0b11 | (0b11 << 8)) & ~(0b10) in cfgs


def test_board_problem_rows():
    p = F.board_problem(0x0F0F0F0F, [0b11], [6])
    assert (p.width, p.height, p.rows) == (8, 4, [15, 15, 15, 15])
    q = F.board_problem(1 | (1 << 11), [0b1], [2], width=11)
    assert (q.width, q.height, q.rows) == (11, 2, [1, 1])


def brute_force(min_m, max_m, min_n, max_n, tgt, sizes):
    pieces = [(m, i) for m in range(min_m, max_m + 1) for i in range(sizes.get(m, 0))]
    out = []
    for r in range(min_n, max_n + 1):
        for c in itertools.combinations(pieces, r):
            if sum(m for m, _ in c) == tgt:
                out.append(c)
    return out


def test_naming_is_a_bijection():
    # the example in the reference's Naming self-test: sizes 2, 4, 5 with
    # 3, 7 and 6 pieces, 2..8 pieces covering 20 cells
    sizes = {2: 3, 4: 7, 5: 6}
    nm = F.Naming(2, 5, 2, 8, 20, sizes)
    combos = brute_force(2, 5, 2, 8, 20, sizes)
    assert nm.size() == len(combos) == 1191
    seen = set()
    for c in combos:
        chosen = [[i for m, i in c if m == mm] for mm in range(2, 6)]
        r = nm.name(chosen)
        assert r is not None and 0 <= r < nm.size()
        seen.add(r)
        assert nm.resolve(r) == [sorted(x) for x in chosen]
    assert len(seen) == nm.size()


def test_naming_order():
    # profiles (pieces per size) in lexicographic order; within one profile
    # the smallest size is the most significant digit and each digit is the
    # lexicographic rank of the chosen subset
    nm = F.Naming(1, 2, 0, 9, 3, {1: 3, 2: 2})
    assert nm.profiles == [(1, 1), (3, 0)]
    got = [nm.resolve(i) for i in range(nm.size())]
    assert got == [[[0], [0]], [[0], [1]], [[1], [0]], [[1], [1]], [[2], [0]], [[2], [1]],
                   [[0, 1, 2], []]]
    assert nm.name([[0], [0, 1]]) is None          # 5 cells, not 3
    assert nm.resolve(nm.size()) is None
    # piece-count limits
    assert F.Naming(1, 2, 2, 2, 3, {1: 3, 2: 2}).size() == 6
    assert F.Naming(1, 2, 3, 3, 3, {1: 3, 2: 2}).size() == 1


def fake_batch_sets(oracle):
    """batch_sets answered by the oracle's exhaustive search (host logic
    only: the arrays a GPU batch would return)."""
    import numpy as np

    def run(probs, arrays=False, **kw):
        assert arrays
        offs, rows, til = [0], [], []
        for p in probs:
            areas = [bin(v).count("1") for v in p.shapes]
            for copies in itertools.product(*[range(k + 1) for k in p.counts]):
                if sum(a * k for a, k in zip(areas, copies)) != p.cells:
                    continue
                q = type(p)(p.width, p.height, p.rows, p.shapes, list(copies), p.sym)
                n = oracle.solve_count(q)
                if n:
                    rows.append(list(copies) + [0] * (64 - len(copies)))
                    til.append(n)
            offs.append(len(rows))
        out = (np.array(offs, np.uint64), np.array(rows, np.uint8).reshape(-1, 64),
               np.array(til, np.uint64))
        return out, [{"status": 0} for _ in probs], {"states_out": 0}
    return run


def test_family_driver_host_logic(monkeypatch, oracle, catalogue_golden):
    """Filtering by area and piece count, board multiplicity (overlapping
    regions) and the ledger, with the batch answered by the oracle."""
    from d4gb import engine as E

    monkeypatch.setattr(E, "batch_sets", fake_batch_sets(oracle))
    free = catalogue_golden["free"]
    shapes = free[1] + free[2] + free[3]
    # 'a' and 'b' share the two '#' cells: picking one twice leaves 5
    # cells, and picking both (in either order) gives one board twice
    fam = F.BoardFamily.from_text("aa##\nbb..\n")
    assert fam.left == 4 and fam.count == 16 and len(set(fam.configs())) == 15
    per_config, ledger = F.tiling_sets(fam, shapes)
    areas = [bin(v).count("1") for v in shapes]
    want = {}
    for m in fam.configs():
        p = F.board_problem(m, shapes, [1] * len(shapes))
        for copies in itertools.product((0, 1), repeat=len(shapes)):
            if sum(a * k for a, k in zip(areas, copies)) != 4:
                continue
            q = F.board_problem(m, shapes, list(copies))
            if oracle.solve_count(q):
                want[copies] = want.get(copies, 0) + 1
        if bin(m).count("1") != 4:
            assert per_config[m] == []
    assert ledger == want and max(want.values()) >= 2
    few, _ = F.tiling_sets(fam, shapes, min_n=3, max_n=3)
    assert all(sum(c) == 3 for v in few.values() for c, _ in v)
    run = F.family_ledger(fam, 1, 3, 0, 9)
    assert sum(run.ledger.values()) == sum(want.values())
    for r, n in run.ledger.items():
        chosen = run.naming.resolve(r)
        copies = tuple(1 if i in chosen[d] else 0
                       for d, size in enumerate((1, 1, 2)) for i in range(size))
        assert want[copies] == n
    assert run.unsolved(fam) == [m for m in fam.configs() if not run.per_config[m]]


@pytest.fixture(scope="module")
def host_check(tmp_path_factory):
    """The C++ facade's Board / Naming, compiled alone (no GPU calls)."""
    import shutil
    import subprocess

    from conftest import REPO

    out = tmp_path_factory.mktemp("host") / "family_host_check"
    cxx = shutil.which("g++") or "g++"
    r = subprocess.run([cxx, "-O1", "-std=c++17", "-Wall", "-Werror",
                        "-I", str(REPO / "d4-pieces_gb300" / "host"),
                        str(REPO / "tests" / "family_host_check.cpp"), "-o", str(out)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def run_check(exe, *args):
    import subprocess

    r = subprocess.run([str(exe)] + [str(a) for a in args], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.splitlines()


@pytest.mark.parametrize("text", ["\naaab....\naaab....\nccdd....\nccdd....\n",
                                  "aa##\nbb..\n",
                                  "aaaaaaaa\naaaaaaaa\naaabaaaa\naaaacaaa\naaaaaaaa\n",
                                  "\n#%X@*.1\nab-_ 0Z\n"])
def test_cpp_board_matches_python(host_check, tmp_path, text):
    f = tmp_path / "board.txt"
    f.write_text(text)
    lines = run_check(host_check, "board", f)
    fam = F.BoardFamily.from_text(text)
    assert lines[0] == f"base {fam.base:x}"
    # the C++ facade keeps the reference's region order (its container's),
    # Python the order of first appearance: same regions, same boards
    n = len(fam.regions)
    assert sorted(lines[1:1 + n]) == sorted(f"region {r:x}" for r in fam.regions)
    assert lines[1 + n] == f"count {fam.count} left {fam.left}"
    assert sorted(lines[2 + n:]) == sorted(f"config {m:x}" for m in fam.configs())


@pytest.mark.parametrize("args", [(2, 5, 2, 8, 20, 3, 0, 7, 6), (1, 2, 0, 9, 3, 3, 2),
                                  (3, 5, 0, 64, 37, 2, 5, 12), (4, 5, 3, 11, 40, 5, 12)])
def test_cpp_naming_matches_python(host_check, args):
    min_m, max_m, min_n, max_n, tgt, *sizes = args
    lines = run_check(host_check, "naming", *args)
    nm = F.Naming(min_m, max_m, min_n, max_n, tgt,
                  {min_m + d: s for d, s in enumerate(sizes)})
    assert lines[0] == f"size {nm.size()}"
    assert lines[-1] == "roundtrip ok"
    for r, line in enumerate(lines[1:-1]):
        want = " ".join(f"{min_m + d}:{i}" for d, c in enumerate(nm.resolve(r)) for i in c)
        assert line == f"rank {r}: {want}".rstrip(), r


@pytest.mark.parametrize("kind", ["bit", "byte"])
def test_ledger_file_layout_and_resume(host_check, tmp_path, kind):
    """The C++ LedgerFile writes the reference's FileBit / FileByte layout;
    a second run skips the configurations the first one solved."""
    import subprocess

    import numpy as np

    path = tmp_path / "ledger.bin"
    configs, names = 11, 5
    first = run_check(host_check, "ledgerfile", path, configs, names, kind, "stop")
    assert first[0].startswith("skipped 0 ")
    desc, tiled, logged = F.read_ledger_file(path, configs, names, kind)
    assert list(desc[:, 2]) == [1, 2] + [0] * (configs - 2)
    second = run_check(host_check, "ledgerfile", path, configs, names, kind)
    assert second[0].startswith("skipped 2 ")
    desc, tiled, logged = F.read_ledger_file(path, configs, names, kind)
    want = np.array([[(r + i) % 3 == 0 for i in range(configs)] for r in range(names)])
    assert (logged == want).all()
    assert list(tiled) == list(want.sum(axis=1))
    assert list(desc[:, 0]) == [0x1000 + i for i in range(configs)]
    assert list(desc[:, 1]) == list(want.sum(axis=0))
    assert list(desc[:, 2]) == [1 + i for i in range(configs)]
    assert [ln.split()[-1] for ln in second[1:]] == [str(v) for v in tiled]
    # a file sized for another family is refused
    r = subprocess.run([str(host_check), "ledgerfile", str(path), str(configs + 1), str(names),
                        kind], capture_output=True, text=True)
    assert r.returncode == 3 and "too short" in r.stdout



@pytest.fixture(scope="module")
def family_sim(tmp_path_factory, oracle, catalogue_golden):
    """The C++ facade with its engine calls answered by the oracle (CPU)."""
    import shutil
    import subprocess

    from conftest import REPO

    d = tmp_path_factory.mktemp("sim")
    exe = d / "family_file_sim"
    lib = REPO / "oracle" / "_build"
    r = subprocess.run([shutil.which("g++") or "g++", "-O1", "-std=c++17", "-Wall", "-Werror",
                        "-I", str(REPO / "d4-pieces_gb300" / "host"),
                        str(REPO / "tests" / "family_file_sim.cpp"), "-o", str(exe),
                        "-L", str(lib), "-ld4oracle", f"-Wl,-rpath,{lib}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    pieces = d / "pieces.txt"
    pieces.write_text("".join(f"{m} {v}\n" for m in sorted(catalogue_golden["free"])
                              for v in catalogue_golden["free"][m]))
    return exe, pieces


def ledger_line(ledger):
    return (f"ledger {len([v for v in ledger.values() if v])} {sum(ledger.values())} "
            f"{sum((r + 1) * v for r, v in ledger.items())}")


def test_cpp_family_file_run_matches_python(monkeypatch, oracle, family_sim, tmp_path):
    """ac ledger, a FileBit run cut after 3 batches and resumed, and a
    FileByte run: all equal the Python driver's ledger; each configuration's
    logged ranks are its board's ranked combinations."""
    import numpy as np

    from d4gb import engine as E

    monkeypatch.setattr(E, "batch_sets", fake_batch_sets(oracle))
    exe, pieces = family_sim
    text = "\naaab....\naaab....\nccdd....\nccdd....\n\n"
    board = tmp_path / "family.txt"
    board.write_text(text)
    fam = F.BoardFamily.from_text(text)
    run = F.family_ledger(fam, 2, 4, 0, 64)
    base = [pieces, board, 2, 4, 0, 64]
    ac = run_check(exe, *base, "ac")
    assert ac[-1] == ledger_line(run.ledger)
    zero = sorted(int(x.split()[-1], 16) for x in ac if x.startswith("ZERO"))
    assert zero == sorted(run.unsolved(fam))
    sizes = [run.naming.sizes[m] for m in range(2, 5)]

    def board_ranks(m):
        out = set()
        for copies, _ in run.per_config[m]:
            chosen, at = [], 0
            for n in sizes:
                chosen.append([j for j in range(n) if copies[at + j]])
                at += n
            out.add(run.naming.name(chosen))
        return out

    for kind, flag in (("bit", "fb"), ("byte", "fB")):
        path = tmp_path / f"ledger.{kind}"
        part = run_check(exe, *base, flag, path, 7, 3)
        assert part[0] == "previously 0 now 21 batches 3"
        rest = run_check(exe, *base, flag, path, 7)
        assert rest[0] == f"previously 21 now {fam.count - 21} batches {-(-(fam.count - 21) // 7)}"
        assert rest[-1] == ac[-1]
        desc, tiled, logged = F.read_ledger_file(path, fam.count, run.naming.size(), kind)
        assert tiled.tolist() == [run.ledger.get(r, 0) for r in range(run.naming.size())]
        assert sorted(desc[:, 0].tolist()) == sorted(fam.configs())
        for i, m in enumerate(desc[:, 0].tolist()):
            ranks = board_ranks(m)
            assert set(np.nonzero(logged[:, i])[0].tolist()) == ranks
            assert desc[i, 1] == len(ranks) and desc[i, 2] > 0
        done = run_check(exe, *base, flag, path, 7)
        assert done[0] == f"previously {fam.count} now 0 batches 0"
