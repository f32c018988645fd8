"""Host-side logic of the product library and its C ABI (no GPU needed).

Only host functions are called here (catalogue, placement tables, canonical
forms, argument validation); nothing launches a kernel.
"""
import re
import subprocess
from pathlib import Path

import pytest

from conftest import REPO, case_problem, decode_grid, load_cases

HEADER = REPO / "include" / "d4e.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(d4e_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_boundary():
    names = declared_functions()
    for must in ("d4e_frow_create", "d4e_frow_transfer", "d4e_searcher_create",
                 "d4e_searcher_get_height", "d4e_searcher_size", "d4e_searcher_next_size",
                 "d4e_searcher_search_GPU", "d4e_searcher_count", "d4e_batch_count"):
        assert must in names


def test_library_exports_every_declared_symbol(engine):
    lib = engine.lib()
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(engine.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (d4e_\w+)", out))
    assert set(declared_functions()) <= exported


def test_catalogue_matches_reference(engine, catalogue_golden):
    for m in range(1, 9):
        assert engine.catalogue(m) == catalogue_golden["free"][m], m
        assert engine.catalogue(m, onesided=True) == catalogue_golden["onesided"][m], m


def test_python_shape_helpers_match_catalogue(catalogue_golden):
    from d4gb.problem import canonical

    for m in range(1, 7):
        for v in catalogue_golden["free"][m]:
            assert canonical(v) == v


def _placements_expected(shapes, counts, sym, width):
    """Distinct allowed orientations anchored at each column (independent
    Python count)."""
    from d4gb.problem import transform

    per_col = [0] * width
    for s, c in zip(shapes, counts):
        if not c:
            continue
        seen = []
        for t in range(8):
            if not (sym >> t) & 1:
                continue
            v = transform(s, t)
            if v in seen:
                continue
            seen.append(v)
            cells = [(b // 8, b % 8) for b in range(64) if (v >> b) & 1]
            a = cells[0]
            wdt = max(c_ for _, c_ in cells) + 1
            for col in range(width):
                x = col - a[1]
                if x >= 0 and x + wdt <= width:
                    per_col[col] += 1
    return per_col


@pytest.mark.parametrize("width", [3, 5, 8])
@pytest.mark.parametrize("sym", [0xFF, 0x69, 0x01])
def test_frow_placement_counts(engine, catalogue_golden, width, sym):
    shapes = catalogue_golden["free"][5][:7]
    counts = [1, 2, 1, 1, 0, 3, 1]
    if width < 5:
        shapes, counts = catalogue_golden["free"][3], [2, 1]
    f = engine.Frow(shapes, counts, sym, width, device=None)
    want = _placements_expected(shapes, counts, sym, width)
    assert [f.placements(c) for c in range(width)] == want


def test_frow_rejects_bad_input(engine):
    with pytest.raises(engine.D4Error) as e:
        engine.Frow([31], [1], 0xFF, 9, device=None)
    assert e.value.code == -1
    with pytest.raises(engine.D4Error) as e:
        engine.Frow([0], [1], 0xFF, 8, device=None)
    assert e.value.code == -1
    with pytest.raises(engine.D4Error) as e:
        engine.Frow([1 | 4], [1], 0xFF, 8, device=None)   # disconnected
    assert e.value.code == -1
    engine.Frow([1], [41], 0xFF, 8, device=None)          # 41 copies: a 6-bit counter
    with pytest.raises(engine.D4Error) as e:
        engine.Frow([1, 3] * 11, [3] * 22, 0xFF, 8, device=None)   # 22 x 2 bits > 40
    assert e.value.code == -4
    # an 8-cell bar fits a 4-wide board upright only (8 rows <= 64 / 4): accepted
    f = engine.Frow([255], [1], 0xFF, 4, device=None)
    assert [f.placements(c) for c in range(4)] == [1, 1, 1, 1]


def test_transfer_without_gpu_fails_like_reference(engine):
    if engine.device_count() > 0:
        pytest.skip("a GPU is present")
    f = engine.Frow([3], [2], 0xFF, 4, device=None)
    with pytest.raises(engine.D4Error) as e:
        f.transfer(0)
    assert e.value.code == -2 and "no CUDA device" in str(e.value)


def test_canonical_grid_matches_oracle(engine, oracle):
    ring = next(c for c in load_cases() if c["name"].startswith("pentomino ring"))
    p = case_problem(ring)
    for t, _ in ring["solutions"][:40]:
        g = decode_grid(t, 8, 8)
        assert (engine.canonical_grid(p, g) == oracle.canonical_grid(p, g)).all()
    grids = [decode_grid(t, 8, 8) for t, _ in ring["solutions"]]
    assert len({engine.canonical_grid(p, g).tobytes() for g in grids}) == 65


def test_generators_are_deterministic():
    from d4gb.problem import batched_mix, single_large

    a = batched_mix(11, 50)
    b = batched_mix(11, 50)
    assert [(x.width, x.height, x.rows, x.shapes, x.counts) for x in a] == \
           [(x.width, x.height, x.rows, x.shapes, x.counts) for x in b]
    for p in a:
        assert 5 <= p.width <= 8 and 5 <= p.height <= 12
        assert p.width * p.height - p.cells <= 4
        assert p.piece_area == p.cells
        assert all(3 <= bin(s).count("1") <= 6 for s in p.shapes)
        assert p.copies <= 40
    s = single_large(3)
    assert (s.width, s.height) == (8, 15) and s.cells == 117 and s.piece_area == 117
    assert s.copies == 24 and all(4 <= bin(v).count("1") <= 6 for v in s.shapes)


def test_empty_area_board_layout():
    from d4gb.problem import pentomino_ring

    p = pentomino_ring([31] * 12)
    ea = p.empty_area()
    assert ea == 0xFFFFFFE7E7FFFFFF
    assert bin(ea).count("1") == 60


def test_cpp_facade_builds_and_fails_like_reference_without_gpu(engine):
    from d4gb import build

    exe = build.EXAMPLE_PATH
    assert exe.exists()
    if engine.device_count() > 0:
        pytest.skip("a GPU is present")
    r = subprocess.run([str(exe), "0xFFFFFFE7E7FFFFFF", "5", "5"], capture_output=True, text=True)
    assert r.returncode == 1 and "no CUDA device" in r.stderr


def test_list_mode_runs_only_through_batch_solutions(engine):
    """D4E_MODE_LIST keeps every row on the device for the listing call;
    d4e_batch_run refuses it (argument check, before any device work)."""
    from d4gb.problem import Problem

    p = Problem(4, 2, [0xF, 0xF], [0x3], [4], 0xFF)
    with pytest.raises(engine.D4Error) as e:
        engine.batch_run([p], mode=engine.MODE_LIST)
    assert e.value.code == -1 and "d4e_batch_solutions" in str(e.value)
