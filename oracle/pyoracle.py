"""ctypes wrapper of the CPU oracle (oracle/_build/libd4oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product library.  Problems are any
object with width / height / rows / shapes / counts / sym attributes.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB = ORACLE_DIR / "_build" / "libd4oracle.so"
REF_BIN = ORACLE_DIR / "_ref" / "d4ref"


def build() -> Path:
    """Compile the C restatement (make in oracle/)."""
    r = subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed\n{r.stdout}\n{r.stderr}")
    return LIB


class _Problem(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("rows", C.POINTER(C.c_uint16)),
        ("n_pieces", C.c_int32),
        ("shapes", C.POINTER(C.c_uint64)),
        ("counts", C.POINTER(C.c_uint32)),
        ("sym", C.c_uint32),
    ]


_lib = None


def _load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = C.CDLL(str(LIB))
        lib.or_solve_count.restype = C.c_int64
        lib.or_solve_count.argtypes = [C.POINTER(_Problem)]
        lib.or_solve.restype = C.c_int64
        lib.or_solve.argtypes = [C.POINTER(_Problem), C.c_int32, C.c_int64,
                                 C.POINTER(C.c_int8), C.POINTER(C.c_int8)]
        lib.or_canonical_grid.restype = None
        lib.or_canonical_grid.argtypes = [C.POINTER(_Problem), C.POINTER(C.c_int8),
                                          C.POINTER(C.c_int8)]
        lib.or_rowdp.restype = C.c_int32
        lib.or_rowdp.argtypes = [C.POINTER(_Problem), C.c_int32, C.c_double, C.c_uint64,
                                 C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                 C.POINTER(C.c_int32), C.POINTER(C.c_uint64)]
        lib.or_rowdp_lean.restype = C.c_int32
        lib.or_rowdp_lean.argtypes = [C.POINTER(_Problem), C.c_int32, C.c_int32,
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_uint64),
                                      C.POINTER(C.c_uint64), C.POINTER(C.c_double)]
        lib.or_check_tiling.restype = C.c_int32
        lib.or_check_tiling.argtypes = [C.POINTER(_Problem), C.c_int32, C.POINTER(C.c_int32),
                                        C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        _lib = lib
    return _lib


def _prob(p):
    rows = (C.c_uint16 * max(len(p.rows), 1))(*p.rows)
    shapes = (C.c_uint64 * max(len(p.shapes), 1))(*p.shapes)
    counts = (C.c_uint32 * max(len(p.counts), 1))(*p.counts)
    st = _Problem(p.width, p.height, C.cast(rows, C.POINTER(C.c_uint16)), len(p.shapes),
                  C.cast(shapes, C.POINTER(C.c_uint64)), C.cast(counts, C.POINTER(C.c_uint32)),
                  p.sym)
    return st, (rows, shapes, counts)


def solve_count(p) -> int:
    st, keep = _prob(p)
    r = _load().or_solve_count(C.byref(st))
    if r < 0:
        raise ValueError("oracle rejected the problem")
    return int(r)


def solve(p, single: bool = False, max_solutions: int = 1 << 20):
    """(n_found, type_grids, step_grids) with grids shaped (k, H, W)."""
    st, keep = _prob(p)
    cells = p.width * p.height
    tg = np.full((max(max_solutions, 1), cells), -1, dtype=np.int8)
    sg = np.full((max(max_solutions, 1), cells), -1, dtype=np.int8)
    n = _load().or_solve(C.byref(st), int(single), max_solutions,
                         tg.ctypes.data_as(C.POINTER(C.c_int8)),
                         sg.ctypes.data_as(C.POINTER(C.c_int8)))
    if n < 0:
        raise ValueError("oracle rejected the problem")
    k = min(int(n), max_solutions)
    return int(n), tg[:k].reshape(k, p.height, p.width), sg[:k].reshape(k, p.height, p.width)


def canonical_grid(p, grid) -> np.ndarray:
    st, keep = _prob(p)
    g = np.ascontiguousarray(np.asarray(grid, dtype=np.int8).reshape(-1))
    out = np.empty_like(g)
    _load().or_canonical_grid(C.byref(st), g.ctypes.data_as(C.POINTER(C.c_int8)),
                              out.ctypes.data_as(C.POINTER(C.c_int8)))
    return out.reshape(p.height, p.width)


def canonical_set(p, grids) -> set:
    return {canonical_grid(p, g).tobytes() for g in grids}


def rowdp(p, threads: int = 1, max_seconds: float = 0.0, max_children: int = 0) -> dict:
    """Exact row DP; max_seconds / max_children bound a sample (see
    d4oracle.h)."""
    st, keep = _prob(p)
    sizes = (C.c_uint64 * max(p.height, 1))()
    count = C.c_uint64()
    done = C.c_int32()
    total = C.c_uint64()
    r = _load().or_rowdp(C.byref(st), threads, max_seconds, max_children, sizes,
                         C.byref(count), C.byref(done), C.byref(total))
    if r != 0:
        raise ValueError("oracle rejected the problem")
    return {"level_sizes": list(sizes)[: done.value], "count": int(count.value),
            "levels_done": done.value, "states_total": int(total.value)}


def rowdp_lean(p, threads: int = 1, max_rows: int = 0) -> dict:
    """Exact row DP de-duplicating children as they are produced (memory =
    distinct states only); max_rows > 0 runs only the first whole rows."""
    st, keep = _prob(p)
    sizes = (C.c_uint64 * max(p.height, 1))()
    raw = (C.c_uint64 * max(p.height, 1))()
    count = C.c_uint64()
    secs = C.c_double()
    r = _load().or_rowdp_lean(C.byref(st), threads, max_rows, sizes, raw, C.byref(count),
                              C.byref(secs))
    if r != 0:
        raise ValueError("oracle rejected the problem" if r == -1 else "host memory ran out")
    rows = min(max_rows, p.height) if max_rows > 0 else p.height
    return {"level_sizes": list(sizes)[:rows], "raw_sizes": list(raw)[:rows],
            "count": int(count.value), "seconds": secs.value, "rows": rows}


def check_tiling(p, types, masks) -> bool:
    """masks: python ints over the W-stride bitboard (bit r*W + c)."""
    st, keep = _prob(p)
    n = len(types)
    t = (C.c_int32 * max(n, 1))(*types)
    lo = (C.c_uint64 * max(n, 1))(*[m & ((1 << 64) - 1) for m in masks])
    hi = (C.c_uint64 * max(n, 1))(*[m >> 64 for m in masks])
    return bool(_load().or_check_tiling(C.byref(st), n, t, lo, hi))


def grid_to_placements(p, type_grid, step_grid):
    """Splits a solution (type grid + step grid) into (types, masks)."""
    tg = np.asarray(type_grid).reshape(-1)
    sg = np.asarray(step_grid).reshape(-1)
    steps = {}
    for cell, (t, s) in enumerate(zip(tg, sg)):
        if s < 0:
            continue
        ty, m = steps.get(int(s), (int(t), 0))
        steps[int(s)] = (ty, m | (1 << cell))
    types = [steps[k][0] for k in sorted(steps)]
    masks = [steps[k][1] for k in sorted(steps)]
    return types, masks


def ref_run(p, mode: str) -> str:
    """Runs the reference's own solver (oracle/_ref/d4ref) on a problem; only
    where the reference sources were available to build it."""
    if not REF_BIN.exists():
        raise FileNotFoundError(REF_BIN)
    lines = [f"{p.width} {p.height} {p.sym} {mode}", " ".join(str(r) for r in p.rows),
             str(len(p.shapes))]
    lines += [f"{s} {c}" for s, c in zip(p.shapes, p.counts)]
    r = subprocess.run([str(REF_BIN)], input="\n".join(lines) + "\n", capture_output=True,
                       text=True, check=True)
    return r.stdout
