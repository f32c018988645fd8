"""Puzzle descriptions and the seeded workload generators.

A :class:`Problem` is a board (``width`` <= 8 columns, ``rows[r]`` bit c set =
cell (r, c) must be covered) plus a piece library (Shape<8> values, bit
8*r + c, with a copy count each) and the allowed transforms ``sym`` in the
reference's Shape::transforms() order.

Workloads (all seeded, synthetic):

* :func:`pentomino_ring` -- 8x8 board minus its central 2x2, the 12 free
  pentominoes once each, all 8 transforms (the reference's CPU-runnable
  case; 520 tilings, 65 up to the board's D4 symmetry).
* :func:`single_large` -- 8 x 15 board with 3 seeded holes, 24 piece copies of
  4..6 cells grown by random accretion (duplicates merge into
  multiplicities), total area 117.
* :func:`batched_mix` -- independent instances with width 5..8, height 5..12,
  0..4 holes and a random 3..6-cell piece set whose area matches the board.
"""
from __future__ import annotations

import functools
import random
from dataclasses import dataclass, field
from typing import List

FULL_D4 = 0xFF
ROTATIONS = 0b01101001  # C4: identity, rot180, rot90 CW, rot90 CCW


@dataclass
class Problem:
    width: int
    height: int
    rows: List[int]
    shapes: List[int]
    counts: List[int]
    sym: int = FULL_D4
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def cells(self) -> int:
        return sum(bin(r).count("1") for r in self.rows)

    @property
    def piece_area(self) -> int:
        return sum(bin(s).count("1") * c for s, c in zip(self.shapes, self.counts))

    @property
    def copies(self) -> int:
        return sum(self.counts)

    def empty_area(self) -> int:
        """The reference's uint64 board (8 wide, <= 8 rows)."""
        assert self.width == 8 and self.height <= 8
        v = 0
        for r, m in enumerate(self.rows):
            v |= m << (8 * r)
        return v


# ---------------------------------------------------------------------------
# Shape<8> helpers (bit 8*r + c), restating the reference's Shape.cpp
# normalize / transform / canonical_form.
# ---------------------------------------------------------------------------
def normalize(v: int) -> int:
    if not v:
        return 0
    while not v & 0xFF:
        v >>= 8
    while not v & 0x0101010101010101:
        v >>= 1
    return v


_REV8 = bytes(int(f"{b:08b}"[::-1], 2) for b in range(256))
_M64 = (1 << 64) - 1


def _transpose8(x: int) -> int:
    """(r, c) -> (c, r) on an 8x8 bitboard (bit 8r + c): three delta swaps
    (the classic diagonal flip of chess bitboards)."""
    t = 0x0F0F0F0F00000000 & (x ^ (x << 28))
    x ^= t ^ (t >> 28)
    t = 0x3333000033330000 & (x ^ (x << 14))
    x ^= t ^ (t >> 14)
    t = 0x5500550055005500 & (x ^ (x << 7))
    x ^= t ^ (t >> 7)
    return x & _M64


def transform(v: int, t: int) -> int:
    """Transform t of the reference's order: bit 1 flips rows (r -> 7 - r),
    bit 0 flips columns (c -> 7 - c), then bit 2 swaps rows and columns."""
    b = v.to_bytes(8, "little")
    if (t >> 1) & 1:
        b = b[::-1]
    if t & 1:
        b = b.translate(_REV8)
    out = int.from_bytes(b, "little")
    if (t >> 2) & 1:
        out = _transpose8(out)
    return normalize(out)


@functools.lru_cache(maxsize=1 << 16)
def canonical(v: int, forms: int = FULL_D4) -> int:
    return min(transform(v, t) for t in range(8) if (forms >> t) & 1)


def cells_to_shape(cells) -> int:
    mr = min(r for r, _ in cells)
    mc = min(c for _, c in cells)
    v = 0
    for r, c in cells:
        v |= 1 << (8 * (r - mr) + (c - mc))
    return v


def grow_polyomino(rng: random.Random, size: int) -> int:
    """Random cell accretion from one seed cell; canonical under D4.  Cells
    stay within an 8x8 frame (size <= 8)."""
    cells = {(0, 0)}
    while len(cells) < size:
        r, c = rng.choice(sorted(cells))
        dr, dc = rng.choice(((0, 1), (0, -1), (1, 0), (-1, 0)))
        cells.add((r + dr, c + dc))
    return canonical(cells_to_shape(cells))


def merge_pieces(shapes: List[int]):
    """Identical shapes merge into one type with a multiplicity (first
    occurrence order)."""
    types: List[int] = []
    counts: List[int] = []
    for s in shapes:
        if s in types:
            counts[types.index(s)] += 1
        else:
            types.append(s)
            counts.append(1)
    return types, counts


def verify_tiling(p: "Problem", type_grid, step_grid) -> bool:
    """Independent cover check of a reported tiling: every board cell is
    covered by exactly one placement and holes by none; each placement
    (cells sharing a step number) is an allowed transform of its piece type;
    no type is used more often than its count."""
    H, W = p.height, p.width
    used = [0] * len(p.shapes)
    groups = {}
    for r in range(H):
        for c in range(W):
            t = int(type_grid[r][c])
            s = int(step_grid[r][c])
            on_board = (p.rows[r] >> c) & 1
            if not on_board:
                if t != -1 or s != -1:
                    return False
                continue
            if s < 0 or not 0 <= t < len(p.shapes):
                return False
            g = groups.setdefault(s, [t, []])
            if g[0] != t:
                return False
            g[1].append((r, c))
    for t, cells in groups.values():
        shape = normalize(cells_to_shape(cells))
        forms = {transform(p.shapes[t], k) for k in range(8) if (p.sym >> k) & 1}
        if shape not in forms:
            return False
        used[t] += 1
    return all(u <= n for u, n in zip(used, p.counts))


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------
PENTOMINOES = None  # filled lazily from the engine's catalogue


def pentomino_ring(pentominoes: List[int]) -> Problem:
    """8x8 minus the central 2x2 (60 cells), 12 free pentominoes x 1, D4."""
    rows = [0xFF] * 8
    rows[3] &= ~0x18 & 0xFF
    rows[4] &= ~0x18 & 0xFF
    return Problem(8, 8, rows, list(pentominoes), [1] * len(pentominoes), FULL_D4,
                   name="pentomino ring 8x8-2x2")


def _piece_sizes(rng: random.Random, area: int, lo: int, hi: int) -> List[int]:
    """Random piece sizes in [lo, hi] summing to `area` (area >= lo)."""
    sizes = []
    rem = area
    while rem > 0:
        options = [s for s in range(lo, hi + 1) if s <= rem and (s == rem or rem - s >= lo)]
        s = rng.choice(options)
        sizes.append(s)
        rem -= s
    return sizes


def single_large(seed: int) -> Problem:
    """8 x 15 board with 3 seeded holes; 24 piece copies of 4..6 cells grown by
    random accretion, sizes adjusted so the area is 117."""
    rng = random.Random(seed)
    W, H = 8, 15
    holes = rng.sample(range(W * H), 3)
    rows = [0xFF] * H
    for h in holes:
        rows[h // W] &= ~(1 << (h % W)) & 0xFF
    sizes = [rng.randint(4, 6) for _ in range(24)]
    while sum(sizes) != 117:
        i = rng.randrange(24)
        if sum(sizes) > 117 and sizes[i] > 4:
            sizes[i] -= 1
        elif sum(sizes) < 117 and sizes[i] < 6:
            sizes[i] += 1
    shapes = [grow_polyomino(rng, s) for s in sizes]
    types, counts = merge_pieces(shapes)
    return Problem(W, H, rows, types, counts, FULL_D4, name=f"single large 8x15 seed {seed}",
                   meta={"seed": seed, "holes": sorted(holes)})


def medium_board(seed: int = 77) -> Problem:
    """8 x 10 board minus 2 cells (78 cells) with 4..6-cell pieces of exactly
    that area (the profiling-size relative of single_large)."""
    rng = random.Random(seed)
    rows = [0xFF] * 6 + [0xF7, 0xEF] + [0xFF] * 2
    sizes = _piece_sizes(rng, 78, 4, 6)
    types, counts = merge_pieces([grow_polyomino(rng, k) for k in sizes])
    return Problem(8, 10, rows, types, counts, FULL_D4, name=f"medium 8x10 seed {seed}")


def batched_instance(rng: random.Random, idx: int = 0) -> Problem:
    W = rng.randint(5, 8)
    H = rng.randint(5, 12)
    n_holes = rng.randint(0, 4)
    holes = rng.sample(range(W * H), n_holes)
    rows = [(1 << W) - 1] * H
    for h in holes:
        rows[h // W] &= ~(1 << (h % W))
    area = W * H - n_holes
    sizes = _piece_sizes(rng, area, 3, 6)
    shapes = [grow_polyomino(rng, s) for s in sizes]
    types, counts = merge_pieces(shapes)
    return Problem(W, H, rows, types, counts, FULL_D4, name=f"mix#{idx} {W}x{H}",
                   meta={"holes": sorted(holes)})


def batched_mix(seed: int, n: int) -> List[Problem]:
    rng = random.Random(seed)
    return [batched_instance(rng, i) for i in range(n)]
