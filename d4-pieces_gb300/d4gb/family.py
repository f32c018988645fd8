"""Board families: one base board, several regions, and one configuration
per choice of a removed cell in every region (the reference's Board<8>,
src/board.hpp:9-57).  The reference's research driver (src/search.cpp:25-54,
the Verify / AtomicCount searchers over Naming-ranked piece combinations)
asks, for every configuration, which piece combinations tile it and how many
configurations each combination tiles; here every configuration is one
instance of a d4e_batch_sets batch, whose final rows give exactly the tiling
combinations with their numbers of tilings.

Text format (the reference's Board / Shape parsers, src/board.hpp:15-38,
src/Shape.hpp:49-77): rows end with a newline (a leading newline is
skipped); a letter or digit marks a cell of the region with that name;
'*', '@', '#', 'X', '%' mark a cell of the base board; ' ', '.', '-', '_' a
position outside it; other characters are ignored.  Every region cell is a
base cell too.  Boards are 8 wide (Shape<8>).
"""
from __future__ import annotations

import bisect
import itertools
import math
from dataclasses import dataclass, field
from typing import Dict, Iterator, List, Sequence, Tuple

import numpy as np

from .problem import Problem

_CELL = set("*1@#X%")
_EMPTY = set(" 0.-_")


def _valid(ch: str) -> bool:
    return ch.isascii() and ch.isalnum()


def parse_shape(text: str, width: int = 8) -> int:
    """Shape<width> text -> bit mask (bit width * row + column).  As in the
    reference, a row longer than the width runs on into the next row's bits
    and bits past 63 are dropped."""
    if text.startswith("\n"):
        text = text[1:]
    row_start, pos, value = 0, 0, 0
    for ch in text:
        if ch in _EMPTY:
            pos += 1
        elif ch in _CELL:
            if row_start + pos < 64:
                value |= 1 << (row_start + pos)
            pos += 1
        elif ch == "\n":
            row_start += width
            pos = 0
    return value


@dataclass
class BoardFamily:
    base: int
    regions: List[int]
    names: List[str] = field(default_factory=list)
    width: int = 8

    @classmethod
    def from_file(cls, path, width: int = 8) -> "BoardFamily":
        with open(path) as f:
            return cls.from_text(f.read(), width)

    @classmethod
    def from_text(cls, text: str, width: int = 8) -> "BoardFamily":
        names: List[str] = []
        for ch in text:
            if _valid(ch) and ch not in names:
                names.append(ch)
        base = "".join("#" if _valid(ch) else ch for ch in text)
        regions = []
        for k in names:
            # The region's own cells; the other regions' cells are outside it
            # (the reference keeps the base's non-region marks as they are).
            regions.append(parse_shape("".join(
                ("#" if ch == k else ".") if _valid(ch) else ch for ch in text), width))
        return cls(parse_shape(base, width), regions, names, width)

    @property
    def left(self) -> int:
        """Cells of every configuration (base minus one cell per region)."""
        return bin(self.base).count("1") - len(self.regions)

    @property
    def count(self) -> int:
        n = 1
        for r in self.regions:
            n *= bin(r).count("1")
        return n

    def configs(self) -> Iterator[int]:
        """Each board of the family: the base with one cell of every region
        removed (regions in order of first appearance in the text)."""
        cells = [[b for b in range(64) if (r >> b) & 1] for r in self.regions]
        for pick in itertools.product(*cells):
            m = self.base
            for b in pick:
                m &= ~(1 << b)
            yield m


def board_problem(mask: int, shapes: Sequence[int], counts: Sequence[int],
                  sym: int = 0xFF, name: str = "", width: int = 8) -> Problem:
    """A board mask (bit width * row + column) as an engine problem; pieces
    are 8-wide catalogue masks (bit 8 * row + column)."""
    full = (1 << width) - 1
    rows = [(mask >> (width * r)) & full for r in range(64 // width)]
    while rows and rows[-1] == 0:
        rows.pop()
    return Problem(width, max(len(rows), 1), rows or [0], list(shapes), list(counts), sym,
                   name=name or f"board {mask:#x}")


def pieces_by_size(min_m: int, max_m: int, onesided: bool = False) -> List[int]:
    """The catalogue's pieces of min_m..max_m cells (the reference's
    known_shapes[m] / known_C_shapes[m] tables), in catalogue order."""
    from . import engine as E

    out: List[int] = []
    for m in range(min_m, max_m + 1):
        out.extend(E.catalogue(m, onesided))
    return out


class Naming:
    """Ranks of piece combinations (the reference's Naming,
    src/naming.cpp:34-90, src/naming.inl:6-72): a combination picks distinct
    pieces, k_m of the sizes[m] pieces of each size m in min_m..max_m, with
    min_n <= sum k_m <= max_n and sum m * k_m == tgt.  Ranks run over the
    size profiles (k_min_m, ..., k_max_m) in lexicographic order; inside a
    profile the rank is mixed-radix over the sizes, the most significant
    digit being the smallest size, each digit the combination's
    lexicographic rank among the C(sizes[m], k_m) choices.  The ranks are a
    file format of the reference (its ledgers are indexed by them), so the
    order here is the reference's."""

    def __init__(self, min_m: int, max_m: int, min_n: int, max_n: int, tgt: int,
                 sizes: Dict[int, int] | Sequence[int]):
        self.min_m, self.max_m, self.min_n, self.max_n, self.tgt = min_m, max_m, min_n, max_n, tgt
        if isinstance(sizes, dict):
            self.sizes = {m: int(sizes.get(m, 0)) for m in range(min_m, max_m + 1)}
        else:
            self.sizes = {m: int(sizes[m]) if m < len(sizes) else 0
                          for m in range(min_m, max_m + 1)}
        self.profiles: List[Tuple[int, ...]] = []
        self._walk([], tgt, 0)
        self.radix = [[math.comb(self.sizes[min_m + d], k) for d, k in enumerate(pr)]
                      for pr in self.profiles]
        self.starts = []
        total = 0
        for r in self.radix:
            self.starts.append(total)
            total += math.prod(r)
        self._size = total

    def _walk(self, cur: List[int], left: int, n: int) -> None:
        m = self.min_m + len(cur)
        if left == 0:
            if n >= self.min_n:
                self.profiles.append(tuple(cur + [0] * (self.max_m - m + 1)))
            return
        if m > self.max_m:
            return
        k = 0
        while k * m <= left and n + k <= self.max_n and k <= self.sizes[m]:
            self._walk(cur + [k], left - k * m, n + k)
            k += 1

    def size(self) -> int:
        return self._size

    def size_pieces(self) -> int:
        return sum(self.sizes.values())

    def name(self, chosen: Sequence[Sequence[int]]) -> int | None:
        """chosen[d]: the picked piece indices of size min_m + d (any order).
        None when the combination is not one of the ranked ones."""
        picks = [sorted(set(c)) for c in chosen]
        profile = tuple(len(c) for c in picks)
        lo = bisect.bisect_left(self.profiles, profile)
        if lo == len(self.profiles) or self.profiles[lo] != profile:
            return None
        nm = 0
        for d, c in enumerate(picks):
            nm = nm * self.radix[lo][d] + _comb_rank(c, self.sizes[self.min_m + d])
        return self.starts[lo] + nm

    def resolve(self, nm: int) -> List[List[int]] | None:
        if not 0 <= nm < self._size:
            return None
        pid = bisect.bisect_right(self.starts, nm) - 1
        nm -= self.starts[pid]
        digits = []
        for r in reversed(self.radix[pid]):
            digits.append(nm % r)
            nm //= r
        digits.reverse()
        return [_comb_unrank(x, k, self.sizes[self.min_m + d])
                for d, (x, k) in enumerate(zip(digits, self.profiles[pid]))]


def _comb_rank(c: Sequence[int], n: int) -> int:
    """Lexicographic rank of the sorted k-subset c of range(n)."""
    k, nm, j = len(c), 0, 0
    for i in range(n):
        if not k:
            break
        if j < len(c) and c[j] == i:
            j += 1
            k -= 1
        else:
            nm += math.comb(n - i - 1, k - 1)
    return nm


def _comb_unrank(nm: int, k: int, n: int) -> List[int]:
    out = []
    for i in range(n):
        if not k:
            break
        below = math.comb(n - i - 1, k - 1)
        if nm < below:
            out.append(i)
            k -= 1
        else:
            nm -= below
    return out


SetList = List[Tuple[Tuple[int, ...], int]]


@dataclass
class FamilySets:
    """Kept piece sets of a family run, as arrays: the distinct boards
    (`masks`), each board's sets in rows offsets[i]..offsets[i+1]-1 of
    `copies` (copies per piece) and `tilings`, and `mult[i]`, how many of
    the family's configurations are board i."""
    masks: List[int]
    mult: np.ndarray
    offsets: np.ndarray
    copies: np.ndarray
    tilings: np.ndarray
    stats: dict

    def per_config(self) -> Dict[int, SetList]:
        out = {}
        for i, m in enumerate(self.masks):
            a, b = int(self.offsets[i]), int(self.offsets[i + 1])
            out[m] = list(zip(map(tuple, self.copies[a:b].tolist()),
                              self.tilings[a:b].tolist()))
        return out

    def ledger(self) -> Tuple[np.ndarray, np.ndarray]:
        """(distinct sets, configurations each tiles): every board's sets
        are distinct, so a set's count is the sum of its boards' mult."""
        if not len(self.copies):
            return self.copies, np.zeros(0, np.int64)
        k = self.copies.shape[1]
        rows = np.ascontiguousarray(self.copies).view(np.dtype((np.void, k))).ravel()
        uniq, inv = np.unique(rows, return_inverse=True)
        per_row = np.repeat(self.mult, np.diff(self.offsets).astype(np.int64))
        n = np.bincount(inv.ravel(), weights=per_row, minlength=len(uniq)).astype(np.int64)
        return uniq.view(np.uint8).reshape(-1, k), n


def family_sets(family: BoardFamily, shapes: Sequence[int], counts: Sequence[int] | None = None,
                sym: int = 0xFF, min_n: int = 0, max_n: int = 1 << 30, device: int = 0,
                max_states: int = 0, sequential: bool = False) -> FamilySets:
    """Every configuration of the family in one piece-set batch; keeps the
    sets of min_n..max_n pieces covering `left` cells (the combinations the
    reference ranks).  Overlapping regions can map two picks to one board:
    each distinct board is solved once and counted with its multiplicity;
    a board that kept more cells (a cell cleared twice) has no kept set."""
    from . import engine as E

    counts = list(counts) if counts is not None else [1] * len(shapes)
    areas = np.array([bin(v).count("1") for v in shapes], np.int64)
    mult_of: Dict[int, int] = {}
    for m in family.configs():
        mult_of[m] = mult_of.get(m, 0) + 1
    uniq = sorted(mult_of)
    probs = [board_problem(m, shapes, counts, sym, width=family.width) for m in uniq]
    (offs, copies, tilings), results, st = E.batch_sets(
        probs, device=device, max_states=max_states, sequential=sequential, arrays=True)
    for m, r in zip(uniq, results):
        if r["status"] != 0:
            raise E.D4Error(r["status"], f"configuration {m:#x} failed")
    k = len(shapes)
    c = copies[:, :k]
    wide = c.astype(np.int64)
    n_pieces = wide.sum(axis=1)
    keep = (n_pieces >= min_n) & (n_pieces <= max_n) & (wide @ areas == family.left)
    board = np.repeat(np.arange(len(uniq)), np.diff(offs).astype(np.int64))
    kept_offs = np.zeros(len(uniq) + 1, np.int64)
    np.cumsum(np.bincount(board[keep], minlength=len(uniq)), out=kept_offs[1:])
    return FamilySets(uniq, np.array([mult_of[m] for m in uniq], np.int64), kept_offs,
                      np.ascontiguousarray(c[keep]), tilings[keep], st)


def tiling_sets(family: BoardFamily, shapes: Sequence[int], counts: Sequence[int] | None = None,
                sym: int = 0xFF, min_n: int = 0, max_n: int = 1 << 30, device: int = 0,
                max_states: int = 0, sequential: bool = False, stats: dict | None = None,
                ) -> Tuple[Dict[int, SetList], Dict[Tuple[int, ...], int]]:
    """For every configuration of the family: the piece multisets of min_n..
    max_n pieces that tile it (counts are maxima; default one copy of each
    piece, as in the reference's piece combinations), with their numbers of
    tilings, all configurations in one batch.  Also returns the ledger: for
    each multiset, how many configurations it tiles (the reference's
    AtomicCount ledger, keyed by the multiset instead of its rank).
    sequential runs the boards one at a time; stats receives the batch's
    engine counters."""
    fs = family_sets(family, shapes, counts, sym, min_n, max_n, device, max_states, sequential)
    if stats is not None:
        stats.update(fs.stats)
    sets, n = fs.ledger()
    return fs.per_config(), dict(zip(map(tuple, sets.tolist()), n.tolist()))


@dataclass
class FamilyRun:
    naming: Naming
    shapes: List[int]
    sets: FamilySets
    ledger: Dict[int, int]          # Naming rank -> configurations it tiles

    @property
    def stats(self) -> dict:
        return self.sets.stats

    @property
    def per_config(self) -> Dict[int, SetList]:
        return self.sets.per_config()

    def unsolved(self, family: BoardFamily) -> List[int]:
        """Configurations no combination tiles (the reference's ZERO-count
        report, src/searcher.cpp:110-115)."""
        empty = {m for i, m in enumerate(self.sets.masks)
                 if self.sets.offsets[i] == self.sets.offsets[i + 1]}
        return [m for m in family.configs() if m in empty]


def family_ledger(family: BoardFamily, min_m: int, max_m: int, min_n: int, max_n: int,
                  rotations_only: bool = False, device: int = 0, max_states: int = 0,
                  sequential: bool = False) -> FamilyRun:
    """The reference's board-family search with its AtomicCount ledger
    (src/search.cpp:36-53, 245-270): pieces are the catalogue's free (or,
    rotations only, one-sided) polyominoes of min_m..max_m cells, each used
    at most once; a combination of min_n..max_n of them covering `left`
    cells is named by its Naming rank; the ledger maps each rank to the
    number of configurations the combination tiles."""
    from .problem import FULL_D4, ROTATIONS

    shapes = pieces_by_size(min_m, max_m, rotations_only)
    sizes = {m: 0 for m in range(min_m, max_m + 1)}
    for v in shapes:
        sizes[bin(v).count("1")] += 1
    naming = Naming(min_m, max_m, min_n, max_n, family.left, sizes)
    fs = family_sets(family, shapes, None, ROTATIONS if rotations_only else FULL_D4,
                     min_n, max_n, device, max_states, sequential)
    sets, counts = fs.ledger()
    # piece index -> (size digit, index within its size)
    digit, within, seen = [], [], {m: 0 for m in range(min_m, max_m + 1)}
    for v in shapes:
        m = bin(v).count("1")
        digit.append(m - min_m)
        within.append(seen[m])
        seen[m] += 1
    ledger: Dict[int, int] = {}
    for row, n in zip(sets.tolist(), counts.tolist()):
        chosen: List[List[int]] = [[] for _ in range(min_m, max_m + 1)]
        for p, k in enumerate(row):
            if k:
                chosen[digit[p]].append(within[p])
        rank = naming.name(chosen)
        if rank is None:
            raise ValueError(f"combination {row} has no Naming rank")
        ledger[rank] = n
    return FamilyRun(naming, shapes, fs, ledger)


def read_ledger_file(path, configs: int, names: int, kind: str = "bit"):
    """Reads a FileBit / FileByte ledger file (the reference's layout,
    src/search.cpp:56-226; written by the C++ facade's LedgerFile):
    returns (descriptors[configs, 4] = shape, count, solved ms, padding;
    tiled[names] = configurations each rank tiles; logged[names, configs]
    booleans)."""
    width = configs if kind == "byte" else (configs + 7) // 8
    raw = np.fromfile(path, dtype=np.uint8)
    want = configs * 32 + names * 8 + names * width
    if raw.size != want:
        raise ValueError(f"ledger file has {raw.size} bytes, this family needs {want}")
    desc = raw[: configs * 32].view(np.uint64).reshape(configs, 4)
    tiled = raw[configs * 32: configs * 32 + names * 8].view(np.uint64)
    led = raw[configs * 32 + names * 8:].reshape(names, width)
    if kind == "byte":
        logged = led != 0
    else:
        logged = np.unpackbits(led, axis=1, bitorder="little")[:, :configs].astype(bool)
    return desc, tiled, logged

