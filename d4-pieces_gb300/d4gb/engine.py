"""ctypes bindings of libd4e.so (include/d4e.h).

Mirrors the reference's host API for the GPU search path:
``compute_frow_on_cpu`` / ``transfer_frow_to_gpu`` (src/frow.h:10-12) become
:class:`Frow`, ``CudaSearcher`` (src/searcher_cuda.h:10-38) becomes
:class:`CudaSearcher`.  Errors raise :class:`D4Error` (the reference throws
``std::runtime_error``).  There is no CPU fallback: importing this module on a
machine without the built library raises immediately.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from .build import LIB_PATH

if not LIB_PATH.exists():
    raise ImportError(f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")

_lib = C.CDLL(str(LIB_PATH))

D4E_OK = 0
D4E_ERR_INVALID = -1
D4E_ERR_CUDA = -2
D4E_ERR_NOMEM = -3
D4E_ERR_UNSUPPORTED = -4
D4E_ERR_STATE = -5
D4E_KEEP_LEVELS = 1
D4E_AUTOTUNE = 2
D4E_DEDUP_DIRECT = 4
D4E_DEDUP_PARTITIONED = 8
_DEDUP_FLAGS = {None: 0, "auto": 0, "direct": D4E_DEDUP_DIRECT,
                "partitioned": D4E_DEDUP_PARTITIONED}
D4E_BATCH_SEQUENTIAL = 1

_u64p = C.POINTER(C.c_uint64)
_u32p = C.POINTER(C.c_uint32)
_u8p = C.POINTER(C.c_uint8)
_i8p = C.POINTER(C.c_int8)
_i16p = C.POINTER(C.c_int16)


class D4Error(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"d4e error {code}: {msg}")
        self.code = code


class Stats(C.Structure):
    _fields_ = [
        ("rows", C.c_uint64),
        ("states_in", C.c_uint64),
        ("states_raw", C.c_uint64),
        ("states_out", C.c_uint64),
        ("peak_frontier", C.c_uint64),
        ("expand_launches", C.c_uint64),
        ("compact_launches", C.c_uint64),
        ("retries", C.c_uint64),
        ("other_launches", C.c_uint64),
        ("h2d_bytes", C.c_uint64),
        ("d2h_bytes", C.c_uint64),
        ("expand_ms", C.c_double),
        ("compact_ms", C.c_double),
        ("run_ms", C.c_double),
        ("record_bytes", C.c_uint64),
        ("slot_bytes", C.c_uint64),
        ("paused", C.c_uint64),
        ("splits", C.c_uint64),
        ("failed", C.c_uint64),
        ("restarts", C.c_uint64),
        ("step_wall_ms", C.c_double),
        ("upload_ms", C.c_double),
        ("keep_ms", C.c_double),
        ("trace_ms", C.c_double),
        ("tune_ms", C.c_double),
        ("tuned_chunk_cap", C.c_uint64),
        ("tuned_chunks_per_warp", C.c_uint64),
        ("tuned_ctas_per_sm", C.c_uint64),
        ("tuned_load", C.c_double),
        ("compact_slots", C.c_uint64),
        ("phase_ms", C.c_double * 6),
        ("partitioned", C.c_uint64),
        ("partition_fallbacks", C.c_uint64),
        ("merge_ms", C.c_double),
        ("tuned_compact_ctas", C.c_uint64),
        ("tuned_compact_stages", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["phase_ms"] = list(self.phase_ms)
        return d


class BatchOpts(C.Structure):
    _fields_ = [
        ("mode", C.c_uint32),
        ("flags", C.c_uint32),
        ("device", C.c_int32),
        ("reserved", C.c_uint32),
        ("memory_budget", C.c_uint64),
        ("max_states", C.c_uint64),
        ("beam", C.c_uint64),
    ]


class Result(C.Structure):
    _fields_ = [
        ("tag", C.c_uint64),
        ("status", C.c_int32),
        ("mode", C.c_uint32),
        ("count", C.c_uint64),
        ("found", C.c_uint32),
        ("rows", C.c_uint32),
        ("queued_ms", C.c_double),
        ("latency_ms", C.c_double),
        ("grid", C.c_int8 * 512),
        ("steps", C.c_int16 * 512),
    ]

    def as_dict(self, width: int = 0, height: int = 0) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in ("grid", "steps")}
        if self.found and width and height:
            n = width * height
            d["grid"] = np.frombuffer(bytes(self.grid), dtype=np.int8)[:n] \
                .reshape(height, width).copy()
            d["steps"] = np.frombuffer(bytes(self.steps), dtype=np.int16)[:n] \
                .reshape(height, width).copy()
        return d


class ServerOpts(C.Structure):
    _fields_ = [
        ("device", C.c_int32),
        ("max_active", C.c_uint32),
        ("memory_budget", C.c_uint64),
        ("max_states", C.c_uint64),
        ("beam", C.c_uint64),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_uint64),
        ("admitted", C.c_uint64),
        ("completed", C.c_uint64),
        ("failed", C.c_uint64),
        ("steps", C.c_uint64),
        ("peak_active", C.c_uint64),
        ("peak_projected", C.c_uint64),
        ("states_out", C.c_uint64),
        ("busy_ms", C.c_double),
        ("moved", C.c_uint64),
        ("lane_steps", C.c_uint64 * 2),
        ("lane_busy_ms", C.c_double * 2),
        ("lane_kernel_ms", C.c_double * 2),
        ("lane_inst_rows", C.c_uint64 * 2),
        ("restarts", C.c_uint64),
        ("paused", C.c_uint64),
        ("lane_admit_ms", C.c_double * 2),
        ("lane_collect_ms", C.c_double * 2),
        ("lane_upload_ms", C.c_double * 2),
        ("lane_solve_one_ms", C.c_double * 2),
        ("lane_retries", C.c_uint64 * 2),
        ("lane_phase_ms", (C.c_double * 6) * 2),
        ("preemptions", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        def plain(v):
            if isinstance(v, (int, float)):
                return v
            return [plain(x) for x in v]
        return {k: plain(getattr(self, k)) for k, _ in self._fields_}


class Instance(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("rows", _u8p),
        ("n_pieces", C.c_uint32),
        ("shapes", _u64p),
        ("counts", _u32p),
        ("sym", C.c_uint32),
    ]


def _sig(name, res, *args):
    f = getattr(_lib, name)
    f.restype = res
    f.argtypes = list(args)
    return f


_lib.d4e_last_error.restype = C.c_char_p
_lib.d4e_version.restype = C.c_char_p
_sig("d4e_show_gpu_devices", C.c_int)
_sig("d4e_device_count", C.c_int, C.POINTER(C.c_int32))
_sig("d4e_catalogue", C.c_int, C.c_uint32, C.c_int32, _u64p, C.c_uint32, _u32p)
_sig("d4e_frow_create", C.c_int, _u64p, _u32p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32,
     C.POINTER(C.c_void_p))
_sig("d4e_frow_transfer", C.c_int, C.c_void_p, C.c_int32)
_sig("d4e_frow_placements", C.c_int, C.c_void_p, C.c_uint32, _u32p)
_sig("d4e_frow_destroy", None, C.c_void_p)
_sig("d4e_searcher_create", C.c_int, C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p))
_sig("d4e_searcher_create_board", C.c_int, C.c_void_p, C.c_uint32, _u8p, C.c_uint32,
     C.POINTER(C.c_void_p))
_sig("d4e_searcher_get_height", C.c_int, C.c_void_p, _u32p)
_sig("d4e_searcher_size", C.c_int, C.c_void_p, _u64p)
_sig("d4e_searcher_bucket_size", C.c_int, C.c_void_p, C.c_uint32, _u64p)
_sig("d4e_searcher_next_size", C.c_int, C.c_void_p, _u64p)
_sig("d4e_searcher_search_GPU", C.c_int, C.c_void_p)
_sig("d4e_searcher_run", C.c_int, C.c_void_p)
_sig("d4e_searcher_count", C.c_int, C.c_void_p, _u64p)
_sig("d4e_searcher_solutions", C.c_int, C.c_void_p, C.c_uint64, C.c_int32, _i8p, _i8p, _u64p)
_sig("d4e_searcher_level_sizes", C.c_int, C.c_void_p, _u64p, C.c_uint32, _u32p)
_sig("d4e_searcher_stats", C.c_int, C.c_void_p, C.POINTER(Stats))
_sig("d4e_searcher_set_limit", C.c_int, C.c_void_p, C.c_uint64)
_sig("d4e_searcher_destroy", None, C.c_void_p)
_sig("d4e_batch_count", C.c_int, C.POINTER(Instance), C.c_uint32, C.c_uint32, C.c_int32, _u64p,
     C.POINTER(Stats))
_sig("d4e_batch_run", C.c_int, C.POINTER(Instance), C.c_uint32, C.POINTER(BatchOpts),
     C.POINTER(Result), C.POINTER(Stats))
_sig("d4e_batch_sets", C.c_int, C.POINTER(Instance), C.c_uint32, C.POINTER(BatchOpts),
     C.POINTER(Result), _u64p, _u8p, _u64p, C.c_uint64, C.POINTER(Stats))
_sig("d4e_batch_solutions", C.c_int, C.POINTER(Instance), C.c_uint32, C.POINTER(BatchOpts),
     C.c_uint64, C.POINTER(Result), _u64p, _i8p, _i16p, C.c_uint64, C.POINTER(Stats))
_sig("d4e_server_create", C.c_int, C.POINTER(ServerOpts), C.POINTER(C.c_void_p))
_sig("d4e_server_submit", C.c_int, C.c_void_p, C.POINTER(Instance), C.c_uint32, C.c_uint64)
_sig("d4e_server_poll", C.c_int, C.c_void_p, C.POINTER(Result), C.c_uint32, _u32p)
_sig("d4e_server_drain", C.c_int, C.c_void_p, C.c_double)
_sig("d4e_server_stats_get", C.c_int, C.c_void_p, C.POINTER(ServerStats))
_sig("d4e_server_destroy", None, C.c_void_p)
_sig("d4e_autotune_clear", None)
_sig("d4e_release_cached_memory", None)
_sig("d4e_canonical_grid", C.c_int, C.c_uint32, C.c_uint32, _u8p, _i8p, _i8p)
_sig("d4e_count_noalloc", C.c_int, C.POINTER(Instance), C.c_void_p, _u64p, _u64p)


def lib() -> C.CDLL:
    return _lib


def _check(rc: int) -> None:
    if rc != D4E_OK:
        raise D4Error(rc, _lib.d4e_last_error().decode())


def _arr(ctype, values):
    a = (ctype * max(len(values), 1))(*values)
    return a


def version() -> str:
    return _lib.d4e_version().decode()


def device_count() -> int:
    n = C.c_int32()
    _check(_lib.d4e_device_count(C.byref(n)))
    return n.value


def show_gpu_devices() -> None:
    _check(_lib.d4e_show_gpu_devices())


def catalogue(m: int, onesided: bool = False) -> list[int]:
    n = C.c_uint32()
    _check(_lib.d4e_catalogue(m, int(onesided), None, 0, C.byref(n)))
    out = (C.c_uint64 * n.value)()
    _check(_lib.d4e_catalogue(m, int(onesided), out, n.value, C.byref(n)))
    return list(out)


class Frow:
    """Placement tables of a piece library for boards of one width
    (compute_frow_on_cpu + transfer_frow_to_gpu)."""

    def __init__(self, shapes: Sequence[int], counts: Sequence[int], sym: int = 0xFF,
                 width: int = 8, device: Optional[int] = 0, show_report: bool = False):
        self._h = C.c_void_p()
        self.shapes = list(shapes)
        self.counts = list(counts)
        self.sym = sym
        self.width = width
        s = _arr(C.c_uint64, self.shapes)
        c = _arr(C.c_uint32, self.counts)
        _check(_lib.d4e_frow_create(s, c, len(self.shapes), sym, width, int(show_report),
                                    C.byref(self._h)))
        if device is not None:
            self.transfer(device)

    def transfer(self, device: int = 0) -> None:
        _check(_lib.d4e_frow_transfer(self._h, device))

    def placements(self, col: int) -> int:
        n = C.c_uint32()
        _check(_lib.d4e_frow_placements(self._h, col, C.byref(n)))
        return n.value

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.d4e_frow_destroy(self._h)
            self._h = C.c_void_p()


class CudaSearcher:
    """One puzzle, one board row per :meth:`search_GPU` (src/searcher_cuda.h:10-38)."""

    def __init__(self, frow: Frow, empty_area: Optional[int] = None,
                 rows: Optional[Sequence[int]] = None, keep_levels: bool = False,
                 autotune: bool = False, dedup: Optional[str] = None):
        self._frow = frow
        self._h = C.c_void_p()
        if empty_area is not None:
            if keep_levels:
                raise ValueError("keep_levels needs the rows= form")
            _check(_lib.d4e_searcher_create(frow._h, C.c_uint64(empty_area), C.byref(self._h)))
            self.width = 8
            self.rows = [(empty_area >> (8 * r)) & 0xFF for r in range(8)]
            while self.rows and self.rows[-1] == 0:
                self.rows.pop()
        else:
            self.rows = list(rows)
            self.width = frow.width
            r = _arr(C.c_uint8, self.rows)
            flags = ((D4E_KEEP_LEVELS if keep_levels else 0) | (D4E_AUTOTUNE if autotune else 0)
                     | _DEDUP_FLAGS[dedup])
            _check(_lib.d4e_searcher_create_board(frow._h, len(self.rows), r, flags,
                                                  C.byref(self._h)))
        self.height = len(self.rows)

    def get_height(self) -> int:
        v = C.c_uint32()
        _check(_lib.d4e_searcher_get_height(self._h, C.byref(v)))
        return v.value

    def size(self, bucket: Optional[int] = None) -> int:
        v = C.c_uint64()
        if bucket is None:
            _check(_lib.d4e_searcher_size(self._h, C.byref(v)))
        else:
            _check(_lib.d4e_searcher_bucket_size(self._h, bucket, C.byref(v)))
        return v.value

    def next_size(self) -> int:
        v = C.c_uint64()
        _check(_lib.d4e_searcher_next_size(self._h, C.byref(v)))
        return v.value

    def search_GPU(self) -> None:
        _check(_lib.d4e_searcher_search_GPU(self._h))

    def run(self) -> None:
        _check(_lib.d4e_searcher_run(self._h))

    def count(self) -> int:
        v = C.c_uint64()
        _check(_lib.d4e_searcher_count(self._h, C.byref(v)))
        return v.value

    def level_sizes(self) -> list[int]:
        n = C.c_uint32()
        _check(_lib.d4e_searcher_level_sizes(self._h, None, 0, C.byref(n)))
        buf = (C.c_uint64 * max(n.value, 1))()
        _check(_lib.d4e_searcher_level_sizes(self._h, buf, n.value, C.byref(n)))
        return list(buf)[: n.value]

    def solutions(self, max_solutions: int, single: bool = False):
        """(type_grids, step_grids) as int8 arrays of shape (n, height, width)."""
        cells = self.width * self.height
        tg = np.full((max(max_solutions, 1), cells), -1, dtype=np.int8)
        sg = np.full((max(max_solutions, 1), cells), -1, dtype=np.int8)
        n = C.c_uint64()
        _check(_lib.d4e_searcher_solutions(self._h, max_solutions, int(single),
                                           tg.ctypes.data_as(_i8p), sg.ctypes.data_as(_i8p),
                                           C.byref(n)))
        k = n.value
        return (tg[:k].reshape(k, self.height, self.width),
                sg[:k].reshape(k, self.height, self.width))

    def set_limit(self, max_states: int) -> None:
        _check(_lib.d4e_searcher_set_limit(self._h, max_states))

    def stats(self) -> dict:
        st = Stats()
        _check(_lib.d4e_searcher_stats(self._h, C.byref(st)))
        return st.as_dict()

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib.d4e_searcher_destroy(self._h)
            self._h = C.c_void_p()


def _instances(problems) -> tuple:
    arr = (Instance * max(len(problems), 1))()
    keep = []
    for i, p in enumerate(problems):
        rows = _arr(C.c_uint8, p.rows)
        shapes = _arr(C.c_uint64, p.shapes)
        counts = _arr(C.c_uint32, p.counts)
        keep += [rows, shapes, counts]
        arr[i] = Instance(p.width, p.height, C.cast(rows, _u8p), len(p.shapes),
                          C.cast(shapes, _u64p), C.cast(counts, _u32p), p.sym)
    return arr, keep


def batch_count(problems, sequential: bool = False, device: int = 0):
    """Counts for a list of problems; returns (counts, stats dict)."""
    arr, keep = _instances(problems)
    out = (C.c_uint64 * max(len(problems), 1))()
    st = Stats()
    _check(_lib.d4e_batch_count(arr, len(problems), D4E_BATCH_SEQUENTIAL if sequential else 0,
                                device, out, C.byref(st)))
    return list(out)[: len(problems)], st.as_dict()


MODE_COUNT = 0
MODE_SOLVE_ONE = 1


D4E_BATCH_WIDE_KEYS = 2
D4E_BATCH_AUTOTUNE = 4


def batch_run(problems, mode: int = MODE_COUNT, sequential: bool = False, device: int = 0,
              memory_budget: int = 0, max_states: int = 0, beam: int = 0,
              wide_keys: bool = False, autotune: bool = False, dedup: Optional[str] = None):
    """Runs a batch through d4e_batch_run; returns (results, stats dict).
    Each result is a dict (status, count, found, rows, latency_ms, and for a
    found solve-one tiling height x width "grid" (types) and "steps")."""
    arr, keep = _instances(problems)
    n = len(problems)
    res = (Result * max(n, 1))()
    flags = ((D4E_BATCH_SEQUENTIAL if sequential else 0) | (D4E_BATCH_WIDE_KEYS if wide_keys else 0)
             | (D4E_BATCH_AUTOTUNE if autotune else 0) | (_DEDUP_FLAGS[dedup] << 1))
    o = BatchOpts(mode, flags, device, 0, memory_budget, max_states, beam)
    st = Stats()
    _check(_lib.d4e_batch_run(arr, n, C.byref(o), res, C.byref(st)))
    return ([res[i].as_dict(problems[i].width, problems[i].height) for i in range(n)],
            st.as_dict())


MODE_SETS = 2
SET_PIECES = 64


def batch_sets(problems, device: int = 0, memory_budget: int = 0, max_states: int = 0,
               sequential: bool = False, wide_keys: bool = False, max_sets: int = 1 << 22,
               arrays: bool = False):
    """Piece-set mode (d4e_batch_sets): for each problem, the piece multisets
    that tile its board (the problem's counts are maxima), as a list of
    (copies per piece, tilings) sorted by copies; plus the results and stats.
    The output buffers are allocated untouched (pages are only mapped where
    sets are written); when the batch has more than max_sets sets it runs
    once more with room for the number the first run reported.  arrays=True
    returns (offsets[n + 1], copies[sets, 64], tilings[sets]) numpy arrays in
    place of the per-problem lists."""
    arr, keep = _instances(problems)
    n = len(problems)
    res = (Result * max(n, 1))()
    flags = (D4E_BATCH_SEQUENTIAL if sequential else 0) | (D4E_BATCH_WIDE_KEYS if wide_keys else 0)
    o = BatchOpts(MODE_SETS, flags, device, 0, memory_budget, max_states, 0)
    offs = np.zeros(n + 1, dtype=np.uint64)
    st = Stats()
    while True:
        copies = np.empty((max(max_sets, 1), SET_PIECES), dtype=np.uint8)
        til = np.empty(max(max_sets, 1), dtype=np.uint64)
        rc = _lib.d4e_batch_sets(arr, n, C.byref(o), res, offs.ctypes.data_as(_u64p),
                                 copies.ctypes.data_as(_u8p), til.ctypes.data_as(_u64p),
                                 max_sets, C.byref(st))
        if rc == D4E_ERR_INVALID and int(offs[n]) > max_sets:
            max_sets = int(offs[n])
            continue
        _check(rc)
        break
    if arrays:
        total = int(offs[n])
        out = (offs, copies[:total], til[:total])
        return out, [res[i].as_dict() for i in range(n)], st.as_dict()
    out = []
    for i, p in enumerate(problems):
        a, b = int(offs[i]), int(offs[i + 1])
        rows = map(tuple, copies[a:b, : len(p.shapes)].tolist())
        out.append(list(zip(rows, til[a:b].tolist())))
    return out, [res[i].as_dict() for i in range(n)], st.as_dict()


MODE_LIST = 3
GRID_CELLS = 512


def batch_solutions(problems, max_per_instance: int = 1 << 16, device: int = 0,
                    memory_budget: int = 0, max_states: int = 0, sequential: bool = False,
                    wide_keys: bool = False, max_total: int = 1 << 16):
    """Every tiling of every problem (d4e_batch_solutions): for each problem
    a pair of arrays (type grids, step grids), each [tilings, height, width]
    (piece type / placement number per cell, -1 = not covered), at most
    max_per_instance tilings per problem; plus the results (count = all
    tilings) and stats.  Runs once more with room for the number needed when
    the batch lists more than max_total tilings."""
    arr, keep = _instances(problems)
    n = len(problems)
    res = (Result * max(n, 1))()
    flags = (D4E_BATCH_SEQUENTIAL if sequential else 0) | (D4E_BATCH_WIDE_KEYS if wide_keys else 0)
    o = BatchOpts(MODE_LIST, flags, device, 0, memory_budget, max_states, 0)
    offs = np.zeros(n + 1, dtype=np.uint64)
    st = Stats()
    while True:
        tg = np.empty((max(max_total, 1), GRID_CELLS), dtype=np.int8)
        sg = np.empty((max(max_total, 1), GRID_CELLS), dtype=np.int16)
        rc = _lib.d4e_batch_solutions(arr, n, C.byref(o), max_per_instance, res,
                                      offs.ctypes.data_as(_u64p), tg.ctypes.data_as(_i8p),
                                      sg.ctypes.data_as(_i16p), max_total, C.byref(st))
        if rc == D4E_ERR_INVALID and int(offs[n]) > max_total:
            max_total = int(offs[n])
            continue
        _check(rc)
        break
    out = []
    for i, p in enumerate(problems):
        a, b = int(offs[i]), int(offs[i + 1])
        cells = p.width * p.height
        out.append((tg[a:b, :cells].reshape(b - a, p.height, p.width).copy(),
                    sg[a:b, :cells].reshape(b - a, p.height, p.width).copy()))
    return out, [res[i].as_dict() for i in range(n)], st.as_dict()


def autotune_clear() -> None:
    """Forgets the launch plans measured so far in this process."""
    _lib.d4e_autotune_clear()


def release_cached_memory() -> None:
    """Returns the device memory kept for the next engine to the driver."""
    _lib.d4e_release_cached_memory()


class Server:
    """Continuous-batching request server (d4e_server_*)."""

    def __init__(self, device: int = 0, memory_budget: int = 0, max_states: int = 0,
                 beam: int = 0, max_active: int = 0):
        o = ServerOpts(device, max_active, memory_budget, max_states, beam)
        h = C.c_void_p()
        _check(_lib.d4e_server_create(C.byref(o), C.byref(h)))
        self._h = h
        self._shape = {}

    def submit(self, problem, mode: int, tag: int) -> None:
        arr, keep = _instances([problem])
        self._shape[tag] = (problem.width, problem.height)
        _check(_lib.d4e_server_submit(self._h, arr, mode, tag))

    def poll(self, max_results: int = 256):
        out = (Result * max_results)()
        n = C.c_uint32()
        _check(_lib.d4e_server_poll(self._h, out, max_results, C.byref(n)))
        res = []
        for i in range(n.value):
            w, h = self._shape.pop(out[i].tag, (0, 0))
            res.append(out[i].as_dict(w, h))
        return res

    def drain(self, timeout_s: float = 600.0) -> None:
        _check(_lib.d4e_server_drain(self._h, timeout_s))

    def stats(self) -> dict:
        st = ServerStats()
        _check(_lib.d4e_server_stats_get(self._h, C.byref(st)))
        return st.as_dict()

    def close(self) -> None:
        if self._h:
            _lib.d4e_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def count(problem, device: int = 0) -> int:
    """Tilings of one problem through the plain searcher path."""
    f = Frow(problem.shapes, problem.counts, problem.sym, problem.width, device)
    s = CudaSearcher(f, rows=problem.rows)
    s.run()
    return s.count()


def count_noalloc(problem, stream=None):
    """(tilings, summed frontier sizes) through d4e_count_noalloc, the entry
    point that allocates no device memory (current device)."""
    arr, keep = _instances([problem])
    cnt = C.c_uint64()
    states = C.c_uint64()
    _check(_lib.d4e_count_noalloc(arr, stream, C.byref(cnt), C.byref(states)))
    return cnt.value, states.value


def canonical_grid(problem, grid) -> np.ndarray:
    g = np.ascontiguousarray(np.asarray(grid, dtype=np.int8).reshape(-1))
    out = np.empty_like(g)
    rows = _arr(C.c_uint8, problem.rows)
    _check(_lib.d4e_canonical_grid(problem.width, problem.height, rows,
                                   g.ctypes.data_as(_i8p), out.ctypes.data_as(_i8p)))
    return out.reshape(problem.height, problem.width)
