#!/usr/bin/env python3
"""Benchmark of the row-by-row tiling engine on one GB300 (replicas on N GPUs).

Workload (one "step"): the exact enumeration of the single large puzzle --
an 8 x 15 board with 3 seeded holes tiled by 24 piece copies of 4..6 cells
(synthetic, seeded; see d4gb.problem.single_large) -- through the engine's C
ABI: placement tables, root state, every board row expanded and
de-duplicated on the device, the tiling count read back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` = frontier states per second (distinct states
summed over the 15 rows / CUDA-event time of the enumeration on the engine's
stream); `e2e` = the same through the C ABI with host buffers, wall clock
including table upload and result read-back.  `--impl reference` times the
CPU restatement of the reference's search path (oracle/, all host threads)
on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "d4-pieces_gb300"))
sys.path.insert(0, str(REPO))

# Seed of the single large puzzle: its peak frontier is 186,425,282 states
# (within the required 1e8..1e9; seeds 0..4 scanned on a GB300: seed 2 peaks
# at 514M, seed 4 above 1e9) and it has 437,783,699,473,187 tilings.
SINGLE_LARGE_SEED = 3
L2_FLUSH_BYTES = 512 << 20
# Rows the CPU baselines time on the single large puzzle: rows 0..3 in full
# (42.5M distinct states; some seconds on a 16-core host).  The GPU's states/s
# over the same rows is reported beside them, so the two compare like for like.
SAME_ROWS = 4
ALG_RECORD_BYTES = 24   # per-state record of the roofline's algorithmic bytes
# Batched mix and serving sections of the default run (the other configs of
# the headline metric: batched vs plain puzzles/s, served vs plain p50/p99).
MIX_INSTANCES = 8192
# Per-instance limit on one row's distinct states in the mix sections: the
# whole mix without a limit takes about 12 minutes of GPU time batched (its
# largest instances have rows of 10^8-10^9 states; 95 do not fit the
# device), so the default run counts every instance whose rows stay within
# 2^22 states and reports the rest (same set in both arms) as over the
# limit, by board size.
MIX_MAX_STATES = 1 << 22
SERVE_SECONDS = 2.0           # 2000 req/s arrival window (4000 requests)
SERVE_MID_SECONDS = 10.0      # 60 req/s arrival window (600 requests)
SERVE_LIGHT_RATE = 8.0        # a rate the plain path keeps up with (~0.5 of its capacity)
SERVE_LIGHT_SECONDS = 20.0    # ... for 20 s (160 requests)
SERVE_GRACE = 15.0            # seconds after the window before unfinished requests are cut


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--seed", type=int, default=SINGLE_LARGE_SEED)
    ap.add_argument("--workload", choices=("single_large", "medium", "batched", "batched_one",
                                           "serve", "family", "list"),
                    default="single_large",
                    help="medium = 8x10 board, 78 cells, 16 pieces (profiling case: frontier "
                         "of ~18M states, a few hundred MB -- larger than L2, a few GB at most)")
    ap.add_argument("--instances", type=int, default=1024,
                    help="batched workload: number of mix instances (seeded)")
    ap.add_argument("--max-states", type=int, default=20_000_000,
                    help="batched workloads: per-instance limit on one row's frontier")
    ap.add_argument("--beam", type=int, default=1024,
                    help="batched solve-one: first sampled-frontier width")
    ap.add_argument("--rate", type=float, default=2000.0, help="serve: arrivals per second")
    ap.add_argument("--duration", type=float, default=60.0, help="serve: seconds of arrivals")
    ap.add_argument("--serve-grace", type=float, default=15.0,
                    help="serve: seconds after the window to wait for results")
    ap.add_argument("--cpu-budget", type=float, default=15.0,
                    help="seconds of host CPU work for the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mix-instances", type=int, default=MIX_INSTANCES,
                    help="default run: instances of the batched mix (counting and solve-one)")
    ap.add_argument("--mix-max-states", type=int, default=MIX_MAX_STATES,
                    help="default run: per-instance row limit in the batched mix sections")
    ap.add_argument("--serve-seconds", type=float, default=SERVE_SECONDS,
                    help="default run: arrival window of the 2000 req/s serving section")
    ap.add_argument("--serve-mid-seconds", type=float, default=SERVE_MID_SECONDS,
                    help="default run: arrival window of the 60 req/s serving section")
    ap.add_argument("--serve-light-seconds", type=float, default=SERVE_LIGHT_SECONDS,
                    help="default run: arrival window of the light-load serving section")
    ap.add_argument("--no-mix", action="store_true",
                    help="default run: skip the batched mix and serving sections")
    ap.add_argument("--autotune", action="store_true",
                    help="measure launch plans in the first warm-up step (D4E_AUTOTUNE); "
                         "the default plan is the one the tuner keeps on this workload")
    ap.add_argument("--no-autotune", action="store_true", help=argparse.SUPPRESS)
    return ap.parse_args()


# ---------------------------------------------------------------------------
# distributed plumbing (replicas: every rank runs the same puzzle on its GPU)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self, n_gpus: int):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------------------
# measurement helpers
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed
    region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def flush_l2(dev: int):
    """Writes a buffer larger than L2 (129 MB) between timed steps."""
    try:
        import torch

        buf = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{dev}")
        buf.fill_(1)
        torch.cuda.synchronize(dev)
        del buf
        return True
    except Exception:
        return False


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profiled_traffic() -> dict | None:
    """DRAM bytes per raw child of k_expand from a one-launch ncu capture of
    the medium case (profiles/k_expand_medium_dram.json), when committed:
    every child is an insert into a random slot of a table far larger than
    L2, so the traffic of a launch grows with its raw children."""
    p = REPO / "profiles" / "k_expand_medium_dram.json"
    if p.exists():
        return json.loads(p.read_text())
    return None


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_once(E, prob, device: int, autotune: bool = False) -> dict:
    t0 = time.perf_counter()
    f = E.Frow(prob.shapes, prob.counts, prob.sym, prob.width, device=device)
    s = E.CudaSearcher(f, rows=prob.rows, autotune=autotune)
    s.run()
    count = s.count()
    wall = time.perf_counter() - t0
    st = s.stats()
    levels = s.level_sizes()
    del s, f
    return {"wall_s": wall, "count": count, "stats": st, "levels": levels}


def cpu_model() -> str:
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            k, _, v = ln.partition(":")
            if k.strip() in ("model name", "Model", "CPU part"):
                return v.strip()
    except OSError:
        pass
    import platform

    return platform.processor() or platform.machine()


def cpu_same_rows(prob) -> dict:
    """The oracle's exact row DP (restating the reference's level search) on
    rows 0..SAME_ROWS-1 of the puzzle, in full, on every host core."""
    from oracle import pyoracle

    pyoracle.build()
    threads = os.cpu_count() or 1
    r = pyoracle.rowdp_lean(prob, threads=threads, max_rows=SAME_ROWS)
    states = sum(r["level_sizes"])
    return {"value": states / r["seconds"], "unit": "states/s", "cores": threads,
            "kind": "port", "cpu": cpu_model(), "rows": f"0-{SAME_ROWS - 1}",
            "states": states, "seconds": r["seconds"], "level_sizes": r["level_sizes"],
            "sample": (f"exact row DP (oracle/, restating the reference's level search "
                       f"src/searcher_cuda.cu:32-82 with whole-row fills) on rows "
                       f"0-{SAME_ROWS - 1} of {prob.height} of the same puzzle, in full: "
                       f"{states} distinct states in {r['seconds']:.1f} s on {threads} threads")}


def cpu_backtracker(E, threads: int | None = None) -> dict:
    """The reference's own CPU algorithm -- the backtracking solve_count
    (src/Piece.cpp:104-139), as the oracle restates it -- on the pentomino
    ring (the 8x8 board minus its centre 2x2, 12 pentominoes, 520 tilings):
    one puzzle per host thread, all threads at once (the solver is
    single-threaded; the reference runs its puzzles in parallel)."""
    from d4gb.problem import pentomino_ring
    from oracle import pyoracle

    pyoracle.build()
    threads = threads or os.cpu_count() or 1
    ring = pentomino_ring(E.catalogue(5))
    counts = [None] * threads

    def work(i):
        counts[i] = pyoracle.solve_count(ring)

    t0 = time.perf_counter()
    ths = [threading.Thread(target=work, args=(i,)) for i in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    el = time.perf_counter() - t0
    if any(c != 520 for c in counts):
        raise RuntimeError(f"backtracker counts {set(counts)} != 520")
    return {"value": threads / el, "unit": "puzzles/s", "cores": threads, "kind": "port",
            "cpu": cpu_model(), "seconds": el,
            "sample": (f"{threads} pentomino-ring puzzles (520 tilings each) counted by the "
                       f"backtracker restatement, one per host thread, in {el:.1f} s")}


def gpu_same_rows(E, prob, device: int, reps: int = 3) -> dict:
    """The engine on rows 0..SAME_ROWS-1 of the puzzle (one search_GPU per
    row, each synchronised), fastest of `reps`."""
    best = None
    for _ in range(reps):
        f = E.Frow(prob.shapes, prob.counts, prob.sym, prob.width, device=device)
        s = E.CudaSearcher(f, rows=prob.rows)
        t0 = time.perf_counter()
        for _ in range(SAME_ROWS):
            s.search_GPU()
        el = time.perf_counter() - t0
        states = sum(s.level_sizes()[:SAME_ROWS])
        del s, f
        best = el if best is None else min(best, el)
    return {"value": states / best, "unit": "states/s", "rows": f"0-{SAME_ROWS - 1}",
            "states": states, "seconds": best}


def gpu_ring(E, device: int, reps: int = 5) -> dict:
    """The plain single-puzzle path on the pentomino ring, fastest of reps."""
    from d4gb.problem import pentomino_ring

    ring = pentomino_ring(E.catalogue(5))
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        f = E.Frow(ring.shapes, ring.counts, ring.sym, ring.width, device=device)
        s = E.CudaSearcher(f, rows=ring.rows)
        s.run()
        n = s.count()
        el = time.perf_counter() - t0
        del s, f
        if n != 520:
            raise RuntimeError(f"ring count {n} != 520")
        best = el if best is None else min(best, el)
    return {"value": 1.0 / best, "unit": "puzzles/s", "seconds": best}


def make_problem(args):
    from d4gb.problem import medium_board, single_large

    if args.workload == "medium":
        return medium_board(77), "medium enumeration: 8x10 board, 2 holes, 16 piece copies of 4-6 cells, seed 77"
    return single_large(args.seed), (f"single large enumeration: 8x15 board, 3 holes, 24 piece "
                                      f"copies of 4-6 cells, seed {args.seed}")


def bench_ours(args, dist: Dist) -> None:
    from d4gb import engine as E

    dev = dist.local_rank
    prob, workload = make_problem(args)
    for _ in range(args.warmup):
        run_once(E, prob, dev, args.autotune and not args.no_autotune)
    flush_l2(dev)
    dist.barrier()
    sampler = ClockSampler(dev)
    sampler.start()
    runs = []
    t_start = time.perf_counter()
    for _ in range(args.steps):
        runs.append(run_once(E, prob, dev, args.autotune and not args.no_autotune))
        flush_l2(dev)
    t_wall = time.perf_counter() - t_start
    clocks = sampler.stop()
    dist.barrier()

    states = sum(r["stats"]["states_out"] for r in runs)
    run_s = sum(r["stats"]["run_ms"] for r in runs) / 1e3
    e2e_s = sum(r["wall_s"] for r in runs)
    max_run_s = dist.max(run_s)
    max_e2e_s = dist.max(e2e_s)
    all_states = dist.sum(states)
    counts = {r["count"] for r in runs}
    if len(counts) != 1:
        raise RuntimeError(f"non-deterministic tiling counts across steps: {counts}")

    st = [r["stats"] for r in runs]
    exp_ms = sum(s["expand_ms"] for s in st)
    exp_launches = sum(s["expand_launches"] for s in st)
    # Algorithmic bytes of the expansion: S = 24 B per state record (window
    # u64 + used u32 + instance u32 + count u64) x (parents read + raw
    # children written), the per-state figure the level search is costed
    # with; the packed records here are 16 B, so this counts 1.5x the bytes
    # they actually occupy.
    alg_bytes = sum(ALG_RECORD_BYTES * (s["states_in"] + s["states_raw"]) for s in st)
    peaks = measured_peaks()
    achieved = alg_bytes / (exp_ms / 1e3) / 1e9 if exp_ms > 0 else None
    traffic = profiled_traffic()
    traffic_per_launch = None
    if traffic and exp_launches:
        traffic_per_launch = (traffic["dram_bytes_per_raw_child"] *
                              sum(s["states_raw"] for s in st) / exp_launches)
    # Dedup output stage (k_compact): scans every table slot, writes each
    # distinct state once and clears its slot.
    cmp_ms = sum(s["compact_ms"] for s in st)
    cmp_bytes = sum(s["compact_slots"] * s["slot_bytes"] + s["states_out"] * s["record_bytes"]
                    + s["states_out"] * s["slot_bytes"] for s in st)
    cmp_achieved = cmp_bytes / (cmp_ms / 1e3) / 1e9 if cmp_ms > 0 else None
    launches = sum(s["expand_launches"] + s["compact_launches"] + s["other_launches"] for s in st)
    h2d = sum(s["h2d_bytes"] for s in st) / len(st)
    d2h = sum(s["d2h_bytes"] for s in st) / len(st)
    levels = runs[0]["levels"]

    if dist.rank != 0:
        return
    line = {
        "metric": "frontier states/s (exact enumeration, single large 8x15 puzzle)",
        "value": all_states / max_run_s,
        "unit": "states/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": max_run_s / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic (seeded generator d4gb.problem.single_large)",
        "puzzles_per_s": dist.world * args.steps / max_run_s,
        "count": counts.pop(),
        "config": {
            "workload": workload,
            "types": len(prob.shapes),
            "multiplicities": prob.counts,
            "peak_frontier": max(levels),
            "level_sizes": levels,
            "states_per_step": states // args.steps,
            "raw_children_per_step": sum(s["states_raw"] for s in st) // args.steps,
            "record_bytes": st[0]["record_bytes"],
            "launch_plan": {"autotuned": args.autotune and not args.no_autotune,
                            "chunk_cap": st[0]["tuned_chunk_cap"],
                            "chunks_per_warp": st[0]["tuned_chunks_per_warp"],
                            "ctas_per_sm": st[0]["tuned_ctas_per_sm"] or "occupancy",
                            "table_load": st[0]["tuned_load"],
                            "compact_ctas_per_sm": st[0]["tuned_compact_ctas"],
                            "compact_stages": st[0]["tuned_compact_stages"]},
            "slot_bytes": st[0]["slot_bytes"],
            "l2": "frontier and table far larger than L2 (GBs); plus a 512 MiB L2 flush between steps",
            "parallelism": f"replicas x{dist.world} (no sharding, no collectives)",
            "wall_s_timed_region": t_wall,
        },
        "e2e": {
            "value": all_states / max_e2e_s,
            "unit": "states/s",
            "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h),
        },
        "roofline": {
            "kernel": "k_expand (row-fill DFS + fused hash-table insert)",
            "bound": "hbm",
            "achieved": achieved,
            "peak": peaks["hbm_gbs"],
            "peak_source": peaks["source"],
            "unit": "GB/s",
            "frac": achieved / peaks["hbm_gbs"] if achieved else None,
            "traffic": traffic_per_launch,
            "algorithmic_bytes_per_launch": alg_bytes / exp_launches if exp_launches else None,
            "algorithmic_bytes": "24 B x (parent states read + raw children inserted) per launch",
            "traffic_source": ("ncu DRAM bytes per raw child of one medium-case launch "
                               "(profiles/k_expand_medium_dram.md) x raw children per launch"),
            "avg_launch_ms": exp_ms / exp_launches if exp_launches else None,
            "launches": exp_launches,
        },
        "dedup_roofline": {
            "kernel": "k_compact (table scan -> distinct states, slots cleared)",
            "bound": "hbm",
            "achieved": cmp_achieved,
            "peak": peaks["hbm_gbs"],
            "unit": "GB/s",
            "frac": cmp_achieved / peaks["hbm_gbs"] if cmp_achieved else None,
            "bytes": "table slots scanned x slot bytes + distinct states x (record + slot) bytes",
            "ms_per_step": cmp_ms / len(st),
        },
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline and dist.world == 1:
        # Like for like: the CPU restatement and the engine on the same whole
        # rows (0..SAME_ROWS-1), and the reference's backtracker against the
        # engine on the pentomino ring.
        cpu = cpu_same_rows(prob)
        gpu = gpu_same_rows(E, prob, dev)
        line["cpu_baseline"] = cpu
        line["same_rows"] = {"rows": cpu["rows"], "gpu_states_per_s": gpu["value"],
                             "cpu_states_per_s": cpu["value"],
                             "ratio": gpu["value"] / cpu["value"],
                             "full_run_ratio": line["value"] / cpu["value"]}
        bt = cpu_backtracker(E)
        ring = gpu_ring(E, dev)
        line["pentomino_ring"] = {"cpu_backtracker": bt, "gpu_plain_puzzles_per_s": ring["value"],
                                  "gpu_seconds": ring["seconds"],
                                  "ratio_vs_all_cores": ring["value"] / bt["value"]}
    if not args.no_mix and dist.world == 1:
        # The headline metric's other configurations: the batched mix
        # (counting, then solve-one) and serving, each against the plain
        # one-puzzle-at-a-time path.
        line["batched_count"] = mix_section(E, dev, args.mix_instances, E.MODE_COUNT,
                                            args.mix_max_states, MIX_BEAM)
        line["batched_solve_one"] = mix_section(E, dev, args.mix_instances, E.MODE_SOLVE_ONE,
                                                args.mix_max_states, MIX_BEAM)
        line["served"] = serve_section(E, dev, 2000.0, args.serve_seconds, args.mix_max_states,
                                       MIX_BEAM, SERVE_GRACE)
        line["served_60"] = serve_section(E, dev, 60.0, args.serve_mid_seconds,
                                          args.mix_max_states, MIX_BEAM, SERVE_GRACE)
        line["served_light"] = serve_section(E, dev, SERVE_LIGHT_RATE, args.serve_light_seconds,
                                             args.mix_max_states, MIX_BEAM, SERVE_GRACE)
        line["batched_list"] = list_section(E, dev, LIST_INSTANCES)
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# reference arm: the CPU restatement of the reference's search path
# ---------------------------------------------------------------------------
def bench_reference(args, dist: Dist) -> None:
    if dist.rank != 0:
        return
    from oracle import pyoracle

    pyoracle.build()
    prob, workload = make_problem(args)
    threads = os.cpu_count() or 1
    # A step = rows 0..SAME_ROWS-1 of the puzzle in full (the ours arm's line
    # reports the GPU's states/s over the same rows as same_rows).
    for _ in range(args.warmup):
        pyoracle.rowdp_lean(prob, threads=threads, max_rows=SAME_ROWS)
    states = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = pyoracle.rowdp_lean(prob, threads=threads, max_rows=SAME_ROWS)
        states += sum(r["level_sizes"])
    el = time.perf_counter() - t0
    v = states / el if el > 0 else None
    sample = (f"exact row DP (oracle/ restating the reference's level search, "
              f"src/searcher_cuda.cu + src/kernel.cuh, with whole-row fills) on the same "
              f"puzzle: per step rows 0-{SAME_ROWS - 1} of {prob.height} in full, "
              f"{threads} threads ({cpu_model()})")
    print(json.dumps({
        "impl": "reference",
        "metric": "frontier states/s (exact enumeration, single large 8x15 puzzle)",
        "value": v,
        "unit": "states/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic (seeded generator d4gb.problem.single_large)",
        "config": {"workload": workload, "parallelism": f"host threads x{threads}",
                   "rows": f"0-{SAME_ROWS - 1} of {prob.height} (the ours arm reports the "
                           f"GPU on the same rows as same_rows)"},
        "cpu_baseline": {"value": v, "unit": "states/s", "cores": threads, "kind": "port",
                         "cpu": cpu_model(), "sample": sample},
        "e2e": {"value": v, "unit": "states/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


# ---------------------------------------------------------------------------
# batched mix: all puzzles in one batch vs one puzzle at a time
# ---------------------------------------------------------------------------
BATCHED_SEED = 2024


def bench_batched(args, dist: Dist) -> None:
    """Batched mix: the same seeded instances once as one batch (one k_expand
    + k_compact pair per board row for all of them) and once through the
    plain path (one puzzle at a time).  Both runs apply the same per-instance
    frontier limit; the counts (or solve-one outcomes) must agree."""
    from d4gb import engine as E
    from d4gb.problem import batched_mix, verify_tiling

    probs = batched_mix(BATCHED_SEED, args.instances)
    mode = E.MODE_SOLVE_ONE if args.workload == "batched_one" else E.MODE_COUNT
    res = {}
    outs = {}
    for arm, seq in (("batched", False), ("plain", True)):
        t0 = time.perf_counter()
        out, st = E.batch_run(probs, mode=mode, sequential=seq, device=dist.local_rank,
                              max_states=args.max_states, beam=args.beam)
        wall = time.perf_counter() - t0
        ok = [r for r in out if r["status"] == 0]
        outs[arm] = out
        res[arm] = {"wall_s": wall, "puzzles_per_s": len(probs) / wall,
                    "states_per_s": st["states_out"] / wall,
                    "completed": len(ok), "over_limit": len(out) - len(ok),
                    "expand_launches": st["expand_launches"],
                    "compact_launches": st["compact_launches"],
                    "other_launches": st["other_launches"],
                    "states": st["states_out"], "expand_ms": st["expand_ms"],
                    "compact_ms": st["compact_ms"], "paused": st["paused"],
                    "restarts": st["restarts"]}
    for a, b in zip(outs["batched"], outs["plain"]):
        if (a["status"], a["count"]) != (b["status"], b["count"]):
            raise RuntimeError("batched and plain results differ")
    extra = {}
    if mode == E.MODE_SOLVE_ONE:
        bad = sum(1 for p, r in zip(probs, outs["batched"])
                  if r["found"] and not verify_tiling(p, r["grid"], r["steps"]))
        if bad:
            raise RuntimeError(f"{bad} solve-one tilings fail the cover check")
        extra["found"] = sum(1 for r in outs["batched"] if r["found"])
        extra["cover_checked"] = extra["found"]
    if dist.rank == 0:
        what = "solve-one" if mode == E.MODE_SOLVE_ONE else "solve-all counts"
        print(json.dumps({
            "metric": f"puzzles/s (batched mix, {what})",
            "value": res["batched"]["puzzles_per_s"],
            "unit": "puzzles/s",
            "n_gpus": dist.world,
            "config": {"workload": f"batched mix: {len(probs)} instances, seed {BATCHED_SEED}, "
                                   "width 5-8, height 5-12, 0-4 holes, 3-6-cell pieces",
                       "max_states_per_row": args.max_states, "beam": args.beam},
            "batched": res["batched"], "plain": res["plain"],
            "speedup_vs_plain": res["batched"]["puzzles_per_s"] / res["plain"]["puzzles_per_s"],
            **extra,
        }), flush=True)


LIST_MAX_CELLS = 40
LIST_PER_INSTANCE = 64
LIST_INSTANCES = 1024


def list_section(E, dev: int, n: int) -> dict:
    """Batched solution listing: the tilings of the batched mix's boards of
    at most LIST_MAX_CELLS cells (up to LIST_PER_INSTANCE per board), once
    as one batch (d4e_batch_solutions) and once one board at a time through
    the same call.  Counts must agree; boards with at most
    LIST_PER_INSTANCE tilings must list the same tilings in both arms; every
    listed tiling passes the independent cover check."""
    from d4gb.problem import batched_mix, verify_tiling

    probs = [p for p in batched_mix(BATCHED_SEED, 16 * n) if p.cells <= LIST_MAX_CELLS][:n]
    res, outs = {}, {}
    for arm, seq in (("batched", False), ("plain", True)):
        t0 = time.perf_counter()
        grids, out, st = E.batch_solutions(probs, max_per_instance=LIST_PER_INSTANCE,
                                           device=dev, sequential=seq)
        wall = time.perf_counter() - t0
        outs[arm] = (grids, out)
        listed = sum(len(g[0]) for g in grids)
        res[arm] = {"wall_s": wall, "puzzles_per_s": len(probs) / wall,
                    "tilings_listed": listed, "tilings_per_s": listed / wall,
                    "expand_launches": st["expand_launches"],
                    "other_launches": st["other_launches"], "states": st["states_out"]}
    (gb, ob), (gp, op) = outs["batched"], outs["plain"]
    for i, p in enumerate(probs):
        if (ob[i]["status"], ob[i]["count"]) != (op[i]["status"], op[i]["count"]):
            raise RuntimeError(f"board {i}: batched and plain counts differ")
        if ob[i]["count"] <= LIST_PER_INSTANCE:
            a = {(t.tobytes(), s_.tobytes()) for t, s_ in zip(*gb[i])}
            b = {(t.tobytes(), s_.tobytes()) for t, s_ in zip(*gp[i])}
            if a != b:
                raise RuntimeError(f"board {i}: batched and plain tilings differ")
        for t, s_ in zip(*gb[i]):
            if not verify_tiling(p, t, s_):
                raise RuntimeError(f"board {i}: a listed tiling fails the cover check")
    return {"workload": f"batched mix boards of at most {LIST_MAX_CELLS} cells: "
                        f"{len(probs)} boards, seed {BATCHED_SEED}, up to "
                        f"{LIST_PER_INSTANCE} tilings listed per board",
            "boards_with_tilings": sum(1 for r in ob if r["count"]),
            "tilings_total": sum(r["count"] for r in ob),
            "batched": res["batched"], "plain": res["plain"],
            "speedup_vs_plain": res["batched"]["puzzles_per_s"] / res["plain"]["puzzles_per_s"],
            "cover_checked": res["batched"]["tilings_listed"]}


def bench_list(args, dist: Dist) -> None:
    """The batched listing section alone (--instances boards)."""
    from d4gb import engine as E

    sec = list_section(E, dist.local_rank, args.instances)
    if dist.rank == 0:
        print(json.dumps({
            "metric": "puzzles/s (batched solution listing)",
            "value": sec["batched"]["puzzles_per_s"],
            "unit": "puzzles/s",
            "n_gpus": dist.world,
            "config": {"workload": sec.pop("workload")},
            **sec,
        }), flush=True)


FAMILY_TEXT = "aaaaaaaa\naaaaaaaa\naaabaaaa\naaaacaaa\naaaaaaaa\n"
FAMILY_MAX_STATES = 1 << 30


def family_cpu_baseline(fam, shapes, budget: float) -> tuple[dict, dict]:
    """The oracle's exact row DP (count mode: the states of the piece-set run,
    which also reads its final row back) over the family's boards in order
    until the time budget is spent; returns the baseline and the counts."""
    from d4gb import family as F
    from oracle import pyoracle

    pyoracle.build()
    threads = os.cpu_count() or 1
    boards = sorted(set(fam.configs()))
    counts, states = {}, 0
    t0 = time.perf_counter()
    for m in boards:
        p = F.board_problem(m, shapes, [1] * len(shapes))
        r = pyoracle.rowdp(p, threads=threads)
        counts[m] = r["count"]
        states += r["states_total"]
        if time.perf_counter() - t0 > budget:
            break
    el = time.perf_counter() - t0
    return ({"value": len(counts) / el, "unit": "configurations/s", "cores": threads,
             "kind": "port", "states_per_s": states / el,
             "sample": (f"exact row DP (oracle/, count mode) on the first {len(counts)} of "
                        f"{len(boards)} boards in {el:.1f} s on {threads} threads")}, counts)


def bench_family(args, dist: Dist) -> None:
    """Board family (the reference's Board<8> + AtomicCount research run):
    8x5 with two fixed holes (regions b, c) and one roaming hole (region a:
    38 configurations of 37 cells); pieces are the free trominoes,
    tetrominoes and pentominoes, each at most once (19 types).  Every
    configuration is one instance of a piece-set batch; the result is the
    ledger of Naming ranks (18,260 ranked combinations).  Plain = the same
    configurations one at a time."""
    from d4gb import engine as E
    from d4gb import family as F
    from d4gb.problem import pentomino_ring

    fam = F.BoardFamily.from_text(FAMILY_TEXT)
    E.batch_run([pentomino_ring(E.catalogue(5))], device=dist.local_rank)  # context warm-up
    # Untimed runs: the first maps the device memory the engine pool keeps
    # for the following calls (a research run makes many such calls).
    for _ in range(max(args.warmup, 1)):
        F.family_ledger(fam, 3, 5, 0, 64, device=dist.local_rank, max_states=FAMILY_MAX_STATES)
    res, runs = {}, {}
    for arm, seq in (("batched", False), ("plain", True)):
        t0 = time.perf_counter()
        run = F.family_ledger(fam, 3, 5, 0, 64, device=dist.local_rank,
                              max_states=FAMILY_MAX_STATES, sequential=seq)
        wall = time.perf_counter() - t0
        runs[arm] = run
        st = run.stats
        res[arm] = {"wall_s": wall, "configs_per_s": fam.count / wall,
                    "states_per_s": st["states_out"] / wall, "states": st["states_out"],
                    "expand_launches": st["expand_launches"],
                    "expand_ms": st["expand_ms"], "compact_ms": st["compact_ms"],
                    "run_ms": st["run_ms"], "step_wall_ms": st["step_wall_ms"],
                    "upload_ms": st["upload_ms"], "phase_ms": st["phase_ms"],
                    "retries": st["retries"], "peak_frontier": st["peak_frontier"],
                    "record_bytes": st["record_bytes"]}
    if runs["batched"].ledger != runs["plain"].ledger:
        raise RuntimeError("batched and plain ledgers differ")
    run = runs["batched"]
    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        cpu, counts = family_cpu_baseline(fam, run.shapes, args.cpu_budget)
        fs = run.sets
        for i, m in enumerate(fs.masks):
            if m in counts:
                got = int(fs.tilings[int(fs.offsets[i]):int(fs.offsets[i + 1])].sum())
                if got != counts[m]:
                    raise RuntimeError(f"board {m:#x}: sets sum to {got} tilings, "
                                       f"the oracle counts {counts[m]}")
        cpu["checked_boards"] = len(counts)
    if dist.rank == 0:
        print(json.dumps({
            "metric": "configurations/s (board family, piece-set ledger)",
            "value": res["batched"]["configs_per_s"],
            "unit": "configurations/s",
            "n_gpus": dist.world,
            "config": {"workload": "board family 8x5, 2 fixed + 1 roaming hole (38 "
                                   "configurations of 37 cells), free 3-5-cell pieces at most "
                                   "once each (19 types), Naming ranks over 3-5 cells",
                       "naming_size": run.naming.size(),
                       "max_states_per_row": FAMILY_MAX_STATES},
            "batched": res["batched"], "plain": res["plain"],
            "speedup_vs_plain": res["batched"]["configs_per_s"] / res["plain"]["configs_per_s"],
            "ledger_entries": len(run.ledger),
            "tiled_configs": len(run.sets.masks) - len(set(run.unsolved(fam))),
            "sets": int(run.sets.offsets[-1]),
            "tilings": int(run.sets.tilings.sum()),
            "cpu_baseline": cpu,
        }), flush=True)


SERVE_SEED = 4242


def _percentile(v, q):
    if not v:
        return None
    s = sorted(v)
    return s[min(len(s) - 1, int(round(q * (len(s) - 1))))]


def bench_serve(args, dist: Dist) -> None:
    """Serving alone (--rate req/s for --duration s): the server and the
    plain per-request path under the same Poisson arrivals."""
    from d4gb import engine as E

    sec = serve_section(E, dist.local_rank, args.rate, args.duration, args.max_states,
                        args.beam, args.serve_grace)
    if dist.rank == 0:
        print(json.dumps({
            "metric": "served puzzles/s (Poisson arrivals, 70% solve-one / 30% solve-all)",
            "value": sec["served"]["puzzles_per_s"],
            "unit": "puzzles/s",
            "n_gpus": dist.world,
            "config": {"workload": f"serving: Poisson {args.rate:g} req/s for {args.duration:g} s, "
                                   f"batched-mix distribution, seed {SERVE_SEED}",
                       "max_states_per_row": args.max_states, "beam": args.beam},
            **sec,
        }), flush=True)


# ---------------------------------------------------------------------------
# batched mix and serving sections of the default run
# ---------------------------------------------------------------------------
MIX_BEAM = 1024


def _service_times(out) -> list[float]:
    """Per-instance service times (ms) of a sequential batch_run: its
    latencies are cumulative from the batch start, in instance order."""
    prev, svc = 0.0, []
    for r in out:
        svc.append(r["latency_ms"] - prev)
        prev = r["latency_ms"]
    return svc


def mix_section(E, dev: int, n: int, mode: int, max_states: int, beam: int) -> dict:
    """Config 3 (counting) or config 4 (solve-one): the batched mix run as one
    batch and one puzzle at a time (the plain path: the same engine, one
    launch sequence per puzzle), results compared instance by instance.
    Amdahl split: the 10 % of instances with the longest plain service time,
    and the rest, each also run as a batch of its own."""
    from d4gb.problem import batched_mix, verify_tiling

    probs = batched_mix(BATCHED_SEED, n)
    arms, outs = {}, {}
    for arm, seq in (("batched", False), ("plain", True)):
        t0 = time.perf_counter()
        out, st = E.batch_run(probs, mode=mode, sequential=seq, device=dev,
                              max_states=max_states, beam=beam)
        wall = time.perf_counter() - t0
        outs[arm] = out
        arms[arm] = {"wall_s": wall, "puzzles_per_s": n / wall,
                     "states_per_s": st["states_out"] / wall, "states": st["states_out"],
                     "completed": sum(1 for r in out if r["status"] == 0),
                     "expand_launches": st["expand_launches"],
                     "compact_launches": st["compact_launches"],
                     "expand_ms": st["expand_ms"], "compact_ms": st["compact_ms"],
                     "peak_frontier": st["peak_frontier"]}
    for a, b in zip(outs["batched"], outs["plain"]):
        if (a["status"], a["count"], a["found"]) != (b["status"], b["count"], b["found"]):
            raise RuntimeError("batched and plain results differ")
    failed = [i for i, r in enumerate(outs["batched"]) if r["status"] != 0]
    by_size: dict[str, int] = {}
    for i in failed:
        k = f"{probs[i].width}x{probs[i].height}"
        by_size[k] = by_size.get(k, 0) + 1
    sec = {"instances": n, "seed": BATCHED_SEED, "max_states_per_row": max_states,
           "failed_by_board_size": dict(sorted(by_size.items(), key=lambda kv: -kv[1])),
           "batched": arms["batched"], "plain": arms["plain"],
           "speedup_vs_plain": arms["batched"]["puzzles_per_s"] / arms["plain"]["puzzles_per_s"],
           "failed": len(failed),
           "failed_status": sorted({outs["batched"][i]["status"] for i in failed})}
    if mode == E.MODE_SOLVE_ONE:
        found = [i for i, r in enumerate(outs["batched"]) if r["found"]]
        bad = sum(1 for i in found
                  if not verify_tiling(probs[i], outs["batched"][i]["grid"],
                                       outs["batched"][i]["steps"]))
        if bad:
            raise RuntimeError(f"{bad} solve-one tilings fail the cover check")
        sec["found"] = len(found)
        sec["cover_checked"] = len(found)
        sec["beam"] = beam
    else:
        sec["tilings"] = sum(r["count"] for r in outs["batched"] if r["status"] == 0)
    # Amdahl split on the plain service times.
    svc = _service_times(outs["plain"])
    order = sorted(range(n), key=lambda i: -svc[i])
    top = sorted(order[: max(1, n // 10)])
    rest = sorted(order[max(1, n // 10):])
    split = {"plain_ms_top10pct": sum(svc[i] for i in top),
             "plain_ms_rest": sum(svc[i] for i in rest)}
    for name, idx in (("top10pct", top), ("rest", rest)):
        t0 = time.perf_counter()
        E.batch_run([probs[i] for i in idx], mode=mode, device=dev, max_states=max_states,
                    beam=beam)
        split[f"batched_ms_{name}"] = (time.perf_counter() - t0) * 1e3
    split["speedup_top10pct"] = split["plain_ms_top10pct"] / split["batched_ms_top10pct"]
    split["speedup_rest"] = split["plain_ms_rest"] / split["batched_ms_rest"]
    split["plain_share_top10pct"] = split["plain_ms_top10pct"] / sum(svc)
    sec["amdahl"] = split
    return sec


def _arrivals(rate: float, seconds: float, seed: int):
    import random

    from d4gb import engine as E
    from d4gb.problem import batched_instance

    rng = random.Random(seed)
    n = int(rate * seconds)
    t, arr = 0.0, []
    for _ in range(n):
        t += rng.expovariate(rate)
        arr.append(t)
    probs = [batched_instance(rng, i) for i in range(n)]
    modes = [E.MODE_SOLVE_ONE if rng.random() < 0.7 else E.MODE_COUNT for _ in range(n)]
    return arr, probs, modes


def _latency_summary(lat_done: list[float], cut: list[float]) -> dict:
    """p50/p99 over every request: the unfinished ones count with the time
    they had waited when the run was cut (a lower bound of their latency)."""
    allv = lat_done + cut
    return {"p50": _percentile(allv, 0.5), "p99": _percentile(allv, 0.99),
            "p50_completed": _percentile(lat_done, 0.5),
            "p99_completed": _percentile(lat_done, 0.99)}


def serve_served(E, dev, arr, probs, modes, max_states, beam, grace: float) -> dict:
    """The continuous-batching server under the arrival stream (open loop)."""
    from d4gb.problem import verify_tiling

    n = len(arr)
    srv = E.Server(device=dev, max_states=max_states, beam=beam)
    results = {}
    t0 = time.perf_counter()
    for i, (p, m, ta) in enumerate(zip(probs, modes, arr)):
        while True:
            now = time.perf_counter() - t0
            if now >= ta:
                break
            for r in srv.poll():
                results[r["tag"]] = r
            time.sleep(min(ta - now, 0.0005))
        srv.submit(p, m, i)
    deadline = t0 + arr[-1] + grace
    while len(results) < n and time.perf_counter() < deadline:
        for r in srv.poll():
            results[r["tag"]] = r
        time.sleep(0.001)
    elapsed = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    done = [r for r in results.values() if r["status"] == 0]
    bad = sum(1 for r in done if r["found"] and
              not verify_tiling(probs[r["tag"]], r["grid"], r["steps"]))
    if bad:
        raise RuntimeError(f"{bad} served solve-one tilings fail the cover check")
    cut = [(elapsed - arr[i]) * 1e3 for i in range(n) if i not in results]
    return {"completed": len(done), "failed": sum(1 for r in results.values() if r["status"]),
            "unfinished": n - len(results), "elapsed_s": elapsed,
            "puzzles_per_s": len(done) / elapsed,
            "latency_ms": _latency_summary([r["latency_ms"] for r in done], cut),
            "cover_checked": sum(1 for r in done if r["found"]),
            "moved_to_slow_lane": st["moved"], "peak_active": st["peak_active"],
            "lanes": {k: st[k] for k in ("lane_steps", "lane_busy_ms", "lane_kernel_ms",
                                         "lane_inst_rows", "lane_admit_ms", "lane_collect_ms")},
            "results": {r["tag"]: (r["status"], r["count"], r["found"]) for r in results.values()}}


def serve_plain(E, dev, arr, probs, modes, max_states, beam, grace: float) -> dict:
    """The plain per-request path under the same arrivals, measured: one
    request at a time in arrival order (FIFO), each through the engine alone
    (d4e_batch_run with one instance)."""
    n = len(arr)
    lat, results, svc = [], {}, []
    t0 = time.perf_counter()
    deadline = t0 + arr[-1] + grace
    for i in range(n):
        now = time.perf_counter() - t0
        if now < arr[i]:
            time.sleep(arr[i] - now)
        if time.perf_counter() > deadline:
            break
        start = time.perf_counter()
        out, _ = E.batch_run([probs[i]], mode=modes[i], sequential=True, device=dev,
                             max_states=max_states, beam=beam)
        done = time.perf_counter() - t0
        svc.append((time.perf_counter() - start) * 1e3)
        r = out[0]
        results[i] = (r["status"], r["count"], r["found"])
        if r["status"] == 0:
            lat.append((done - arr[i]) * 1e3)
    elapsed = time.perf_counter() - t0
    cut = [(elapsed - arr[i]) * 1e3 for i in range(n) if i not in results]
    return {"completed": len(lat), "unfinished": n - len(results), "elapsed_s": elapsed,
            "puzzles_per_s": len(lat) / elapsed,
            "latency_ms": _latency_summary(lat, cut),
            "mean_service_ms": sum(svc) / len(svc) if svc else None,
            "results": results}


def serve_section(E, dev: int, rate: float, seconds: float, max_states: int, beam: int,
                  grace: float) -> dict:
    """Config 5 (shortened): Poisson arrivals at `rate` for `seconds`, 70 %
    solve-one / 30 % counting from the batched-mix distribution, through the
    server and through the plain per-request path under the same arrivals;
    every result of both arms compared."""
    arr, probs, modes = _arrivals(rate, seconds, SERVE_SEED)
    served = serve_served(E, dev, arr, probs, modes, max_states, beam, grace)
    plain = serve_plain(E, dev, arr, probs, modes, max_states, beam, grace)
    rs, rp = served.pop("results"), plain.pop("results")
    for i in set(rs) & set(rp):
        if rs[i][0] == 0 and rp[i][0] == 0 and rs[i] != rp[i]:
            raise RuntimeError(f"request {i}: served and plain results differ")
    # Error statuses per arm, and the requests that failed in one arm only.
    for arm, res, other in (("served", rs, rp), ("plain", rp, rs)):
        hist = {}
        for r in res.values():
            if r[0]:
                hist[str(r[0])] = hist.get(str(r[0]), 0) + 1
        arm_d = served if arm == "served" else plain
        arm_d["failed_status"] = hist
        arm_d["failed_here_only"] = sum(1 for i in set(res) & set(other)
                                        if res[i][0] and not other[i][0])
    load = (rate * plain["mean_service_ms"] / 1e3) if plain["mean_service_ms"] else None
    return {"rate_req_s": rate, "arrival_window_s": seconds, "requests": len(arr),
            "grace_s": grace, "offered_load_vs_plain_capacity": load,
            "served": served, "plain": plain,
            "speedup_vs_plain": served["puzzles_per_s"] / plain["puzzles_per_s"]
            if plain["puzzles_per_s"] else None}


def main() -> None:
    args = parse_args()
    dist = Dist(args.gpus)
    try:
        if args.impl == "reference":
            bench_reference(args, dist)
        elif args.workload in ("batched", "batched_one"):
            bench_batched(args, dist)
        elif args.workload == "serve":
            bench_serve(args, dist)
        elif args.workload == "family":
            bench_family(args, dist)
        elif args.workload == "list":
            bench_list(args, dist)
        else:
            bench_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
