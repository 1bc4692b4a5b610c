#!/usr/bin/env python3
"""Benchmark: bit-exact range-sum answers/s on GB300, batched vs plain, every config.

Default (``--workload batched_trees``): 4,096 independent version trees of uneven
size (lognormal state counts, median 2,000, about 27.5M states, 220M events, 4.1M
queries; biworlddb-artifact_gb300/workloads.py).  One step = one replay of the whole
batch as a single autotuned pipeline replayed from a CUDA graph.  Every batched
answer is checked against the oracle (all trees).  The same line reports the plain
form (4,096 sequential bw_replay_launch calls) and, as sub-records with their own
roofline, e2e and CPU baseline:

* ``plain_chain``: the plain chain replay (20,000 states, 1M events, 10k queries,
  4,096 keys) and ``plain_chain_x100`` (the same generator at 100x: 2M states,
  100M events, 1M queries), both on the single-pass chain path;
* ``trip_tree``: the trip-log-shaped tree (300k states, 40M events, 50M queries,
  65,536 keys) on the general pipeline;
* ``csr_lut``: the sparse-key CSR rank-LUT (10M u64 keys, 100M point and range
  lookups, LUT budgets 64/256/1024 MiB);
* ``csr_versioned``: config 3's versioned dimension -- the csr_lut keys, events and
  lookups on a 100,000-state chain with forks: rank index, rank mapping and two
  replays over the 10M-rank domain per step;
* ``reference_chain``: the reference's own published GPU workload -- a 300,000-state
  chain, seed 7, factor period 37, q=2, per-state ranges, on the synthetic 100k-row
  fixture -- through the worker binary (both arms: the event replay and the
  gpu_v7.h drop-in), beside the reference's published RTX 4090 numbers;
* ``served``: the served store (config 5) at 1M/5M/20M requests/s.

Other workloads: ``--workload plain_chain|trip_tree|csr_lut|serving`` prints that
record as the line (``--scale`` multiplies the sizes).

* value: answers/s with inputs resident in HBM (CUDA events around K steps).
  Inputs smaller than twice L2 are timed one replay at a time with a 256 MiB write
  between replays (L2 flushed); larger ones need no flush.
* e2e: the same through the public API with pinned host buffers: every step
  copies parent/events/queries host->device and the answers device->host.
* roofline: the dominant kernel -- the chain sweep (k_chain_sweep) on chains, the
  Euler-tile tree sweep (k_esweep) on forests, the tree sweep (k_sweep) on single
  trees -- with its algorithmic bytes (16 per event
  record, 12 per query record, 8 per answer) over its mean launch time (CUDA
  events on the launch stream), against the measured HBM copy bandwidth.
* cpu_baseline: the oracle's restatement of the reference's CPU path on the box's
  host cores: the block-parallel chain executor (batch_engine_v7.hpp:832-968) on
  every thread for chains, the preorder apply/undo replay
  (batch_engine_v7.hpp:1021-1059) on one thread for trees.

--impl reference times the reference's CPU algorithm for the default workload on
every host thread, all 4,096 trees per step (the same configuration).  Under
torchrun with N>1 every rank runs an independent replica (weak scaling); rank 0
prints.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
import zlib
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "bit-exact range-sum answers/s (plain version-tree replay)"
BATCHED_METRIC = "bit-exact range-sum answers/s (batched uneven trees: one autotuned CUDA-graph launch)"
L2_BYTES = 129 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batched_trees")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--blocks", type=int, default=0)
    ap.add_argument("--path", default="auto", choices=["auto", "chain", "general"],
                    help="plain workloads: force the chain path or the general pipeline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU sample duration")
    ap.add_argument("--plain-steps", type=int, default=2, help="steps of the sequential plain form")
    ap.add_argument("--sample-check", action="store_true", help="batched: check 65 trees instead of all")
    ap.add_argument("--no-autotune", action="store_true", help="batched: use the default tuning")
    ap.add_argument("--tuning", default=None, help="batched: JSON tuning to use instead of the autotuner")
    ap.add_argument("--e2e-chunks", type=int, default=6, help="batched: tree chunks of the host-buffer replay")
    ap.add_argument("--no-serving", action="store_true", help="batched: skip the served-store runs")
    ap.add_argument("--no-subrecords", action="store_true", help="batched: skip the per-config sub-records")
    ap.add_argument("--sub-steps", type=int, default=10, help="timed steps of each sub-record")
    ap.add_argument("--loads", default="1e6,5e6,2e7,4e7,8e7", help="serving: offered loads in requests/s")
    ap.add_argument("--hbm-cap-gb", type=float, default=120.0, help="serving: admission cap of the store")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(ms: float, device) -> float:
    """The slowest rank's time (all_reduce MAX); the time itself on one rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel: str, workload: str):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu summary, if any."""
    p = ROOT / "profiles" / f"{kernel}_{workload}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def oracle_mod():
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle
    return oracle


def load_pkg():
    import __graft_entry__ as g
    return g.package()


# ----------------------------------------------------------------------------- CPU legs
def cpu_tree_sample(w, seconds: float):
    """Oracle preorder replay over the first Euler steps of the workload, one thread."""
    oracle = oracle_mod()
    S = len(w.parent)
    probe = max(1, min(S, 2000))
    _, done, secs = oracle.ev_sweep_prefix(w.parent, w.n_keys, w.events, w.queries, probe)
    rate_steps = probe / max(secs, 1e-9)
    limit = int(min(2 * S, max(probe, rate_steps * seconds)))
    _, done, secs = oracle.ev_sweep_prefix(w.parent, w.n_keys, w.events, w.queries, limit)
    return {"value": done / max(secs, 1e-9), "unit": "answers/s", "cores": 1, "kind": "port",
            "sample": f"preorder replay of the first {limit} of {2 * S} Euler steps ({S} states; "
                      f"{done} answers, {secs:.1f} s)"}


def cpu_chain_sample(w, seconds: float):
    """Oracle block-parallel chain executor (run_blocks, batch_engine_v7.hpp:832-968)
    on every host thread, whole workload per run, repeated for about `seconds`."""
    oracle = oracle_mod()
    threads = oracle.max_threads()
    runs, t0 = 0, time.perf_counter()
    while True:
        oracle.ev_blocks(w.parent, w.n_keys, w.events, w.queries, blocks=threads, threads=threads)
        runs += 1
        el = time.perf_counter() - t0
        if el >= seconds or runs >= 200:
            break
    return {"value": runs * len(w.queries) / el, "unit": "answers/s", "cores": threads, "kind": "port",
            "sample": f"block-parallel chain executor over the whole workload, {runs} runs in {el:.1f} s "
                      f"({len(w.events)} events, {len(w.queries)} queries)"}


def cpu_sample(w, seconds: float):
    return cpu_chain_sample(w, seconds) if w.chain else cpu_tree_sample(w, seconds)


def oracle_answers(w):
    oracle = oracle_mod()
    if w.chain:
        t = oracle.max_threads()
        return oracle.ev_blocks(w.parent, w.n_keys, w.events, w.queries, blocks=t, threads=t)
    return oracle.ev_sweep(w.parent, w.n_keys, w.events, w.queries)


def forest_cpu_sample(w, seconds: float, threads: int = 1, seed: int = 5, all_trees: bool = False):
    """Oracle preorder replay (the reference's tree path, batch_engine_v7.hpp:1021-1059,
    ported) of whole trees in a seeded random order until `seconds` of work (or all
    trees); trees run on `threads` host threads (the oracle call releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    oracle = oracle_mod()
    order = np.random.default_rng(seed).permutation(w.n_trees)

    def one(t):
        tr = w.tree(int(t))
        oracle.ev_sweep(tr.parent, tr.n_keys, tr.events, tr.queries)
        return len(tr.queries), len(tr.parent)

    answers = states = trees = 0
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as pool:
        i = 0
        while i < len(order) and (all_trees or time.perf_counter() - t0 < seconds):
            batch = order[i:i + 4 * threads]
            for a, st in pool.map(one, batch):
                answers += a
                states += st
            trees += len(batch)
            i += len(batch)
    secs = time.perf_counter() - t0
    return {"value": answers / max(secs, 1e-9), "unit": "answers/s", "cores": threads, "kind": "port",
            "sample": f"preorder replay of {trees} of {w.n_trees} trees in a seeded random order "
                      f"({states} states, {answers} answers, {secs:.1f} s)", "trees": trees}


def forest_check_all(w, ans, threads: int) -> int:
    """Every tree's batched answers against the oracle's preorder replay (parallel)."""
    from concurrent.futures import ThreadPoolExecutor
    oracle = oracle_mod()

    def one(t):
        tr = w.tree(int(t))
        q0, q1 = int(w.query_off[t]), int(w.query_off[t + 1])
        return bool(np.array_equal(ans[q0:q1], oracle.ev_sweep(tr.parent, tr.n_keys, tr.events, tr.queries)))

    with ThreadPoolExecutor(max_workers=threads) as pool:
        bad = [t for t, ok in zip(range(w.n_trees), pool.map(one, range(w.n_trees))) if not ok]
    if bad:
        raise SystemExit(f"batched answers of {len(bad)} trees differ from the oracle (first: tree {bad[0]})")
    return w.n_trees


def reference_arm(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    w = load_pkg().workloads.make(args.workload, args.seed, args.scale)
    threads = os.cpu_count() or 1
    if args.workload == "batched_trees":
        # every step replays all trees (the same configuration as the GPU arm)
        vals = [forest_cpu_sample(w, 0.0, threads, seed=5 + i, all_trees=True)
                for i in range(args.warmup + args.steps)][args.warmup:]
        v = statistics.median([x["value"] for x in vals])
        line = {"impl": "reference", "metric": BATCHED_METRIC, "value": v, "unit": "answers/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * len(w.queries) / v, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int64", "data": "synthetic",
                "config": dict(w.describe(), l2="inputs larger than L2"), "same_config": True,
                "cpu_baseline": {"value": v, "unit": "answers/s", "cores": threads, "kind": "port",
                                 "sample": vals[-1]["sample"]},
                "e2e": {"value": v, "unit": "answers/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    if args.workload == "csr_lut":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the version-chain "
                          "replay workloads; csr_lut has no reference CPU arm here"}), flush=True)
        return 0
    steps = args.steps if w.chain else min(args.steps, 3)
    vals = []
    for i in range(args.warmup + steps):
        if w.chain:
            s = cpu_chain_sample(w, 0.0)
        else:
            t0 = time.perf_counter()
            oracle_mod().ev_sweep(w.parent, w.n_keys, w.events, w.queries)
            el = time.perf_counter() - t0
            s = {"value": len(w.queries) / el, "cores": 1,
                 "sample": f"preorder replay of the whole workload in {el:.1f} s"}
        if i >= args.warmup:
            vals.append(s)
    v = statistics.median([x["value"] for x in vals])
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "answers/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * len(w.queries) / v,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic", "config": dict(w.describe(), l2="inputs larger than L2"), "same_config": True,
            "cpu_baseline": {"value": v, "unit": "answers/s", "cores": vals[-1]["cores"], "kind": "port",
                             "sample": vals[-1]["sample"]},
            "e2e": {"value": v, "unit": "answers/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- GPU records
def timed_replays(torch, plan, stream, d_parent, d_events, d_queries, d_answers, steps: int, flush: bool):
    """Mean ms of `steps` replays (CUDA events on the launch stream).  With `flush`,
    every replay is timed alone after a 256 MiB write that evicts L2."""
    buf = torch.empty(256 << 20, dtype=torch.uint8, device=d_parent.device) if flush else None
    plan.timing_reset()
    torch.cuda.synchronize()
    if not flush:
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(steps):
            plan.launch(d_parent, d_events, d_queries, d_answers)
        t1.record(stream)
        torch.cuda.synchronize()
        return t0.elapsed_time(t1) / steps
    pairs = []
    for i in range(steps):
        buf.fill_(i & 255)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        plan.launch(d_parent, d_events, d_queries, d_answers)
        b.record(stream)
        pairs.append((a, b))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in pairs) / steps


def plain_record(args, bw, dev, name: str, scale: float, steps: int, warmup: int, cpu_seconds: float,
                 ws: int = 1, clocks: bool = False) -> dict:
    """One plain workload (one tree): correctness against the oracle, device-resident
    replays, the host-buffer e2e form, the roofline of the dominant kernel and the CPU
    baseline.  Returns the record (the bench line's fields without the boilerplate)."""
    import torch
    t_gen = time.perf_counter()
    w = bw.workloads.make(name, args.seed, scale)
    gen_s = time.perf_counter() - t_gen
    S, E, Q = len(w.parent), len(w.events), len(w.queries)
    h_parent = torch.from_numpy(w.parent).pin_memory()
    h_events = torch.from_numpy(w.events.view(np.int64).reshape(-1, 2)).pin_memory()
    h_queries = torch.from_numpy(w.queries.view(np.int32).reshape(-1, 3)).pin_memory()
    h_answers = torch.empty(Q, dtype=torch.int64).pin_memory()
    d_parent, d_events, d_queries = h_parent.to(dev), h_events.to(dev), h_queries.to(dev)
    d_answers = torch.empty(Q, dtype=torch.int64, device=dev)
    plan = bw.Replay(d_parent, w.n_keys, E, Q, blocks=args.blocks, chain=w.chain, timing=True, path=args.path,
                     wide=w.chain and bw.wide_deltas(w.events))
    chain_path = plan.chain_path(d_events)
    stream = torch.cuda.current_stream(dev)
    for i in range(max(1, warmup)):
        plan.launch(d_parent, d_events, d_queries, d_answers)
        if i == 0:
            st = plan.status()
            if st:
                raise SystemExit(f"{name}: device rejected the workload: {bw.STATUS_NAMES.get(st, st)}")
    torch.cuda.synchronize()
    ans0 = d_answers.cpu().numpy()
    if not np.array_equal(ans0, oracle_answers(w)):
        raise SystemExit(f"{name}: GPU answers differ from the oracle")
    digest = oracle_mod().sha256_hex(ans0.tobytes())
    in_bytes = 4 * S + 16 * E + 12 * Q
    flush = in_bytes < 2 * L2_BYTES
    kernels, blocks = plan.info()
    clk_s = ClockSampler(int(dev.index or 0)) if clocks else None
    if clk_s:
        clk_s.start()
    ms = timed_replays(torch, plan, stream, d_parent, d_events, d_queries, d_answers, steps, flush)
    clk = clk_s.stop() if clk_s else None
    stage_ms, n_timed = plan.stage_times()
    stage_mean = {k: v / max(1, n_timed) for k, v in stage_ms.items()}
    ms = max_over_ranks(ms, dev)
    if not np.array_equal(d_answers.cpu().numpy(), ans0):
        raise SystemExit(f"{name}: answers changed between steps")
    e2e = None
    if not args.no_e2e:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            d_parent.copy_(h_parent, non_blocking=True)
            d_events.copy_(h_events, non_blocking=True)
            d_queries.copy_(h_queries, non_blocking=True)
            plan.launch(d_parent, d_events, d_queries, d_answers)
            h_answers.copy_(d_answers, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ems = max_over_ranks(e0.elapsed_time(e1) / steps, dev)
        if not np.array_equal(h_answers.numpy(), ans0):
            raise SystemExit(f"{name}: e2e answers differ")
        e2e = {"value": ws * Q / (ems / 1e3), "unit": "answers/s", "h2d_bytes_per_step": in_bytes,
               "d2h_bytes_per_step": 8 * Q, "ms_per_step": ems}
    peak, peak_kind = measured_peaks()
    kernel = "k_chain_sweep" if chain_path else "k_sweep"
    sweep_bytes = 16 * E + 20 * Q
    sweep_ms = stage_mean["sweep"]
    achieved = sweep_bytes / (sweep_ms / 1e3) / 1e9
    tag = name if scale == 1.0 else f"{name}_x{scale:g}"
    rec = {
        "value": ws * Q / (ms / 1e3), "unit": "answers/s", "ms_per_step": ms, "steps": steps,
        "config": dict(w.describe(), scale=scale, blocks=blocks, path="chain" if chain_path else "general",
                       l2=("inputs fit in L2: 256 MiB written between timed replays" if flush
                           else "inputs larger than L2 (no flush needed)"), answers_sha256=digest),
        "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": profiled_traffic(kernel, tag),
                     "algorithmic_bytes_per_launch": sweep_bytes, "mean_launch_ms": sweep_ms},
        "pipeline": {"stages_ms": stage_mean, "whole_step_gbs": w.algorithmic_bytes / (ms / 1e3) / 1e9,
                     "whole_step_frac": w.algorithmic_bytes / (ms / 1e3) / 1e9 / peak,
                     "kernels_per_step": kernels},
        "gpu_launches": kernels * steps, "exact": True, "setup": {"generate_s": gen_s}}
    if clk is not None:
        rec["clocks"] = clk
    if e2e:
        rec["e2e"] = e2e
    if cpu_seconds > 0:
        rec["cpu_baseline"] = cpu_sample(w, cpu_seconds)
    return rec


def csr_record(args, bw, dev, steps: int, warmup: int, scale: float = 1.0) -> dict:
    """Sparse-key rank index (10M distinct u64 keys, 20M events, 100M point and 100M
    range lookups): build time and lookup throughput at LUT budgets 64/256/1024 MiB."""
    import torch
    oracle = oracle_mod()
    w = bw.workloads.make("csr_lut", args.seed, scale)
    L = len(w.point)
    d_keys = torch.from_numpy(w.keys.view(np.int64)).to(dev)
    d_amt = torch.from_numpy(w.amounts).to(dev)
    d_point = torch.from_numpy(w.point.view(np.int64)).to(dev)
    d_ranges = torch.from_numpy(np.ascontiguousarray(w.ranges).view(np.int64)).to(dev)
    out_p = torch.empty(L, dtype=torch.int64, device=dev)
    out_r = torch.empty((L, 2), dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev)
    peak, peak_kind = measured_peaks()

    def timed(fn, n):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(n):
            fn()
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    budgets = {}
    rng = np.random.default_rng(7)
    sample = rng.integers(0, L, 200_000)
    for mib in (64, 256, 1024):
        idx = bw.CsrIndex(d_keys, d_amt, key_bits=w.key_bits, lut_budget_bytes=mib << 20)
        build_ms = timed(idx.rebuild, steps)
        p_ms = timed(lambda: idx.point(d_point, out_p), steps)
        r_ms = timed(lambda: idx.range(d_ranges, out_r), steps)
        uk, pre = idx.arrays()
        uk = uk.cpu().numpy().view(np.uint64)
        pre = pre.cpu().numpy()
        if not (np.array_equal(out_p.cpu().numpy()[sample], oracle.csr_point(uk, w.point[sample])) and
                np.array_equal(out_r.cpu().numpy()[sample], oracle.csr_range(uk, pre, w.ranges[sample]))):
            raise SystemExit(f"CSR lookups differ from the oracle at budget {mib} MiB")
        budgets[f"{mib}MiB"] = {
            "shift": idx.shift, "buckets": idx.n_buckets, "distinct_keys": idx.count(), "build_ms": build_ms,
            "point_lookups_per_s": L / (p_ms / 1e3), "point_ms": p_ms, "point_gbs": 16 * L / (p_ms / 1e3) / 1e9,
            "range_lookups_per_s": L / (r_ms / 1e3), "range_ms": r_ms, "range_gbs": 32 * L / (r_ms / 1e3) / 1e9}
        del idx
    head = budgets["64MiB"]
    return {"value": head["point_lookups_per_s"], "unit": "lookups/s", "ms_per_step": head["point_ms"],
            "config": dict(w.describe(), l2="lookup arrays larger than L2 (no flush needed)"),
            "roofline": {"bound": "hbm", "kernel": "k_csr_point", "achieved": head["point_gbs"], "peak": peak,
                         "unit": "GB/s", "frac": head["point_gbs"] / peak, "peak_kind": peak_kind,
                         "traffic": profiled_traffic("k_csr_point", "csr_lut"),
                         "algorithmic_bytes_per_launch": 16 * L},
            "budgets": budgets, "exact": "200,000 sampled lookups per budget against the oracle",
            "gpu_launches": 3 * 3 * steps}


def csr_versioned_record(args, bw, dev, steps: int, scale: float = 1.0) -> dict:
    """Config 3's versioned dimension: the csr_lut keys, events and lookups on a
    100,000-state chain with forks.  Per step: the keys' rank index (bw_csr_build),
    events and lookups mapped to ranks (bw_csr_events, bw_csr_queries), and one
    replay over the 10M-rank domain for the point lookups and one for the range
    lookups.  Checked against the oracle on 100,000 sampled lookups of each kind."""
    import torch
    oracle = oracle_mod()
    t_gen = time.perf_counter()
    w = bw.workloads.csr_versioned(args.seed, scale)
    gen_s = time.perf_counter() - t_gen
    S, E, L = len(w.parent), len(w.ev_key), len(w.pt_key)

    def t(a, dt):
        return torch.from_numpy(np.ascontiguousarray(a).view(dt)).to(dev)
    p = torch.from_numpy(w.parent).to(dev)
    es, ek, ed = t(w.ev_state, np.int32), t(w.ev_key, np.int64), t(w.ev_delta, np.int64)
    ps, pk = t(w.pt_state, np.int32), t(w.pt_key, np.int64)
    rs, rl, rh = t(w.rg_state, np.int32), t(w.rg_lo, np.int64), t(w.rg_hi, np.int64)
    stream = torch.cuda.current_stream(dev)
    ev0, ev1, ev2, ev3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
    times = []
    for i in range(1 + steps):
        torch.cuda.synchronize()
        ev0.record(stream)
        idx = bw.CsrIndex(ek, ed, key_bits=w.key_bits)
        ev_r = idx.events(es, ek, ed)
        q_pt, q_rg = idx.queries(ps, pk), idx.queries(rs, rl, rh)
        ev1.record(stream)
        a_pt = bw.replay(p, max(1, idx.count()), ev_r, q_pt, check=False)
        ev2.record(stream)
        a_rg = bw.replay(p, max(1, idx.count()), ev_r, q_rg, check=False)
        ev3.record(stream)
        torch.cuda.synchronize()
        if i:
            times.append((ev0.elapsed_time(ev1), ev1.elapsed_time(ev2), ev2.elapsed_time(ev3)))
    idx_ms, pt_ms, rg_ms = (statistics.median(x) for x in zip(*times))
    # oracle on sampled lookups (ranks on the host, preorder replay over the rank domain)
    rng = np.random.default_rng(11)
    keys = np.unique(w.ev_key)
    evo = np.empty(E, dtype=bw.workloads.EVENT_DTYPE)
    evo["state"], evo["key"], evo["delta"] = w.ev_state, np.searchsorted(keys, w.ev_key), w.ev_delta
    sp, sr = np.sort(rng.choice(L, 100_000, replace=False)), np.sort(rng.choice(L, 100_000, replace=False))
    qo = np.empty(200_000, dtype=bw.workloads.QUERY_DTYPE)
    r = np.searchsorted(keys, w.pt_key[sp])
    pres = (r < len(keys)) & (keys[np.minimum(r, len(keys) - 1)] == w.pt_key[sp])
    qo["state"][:100_000], qo["lo"][:100_000], qo["hi"][:100_000] = w.pt_state[sp], np.where(pres, r, 0), \
        np.where(pres, r + 1, 0)
    qo["state"][100_000:] = w.rg_state[sr]
    qo["lo"][100_000:], qo["hi"][100_000:] = np.searchsorted(keys, w.rg_lo[sr]), np.searchsorted(keys, w.rg_hi[sr])
    t_cpu = time.perf_counter()
    want_pt = oracle.ev_sweep(w.parent, len(keys), evo, qo[:100_000])
    want_rg = oracle.ev_sweep(w.parent, len(keys), evo, qo[100_000:])
    cpu_s = time.perf_counter() - t_cpu
    if not (np.array_equal(a_pt.cpu().numpy()[sp], want_pt) and np.array_equal(a_rg.cpu().numpy()[sr], want_rg)):
        raise SystemExit("csr_versioned: GPU answers differ from the oracle")
    peak, peak_kind = measured_peaks()
    step_ms = idx_ms + pt_ms + rg_ms
    sweep_bytes = 16 * E + 20 * L
    return {"value": 2 * L / (step_ms / 1e3), "unit": "lookups/s", "ms_per_step": step_ms, "steps": steps,
            "config": {"workload": "csr_versioned", "states": S, "events": E, "distinct_keys": int(w.n_keys),
                       "point_lookups": L, "range_lookups": L, "topology": "tree (chain with forks, p=0.9)",
                       "key_universe_bits": w.key_bits, "l2": "inputs larger than L2 (no flush needed)"},
            "phases_ms": {"index_and_rank_mapping": idx_ms, "point_replay": pt_ms, "range_replay": rg_ms},
            "roofline": {"bound": "hbm", "kernel": "k_sweep", "achieved": sweep_bytes / (pt_ms / 1e3) / 1e9,
                         "peak": peak, "unit": "GB/s", "frac": sweep_bytes / (pt_ms / 1e3) / 1e9 / peak,
                         "peak_kind": peak_kind, "traffic": None, "algorithmic_bytes_per_launch": sweep_bytes,
                         "note": "whole point replay over the rank domain; a 10M-key domain takes several rank "
                                 "slices per block, each sweeping the block's events again"},
            "cpu_baseline": {"value": 200_000 / cpu_s, "unit": "lookups/s", "cores": 1, "kind": "port",
                             "sample": f"preorder replay of all {E} events answering 200,000 sampled lookups "
                                       f"({cpu_s:.1f} s)"},
            "exact": "100,000 sampled point and 100,000 range lookups against the oracle",
            "setup": {"generate_s": gen_s}}


# the reference's published GPU numbers for its own workload (300,000-state chain,
# seed 7, factor period 37, q=2, per-state ranges; RTX 4090 + EPYC 9554)
REFERENCE_PUBLISHED = {
    "hardware": "RTX 4090 + EPYC 9554 (intel / taxi2024 fixtures)",
    "gpu_v7_kernel_ms": {"B32": [11.375, 9.533], "B64": [6.522, 4.600], "B128": [3.505, 2.279]},
    "gpu_v7_full_ms": {"B32": [169.1, 184.7], "B64": [192.0, 181.5], "B128": [233.5, 183.5]},
    "gpu_snapshot_full_ms": {"B32": [129.0, 144.3], "B64": [134.8, 139.1]},
    "best_kernel_answers_per_s": 599998 / 2.279e-3,
    "source": "results/batch_gpu_20261031/summary.json:3-90, results/batch_gpu3_20261031/summary.json:3-78"}


def reference_chain_record(args, bw, dev, steps: int) -> dict:
    """The reference's own GPU workload through the worker binary, one process per
    measurement as the reference measures it (both arms: the event replay and the
    gpu_v7.h drop-in with B=128), plus the warm chain-path replay timed in-process."""
    import torch
    gold = json.loads((ROOT / "tests" / "golden" / "golden.json").read_text())
    case = next(c for c in gold["large_cases"] if c["fixture"] == "survey_100k")
    img = zlib.decompress((ROOT / "tests" / "golden" / "survey_100k.bin.z").read_bytes())
    out = {"workload": "300,000-state chain, seed 7, factor period 37, q=2, per-state ranges, "
                       "synthetic 100k-row 64-group fixture (the reference's 300k survey run)",
           "want_sha256": case["reference"], "published": REFERENCE_PUBLISHED, "worker": {}}
    with tempfile.TemporaryDirectory() as tmp:
        fx = Path(tmp) / "survey_100k.bin"
        fx.write_bytes(img)
        env = dict(os.environ, BWH_RANGE_SCOPE="per_state")
        for arm in ("gb300", "gpu_v7"):
            recs = []
            for r in range(3):
                js = Path(tmp) / f"{arm}{r}.json"
                p = subprocess.run([str(bw._build.WORKER), "--fixture", str(fx), "--base-id", "survey_100k",
                                    "--topology", "0", "--seed", "7", "--factor-period", "37", "--q", "2",
                                    "--repeat", str(r), "--states", "300000", "--arm", arm, "--blocks",
                                    "128" if arm == "gpu_v7" else "0", "--answers", str(Path(tmp) / "a.bin"),
                                    "--json", str(js)], capture_output=True, text=True, env=env)
                if p.returncode:
                    raise SystemExit(f"worker {arm} failed rc={p.returncode}: {p.stderr[-400:]}")
                recs.append(json.loads(js.read_text()))
            if any(x["answers_sha256"] != case["reference"] for x in recs):
                raise SystemExit(f"worker {arm}: answers differ from the reference SHA-256")
            med = sorted(recs, key=lambda x: x["full_ns"])[1]
            out["worker"][arm] = {"full_ms": med["full_ns"] / 1e6,
                                  "phases_ms": {k: v / 1e6 for k, v in med["phases_ns"].items()},
                                  "kernel_ms": (med["gpu"]["kernel_ns"] + med["gpu"]["carry_ns"]
                                                + med["gpu"]["combine_ns"]) / 1e6,
                                  "upload_ms": med["gpu"]["upload_ns"] / 1e6,
                                  "download_ms": med["gpu"]["download_ns"] / 1e6,
                                  "blocks": med["gpu"]["blocks"], "kernels": med["gpu"]["kernels"],
                                  "answers_sha256": med["answers_sha256"], "runs": len(recs)}
    # warm, device-resident replay of the same workload
    w = bw.native_workload(img, 300000, 0, 7, 37, 2, True)
    S, E, Q = len(w.parent), len(w.events), len(w.queries)
    d_parent = torch.from_numpy(w.parent).to(dev)
    d_events = torch.from_numpy(w.events.view(np.int64).reshape(-1, 2)).to(dev)
    d_queries = torch.from_numpy(w.queries.view(np.int32).reshape(-1, 3)).to(dev)
    d_answers = torch.empty(Q, dtype=torch.int64, device=dev)
    plan = bw.Replay(d_parent, w.n_keys, E, Q, chain=True, timing=True, wide=bw.wide_deltas(w.events))
    chain_path = plan.chain_path(d_events)
    for _ in range(3):
        plan.launch(d_parent, d_events, d_queries, d_answers)
    torch.cuda.synchronize()
    if bw.sha256_hex(d_answers.cpu().numpy().tobytes()) != case["reference"]:
        raise SystemExit("reference chain: warm replay answers differ from the reference SHA-256")
    stream = torch.cuda.current_stream(dev)
    ms = timed_replays(torch, plan, stream, d_parent, d_events, d_queries, d_answers, steps,
                       4 * S + 16 * E + 12 * Q < 2 * L2_BYTES)
    stage_ms, n = plan.stage_times()
    peak, peak_kind = measured_peaks()
    sweep = stage_ms["sweep"] / max(1, n)
    out["warm_replay"] = {"path": "chain" if chain_path else "general", "ms": ms, "answers_per_s": Q / (ms / 1e3),
                          "sweep_ms": sweep, "events": E, "queries": Q, "keys": int(w.n_keys),
                          "sweep_frac_of_peak": (16 * E + 20 * Q) / (sweep / 1e3) / 1e9 / peak,
                          "vs_best_published_kernel": (Q / (ms / 1e3)) / REFERENCE_PUBLISHED[
                              "best_kernel_answers_per_s"]}
    best_full = min(min(v) for v in REFERENCE_PUBLISHED["gpu_snapshot_full_ms"].values())
    out["worker_full_vs_best_published_full"] = best_full / out["worker"]["gb300"]["full_ms"]
    out["exact"] = True
    return out


def bench_batched(args):
    """Batched uneven trees: autotuned forest plan replayed from a CUDA graph, against
    4,096 sequential plain launches (one bw_replay_launch per tree)."""
    import ctypes as C
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")
    bw = load_pkg()
    bw.build()
    t_gen = time.perf_counter()
    # N > 1: every rank replays its own batch of trees (seed + rank): independent
    # objects sharded across GPUs with no exchange, per-GPU work fixed (weak scaling)
    w = bw.workloads.make("batched_trees", args.seed + rank, args.scale)
    gen_s = time.perf_counter() - t_gen
    T, S, E, Q = w.n_trees, len(w.parent), len(w.events), len(w.queries)
    shape = (w.state_off, w.event_off, w.query_off, w.n_keys)
    h_parent = torch.from_numpy(w.parent).pin_memory()
    h_events = torch.from_numpy(w.events.view(np.int64).reshape(-1, 2)).pin_memory()
    h_queries = torch.from_numpy(w.queries.view(np.int32).reshape(-1, 3)).pin_memory()
    h_answers = torch.empty(Q, dtype=torch.int64).pin_memory()
    d_parent, d_events, d_queries = h_parent.to(dev), h_events.to(dev), h_queries.to(dev)
    d_answers = torch.empty(Q, dtype=torch.int64, device=dev)
    stream = torch.cuda.Stream(dev)
    oracle = oracle_mod()
    threads = os.cpu_count() or 1

    def ev_timer():
        return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    with torch.cuda.stream(stream):
        t_tune = time.perf_counter()
        if args.tuning:
            tuning, tune_ms = json.loads(args.tuning), None
        elif args.no_autotune:
            tuning, tune_ms = None, None
        else:
            tuning, tune_ms = bw.forest_autotune(*shape, d_parent, d_events, d_queries, d_answers, reps=2,
                                                 stream=stream)
        tune_s = time.perf_counter() - t_tune
        f = bw.Forest(*shape, tuning=tuning, device=dev, stream=stream)
        f.launch_timed(d_parent, d_events, d_queries, d_answers, stream)
        st = f.status(stream)
        if st:
            raise SystemExit(f"device rejected the workload: {bw.STATUS_NAMES.get(st, st)}")
        ans0 = d_answers.cpu().numpy()
        # parity: every tree against the oracle (or, when asked, the largest and 64 seeded)
        t_chk = time.perf_counter()
        if args.sample_check:
            rng = np.random.default_rng(123)
            check = np.unique(np.concatenate([[int(np.argmax(np.diff(w.state_off)))],
                                              rng.choice(T, size=min(T, 64), replace=False)]))
            for t in check:
                tr = w.tree(int(t))
                q0, q1 = int(w.query_off[t]), int(w.query_off[t + 1])
                if not np.array_equal(ans0[q0:q1], oracle.ev_sweep(tr.parent, tr.n_keys, tr.events, tr.queries)):
                    raise SystemExit(f"batched answers of tree {t} differ from the oracle")
            checked = len(check)
        else:
            checked = forest_check_all(w, ans0, threads)
        check_s = time.perf_counter() - t_chk
        digest = oracle.sha256_hex(ans0.tobytes())
        stages = [f.launch_timed(d_parent, d_events, d_queries, d_answers, stream) for _ in range(3)]
        stage_ms = {k: statistics.median([x[k] for x in stages]) for k in stages[0]}
        f.capture(d_parent, d_events, d_queries, d_answers, stream)
        for _ in range(args.warmup):
            f.replay(stream)
        stream.synchronize()

        # ---- timed region: graph replays, inputs resident in HBM
        clocks = ClockSampler(local)
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        clocks.start()
        t0, t1 = ev_timer()
        t0.record(stream)
        for _ in range(args.steps):
            f.replay(stream)
        t1.record(stream)
        torch.cuda.synchronize()
        if ws > 1:
            torch.distributed.barrier()
        clk = clocks.stop()
        ms = t0.elapsed_time(t1) / args.steps
        if not np.array_equal(d_answers.cpu().numpy(), ans0):
            raise SystemExit("answers changed between graph replays")
        ms = max_over_ranks(ms, dev)
        info = f.info()

        # ---- e2e through the public API: pinned host inputs in, answers out, every
        # step; the host-buffer form overlaps chunk copies with the replay of others
        e2e = None
        if not args.no_e2e:
            # each chunk holds a sixth of the trees: half the block work keeps its
            # CTAs busy to the end of the chunk (measured: 18.7 vs 19.4 ms per step)
            e2e_tuning = dict(tuning) if tuning else None
            if e2e_tuning and e2e_tuning.get("block_work", 0) > 0 and args.e2e_chunks > 1:
                e2e_tuning["block_work"] = max(65536, e2e_tuning["block_work"] // 2)
            hf = bw.HostForest(*shape, chunks=args.e2e_chunks, tuning=e2e_tuning, device=dev)
            for _ in range(2):
                hf.run(h_parent, h_events, h_queries, h_answers)
            torch.cuda.synchronize()
            if not np.array_equal(h_answers.numpy(), ans0):
                raise SystemExit("host-buffer answers differ")
            h_answers.zero_()
            torch.cuda.synchronize()
            e0, e1 = ev_timer()
            e0.record(hf.work_stream)
            t_wall = time.perf_counter()
            for _ in range(args.steps):
                hf.run(h_parent, h_events, h_queries, h_answers)
            e1.record(hf.work_stream)
            torch.cuda.synchronize()
            wall_ms = (time.perf_counter() - t_wall) * 1e3 / args.steps
            ems = e0.elapsed_time(e1) / args.steps
            if not np.array_equal(h_answers.numpy(), ans0) or hf.status():
                raise SystemExit("e2e answers differ")
            ems = max_over_ranks(ems, dev)
            e2e = {"value": ws * Q / (ems / 1e3), "unit": "answers/s",
                   "h2d_bytes_per_step": 4 * S + 16 * E + 12 * Q, "d2h_bytes_per_step": 8 * Q, "ms_per_step": ems,
                   "host_wall_ms_per_step": wall_ms, "chunks": len(hf.parts),
                   "tuning": e2e_tuning,
                   "form": "HostForest: per-chunk plans, copies of chunk k+1 overlap the replay of chunk k"}
            del hf

        # ---- plain form: one bw_replay_launch per tree, in sequence, same stream
        plain_ms = None
        lib = bw.gpu_lib()
        args_t = []
        need = 0
        for t in range(T):
            a = bw.BwReplayArgs()
            s0, e0_, q0 = int(w.state_off[t]), int(w.event_off[t]), int(w.query_off[t])
            a.n_states = int(w.state_off[t + 1]) - s0
            a.parent = d_parent.data_ptr() + 4 * s0
            a.n_keys = int(w.n_keys[t])
            a.n_events = int(w.event_off[t + 1]) - e0_
            a.events = d_events.data_ptr() + 16 * e0_ if a.n_events else None
            a.n_queries = int(w.query_off[t + 1]) - q0
            a.queries = d_queries.data_ptr() + 12 * q0 if a.n_queries else None
            a.answers = d_answers.data_ptr() + 8 * q0 if a.n_queries else None
            a.stream = stream.cuda_stream
            nb = C.c_size_t(0)
            if lib.bw_replay_workspace_size(C.byref(a), C.byref(nb)):
                raise SystemExit("plain workspace size failed")
            need = max(need, int(nb.value))
            args_t.append(a)
        pws = torch.empty(need, dtype=torch.uint8, device=dev)
        for a in args_t:
            a.workspace = pws.data_ptr()
            a.workspace_bytes = need
        plain_kernels = 0
        if args.plain_steps > 0:
            d_answers.zero_()
            k_info = C.c_int32(0)
            p0, p1 = ev_timer()
            torch.cuda.synchronize()
            p0.record(stream)
            for _ in range(args.plain_steps):
                for a in args_t:
                    if lib.bw_replay_launch(C.byref(a)):
                        raise SystemExit("plain launch failed")
                    lib.bw_replay_last_info(C.byref(a), C.byref(k_info), None)
                    plain_kernels += int(k_info.value)
            p1.record(stream)
            torch.cuda.synchronize()
            plain_ms = p0.elapsed_time(p1) / args.plain_steps
            if not np.array_equal(d_answers.cpu().numpy(), ans0):
                raise SystemExit("plain per-tree answers differ from the batched answers")

    peak, peak_kind = measured_peaks()
    sweep_bytes = 16 * E + 20 * Q
    sweep_kernel = "k_esweep" if int(info["tuning"].get("tile", 0)) == 6 else "k_sweep"   # tile 6: Euler-tile sweep
    top = max(stage_ms, key=stage_ms.get)
    achieved = sweep_bytes / (stage_ms["sweep"] / 1e3) / 1e9
    value = ws * Q / (ms / 1e3)
    plain_value = ws * Q / (plain_ms / 1e3) if plain_ms else None
    line = {
        "metric": BATCHED_METRIC, "value": value, "unit": "answers/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": dict(w.describe(), blocks=info["blocks"], tuning=info["tuning"],
                       l2="inputs (3.9 GB) larger than L2 (no flush needed)", answers_sha256=digest,
                       parallelism=f"tree-sharded x{ws} (a batch per rank, no exchange)" if ws > 1 else "single"),
        "full_check": checked == T, "checked_trees": int(checked), "check_s": check_s,
        "plain": {"value": plain_value, "unit": "answers/s", "ms_per_step": plain_ms,
                  "launches_per_step": T, "kernels_per_step": plain_kernels // max(1, args.plain_steps),
                  "form": "one bw_replay_launch per tree, sequential on one stream"},
        "batched_vs_plain": value / plain_value if plain_value else None,
        "roofline": {"bound": "hbm", "kernel": sweep_kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": profiled_traffic(sweep_kernel, w.name),
                     "algorithmic_bytes_per_launch": sweep_bytes, "mean_launch_ms": stage_ms["sweep"]},
        "pipeline": {"stages_ms": stage_ms, "dominant_stage": top,
                     "whole_step_gbs": w.algorithmic_bytes / (ms / 1e3) / 1e9,
                     "whole_step_frac": w.algorithmic_bytes / (ms / 1e3) / 1e9 / peak},
        "autotune": {"seconds": tune_s, "best_ms": tune_ms, "tuning": tuning},
        "gpu_launches": info["kernels"] * args.steps,
        "clocks": clk,
        "setup": {"generate_s": gen_s},
    }
    if e2e:
        line["e2e"] = e2e
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = forest_cpu_sample(w, args.cpu_seconds, 1)
    del d_events, d_queries, d_parent, d_answers, f, pws, h_events, h_queries, h_parent, h_answers
    torch.cuda.empty_cache()
    if rank == 0 and not args.no_subrecords:
        sub_cpu = 0.0 if args.no_cpu_baseline else min(8.0, args.cpu_seconds)
        subs = {}
        for key, name, scale in (("plain_chain", "plain_chain", 1.0), ("plain_chain_x100", "plain_chain", 100.0),
                                 ("trip_tree", "trip_tree", 1.0)):
            t_sub = time.perf_counter()
            subs[key] = plain_record(args, bw, dev, name, scale, args.sub_steps, 3, sub_cpu)
            subs[key]["wall_s"] = time.perf_counter() - t_sub
            torch.cuda.empty_cache()
        t_sub = time.perf_counter()
        subs["csr_lut"] = csr_record(args, bw, dev, args.sub_steps, 3)
        subs["csr_lut"]["wall_s"] = time.perf_counter() - t_sub
        torch.cuda.empty_cache()
        t_sub = time.perf_counter()
        subs["csr_versioned"] = csr_versioned_record(args, bw, dev, min(args.sub_steps, 2))
        subs["csr_versioned"]["wall_s"] = time.perf_counter() - t_sub
        torch.cuda.empty_cache()
        t_sub = time.perf_counter()
        subs["reference_chain"] = reference_chain_record(args, bw, dev, args.sub_steps)
        subs["reference_chain"]["wall_s"] = time.perf_counter() - t_sub
        torch.cuda.empty_cache()
        line.update(subs)
        line["gpu_launches"] += sum(int(s.get("gpu_launches") or 0) for s in subs.values())
    if not args.no_serving:
        line["served"] = run_serving(args, bw, args.seed, args.scale)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_serving(args, bw, seed: int, scale: float):
    """Served store on the trip-log tree: the request log at each offered load (open
    loop, Poisson arrivals), every answer checked against the oracle's replay of the
    final tree.  Returns a dict of per-load latency percentiles and rates; the
    highest loads show where achieved falls below offered (saturation)."""
    oracle = oracle_mod()
    t = time.perf_counter()
    log = bw.workloads.serving(seed, scale)
    gen_s = time.perf_counter() - t
    b = log.base
    t = time.perf_counter()
    srv = bw.Server(b.parent, b.n_keys, b.events, max_versions=len(b.parent) + len(log.requests),
                    max_events=len(b.events) + len(log.commit_events),
                    hbm_cap_bytes=int(args.hbm_cap_gb * 1e9))
    build_s = time.perf_counter() - t
    par, ev, qs, order = log.final_forest()
    want = np.zeros(len(log.requests), dtype=np.int64)
    want[order] = oracle.ev_sweep(par, b.n_keys, ev, qs)
    q = log.requests["kind"] == 0
    loads = []
    for rate in [float(x) for x in args.loads.split(",") if x] + [None]:
        srv.reset()
        arr = None if rate is None else log.arrival / rate
        ans, lat, st = srv.run(log.requests, log.commit_events, arr, max_inflight=1 << 16)
        if not np.array_equal(ans[q], want[q]):
            raise SystemExit(f"served answers differ from the oracle at {rate} requests/s")
        loads.append({"offered_rps": rate if rate is not None else "all at once",
                      "achieved_rps": st["requests"] / st["wall_s"],
                      "answers_per_s": st["queries"] / st["wall_s"],
                      "p50_us": float(np.percentile(lat, 50)), "p99_us": float(np.percentile(lat, 99)),
                      "p50_query_us": float(np.percentile(lat[q], 50)),
                      "p99_query_us": float(np.percentile(lat[q], 99)), "wall_s": st["wall_s"]})
    info = srv.info()
    srv.close()
    return {"config": log.describe(), "store": {"checkpoints": info["checkpoints"], "spacing": info["spacing"],
                                                "store_gb": info["store_bytes"] / 1e9,
                                                "cap_gb": args.hbm_cap_gb,
                                                "loop_warps": info["warps"]},
            "loads": loads, "saturated_answers_per_s": max(x["answers_per_s"] for x in loads),
            "exact": True, "answers_sha256": oracle.sha256_hex(want[q].tobytes()),
            "setup_s": {"generate": gen_s, "store_build": build_s}}


def bench_serving(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    bw = load_pkg()
    bw.build()
    clocks = ClockSampler(local)
    clocks.start()
    res = run_serving(args, bw, args.seed, args.scale)
    clk = clocks.stop()
    top = [x for x in res["loads"] if x["offered_rps"] != "all at once"][-1]
    line = {"metric": "served range-sum answers/s (persistent request loop, open-loop Poisson arrivals)",
            "value": top["answers_per_s"], "unit": "answers/s", "n_gpus": 1, "steps": len(res["loads"]),
            "warmup": 0, "ms_per_step": top["wall_s"] * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64", "data": "synthetic",
            "config": dict(res["config"], offered_rps=top["offered_rps"]),
            "p50_us": top["p50_us"], "p99_us": top["p99_us"], "served": res, "gpu_launches": 1 + len(res["loads"]),
            "clocks": clk}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def bench_plain(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")
    bw = load_pkg()
    bw.build()
    if ws > 1:
        torch.distributed.barrier()
    cpu = 0.0 if (args.no_cpu_baseline or rank != 0 or ws > 1) else args.cpu_seconds
    rec = plain_record(args, bw, dev, args.workload, args.scale, args.steps, args.warmup, cpu, ws=ws, clocks=True)
    line = {"metric": METRIC, "value": rec.pop("value"), "unit": rec.pop("unit"), "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": rec.pop("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic"}
    cfg = rec.pop("config")
    cfg["parallelism"] = f"replicas{ws}" if ws > 1 else "single"
    line["config"] = cfg
    line.update(rec)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def bench_csr(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device(f"cuda:{local}")
    bw = load_pkg()
    bw.build()
    clocks = ClockSampler(local)
    clocks.start()
    rec = csr_record(args, bw, dev, args.steps, args.warmup, args.scale)
    clk = clocks.stop()
    line = {"metric": "exact sparse-key rank lookups/s (CSR rank-LUT, point)", "value": rec.pop("value"),
            "unit": rec.pop("unit"), "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": rec.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic", "clocks": clk}
    line.update(rec)
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def bench_csr_versioned(args):
    """``--workload csr_versioned``: config 3's versioned dimension alone, one line."""
    import torch
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    bw = load_pkg()
    bw.build()
    rec = csr_versioned_record(args, bw, dev, args.steps, args.scale)
    line = {"metric": "exact versioned sparse-key lookups/s (CSR ranks + version-tree replay)", "n_gpus": 1,
            "warmup": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
            "data": "synthetic", **rec}
    print(json.dumps(line), flush=True)
    return 0


def bench_reference_chain(args):
    """``--workload reference_chain``: the reference's own GPU workload alone (its
    300,000-state chain) through both worker arms and the warm replay, one JSON line."""
    import torch
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    bw = load_pkg()
    bw.build()
    rec = reference_chain_record(args, bw, dev, args.steps)
    w = rec["warm_replay"]
    line = {"metric": "bit-exact range-sum answers/s (the reference's 300,000-state chain, warm replay)",
            "value": w["answers_per_s"], "unit": "answers/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": w["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64", "data": "synthetic", "config": {"workload": "reference_chain"},
            **rec}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "reference_chain":
        return bench_reference_chain(args)
    if args.workload == "csr_versioned":
        return bench_csr_versioned(args)
    if args.workload == "csr_lut":
        return bench_csr(args)
    if args.workload == "batched_trees":
        return bench_batched(args)
    if args.workload == "serving":
        return bench_serving(args)
    return bench_plain(args)


if __name__ == "__main__":
    sys.exit(main())
