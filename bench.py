#!/usr/bin/env python3
"""Benchmark of the overlap hot path: overlapped read-bases/sec on one GB300.

Workload (per GPU): a seeded 5 Mb genome carrying 30 copies of a 5 kb repeat
at 1 % divergence and 2 % (AT)n tracts of 200-2,000 bp; HiFi-like reads at
40x, lognormal(15 kb, 3 kb), 0.2 % substitution+indel error; k = 17; solid
k-mers seen >= 2 times, repetitive above 5 x coverage.  Synthetic data: no
dataset exists here, so the generator reproduces the named shapes.

A step is one pass of the overlap stage (candidate hits -> Flye's KmerMatch
sort -> chaining DP -> backtrack -> overlap rows) over every read of the
workload against the device-resident index, batched: all reads in one pass.

* ``value``: read bases per second on the device with the reads already in
  HBM (CUDA events on the library's stream, stages 0-4);
* ``e2e``: the same metric through the public C ABI with host buffers
  (pinned), the host->device copy of the reads and the device->host copy of
  the rows inside the timed region;
* ``plain``: the one-read-per-launch path on a sample of reads, with per-read
  p50/p99 latency;
* ``roofline``: the dominant stage's algorithmic bytes / its event time
  against the measured HBM copy bandwidth;
* ``cpu_baseline``: the CPU oracle (a restatement of the reference's CPU
  path) on the host's cores over a bounded sample of the same reads, with
  the host's CPU model;
* ``launch_shape``: blocks per SM of the counter-driven kernels, as the
  autotuner chose them on the first ``--autotune`` reads before the timed
  steps;
* ``stage_rooflines``: every stage's algorithmic GB/s and fraction of the
  HBM peak, with hit generation and chaining on their own;
* ``configs``: the plain 1 Mb overlap configuration and the read-to-graph
  configuration, each batched and one read per call, and the scale
  configuration (500 Mb genome, 15 Gbp of ONT reads, 180 GB budget; one
  warm-up call and one timed call through the C ABI from pinned buffers;
  ``--scale-genome`` shrinks it with its budget);
* ``serving``: continuous batching through cuflye_submit / cuflye_poll on a
  100 Mb indexed genome at several Poisson arrival rates (p50 / p99).

``--impl reference`` times that CPU implementation alone, on the same
workload, metric and unit.  Under torchrun the reads are split over the ranks,
balanced by length (strong scaling: every rank holds the index of all reads,
and reads are independent queries); ``value`` sums all ranks' bases over the
slowest rank's time.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "overlapped read-bases/sec on 1 GB300 (batched vs plain); p50/p99 query latency"
UNIT = "read-bases/s"
WORKLOAD = ("5 Mb genome, 30 x 5 kb repeat (1% div) + 2% (AT)n; HiFi 40x lognormal(15 kb, 3 kb), "
            "0.2% error; k=17; batched: all reads in one pass")


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def reduce_max(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {}


class ClockSampler:
    """nvidia-smi samples during the timed region (clocks, throttle reasons)."""

    def __init__(self, index: int, path: Path):
        self.path = path
        self.proc = None
        try:
            self.fh = open(path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={index}", "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait(timeout=10)
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "samples": len(sm),
                "reasons": sorted(reasons)}


def make_workload(args):
    from cuflye_gb300 import synth
    return synth.batched_repeats(seed=args.seed, genome_len=args.genome_len,
                                 coverage=args.coverage)


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    import platform
    import re
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        m = re.search(r"^Model name:\s*(.+)$", out, re.M)
        if m:
            return m.group(1).strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        txt = Path("/proc/cpuinfo").read_text()
        m = re.search(r"^model name\s*:\s*(.+)$", txt, re.M)
        if m:
            return m.group(1).strip()
        part = re.search(r"^CPU part\s*:\s*(\S+)", txt, re.M)
        if part:
            return f"{platform.machine()} CPU part {part.group(1)}"
    except OSError:
        pass
    return platform.machine()


def oracle_index(wl):
    """The CPU oracle's index of the workload's reads, and its build time."""
    from oracle import oracle as O
    O.build()
    O.set_stable(False)  # libstdc++ std::sort order at every sort point, as Flye
    reads = wl.reads
    b = O.SeqBatch(reads.ids, reads.offsets, reads.bases.tobytes())
    t0 = time.time()
    idx = O.Index.build(wl.k, b, wl.min_freq, wl.max_freq)
    return idx, time.time() - t0


def oracle_run(wl, idx, picks) -> tuple[dict, float]:
    """The CPU oracle over the reads `picks` on all host cores: its rows and
    its wall time."""
    from oracle import oracle as O
    sub = wl.reads.subset(picks)
    qb = O.SeqBatch(sub.ids, sub.offsets, sub.bases.tobytes())
    t = time.perf_counter()
    res = O.overlaps(idx, qb, O.default_params(**wl.params), threads=os.cpu_count() or 1)
    return res, time.perf_counter() - t


def bench_config(wl) -> dict:
    """The workload's description, identical in both arms' lines."""
    return {"workload": WORKLOAD, "reads": wl.reads.n, "read_bases": wl.reads.total_bases,
            "k": wl.k, "l2": "inputs larger than L2 (about 12 B x 7e9 hits per step, "
                              "index 1.5 GB)"}


def rows_tuples(rows) -> list:
    """ABI overlap rows (GPU) as comparable tuples, divergence as float bits."""
    return [(int(r["cur_id"]), int(r["cur_begin"]), int(r["cur_end"]), int(r["cur_len"]),
             int(r["ext_id"]), int(r["ext_begin"]), int(r["ext_end"]), int(r["ext_len"]),
             int(r["score"]), np.float32(r["seq_divergence"]).view(np.uint32).item())
            for r in rows]


def oracle_tuples(res) -> list:
    return [tuple(int(v) for v in row) + (np.float32(dv).view(np.uint32).item(),)
            for row, dv in zip(res["cols"], res["divergence"])]


def run_reference(args, world, rank) -> None:
    """The reference's CPU path (the oracle, a restatement of it) on every
    host core.  Step i takes the next --reference-sample reads of the
    workload (wrapping around), so the timed steps together cover
    steps x sample reads."""
    if rank != 0:
        return
    wl = make_workload(args)
    idx, build_s = oracle_index(wl)
    n, m = wl.reads.n, max(1, min(args.reference_sample, wl.reads.n))
    times, bases = [], []
    for step in range(args.warmup + args.steps):
        picks = (np.arange(m) + step * m) % n
        _, t = oracle_run(wl, idx, picks)
        times.append(t)
        bases.append(int(np.diff(wl.reads.offsets)[picks].sum()))
    timed, tb = times[args.warmup:], bases[args.warmup:]
    v = sum(tb) / sum(timed)
    cores = os.cpu_count() or 1
    covered = min(n, args.steps * m)
    sample = (f"each step the next {m} reads of the workload (wrapping), {covered} distinct "
              f"reads and {sum(tb)} bases over the {args.steps} timed steps, against the full "
              f"index; CPU oracle on {cores} threads")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000 * sum(timed) / len(timed), "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": bench_config(wl),
            "index_build_s": round(build_s, 2),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "cpu_model": cpu_model(),
                             "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


_PINNED = []  # keeps the pinned host allocations alive for the whole run


def pinned_like(a: np.ndarray) -> np.ndarray:
    """A copy of `a` in page-locked host memory (torch's pinned allocator)."""
    import torch
    t = torch.empty(max(a.nbytes, 1), dtype=torch.uint8).pin_memory()
    _PINNED.append(t)
    v = t.numpy()[: a.nbytes].view(a.dtype).reshape(a.shape)
    v[...] = a
    return v


def serving_run(args, device: int) -> dict:
    """Continuous batching (cuflye_submit / cuflye_poll) on the serving
    workload: single-read requests arriving by a Poisson process at each
    offered rate, p50/p99 latency from submit to rows, throughput, and the
    plain one-read-per-call path on the same queries."""
    import queue
    import threading
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import CudaBackend, CudaServer, OverlapParams, Sequences
    sw = synth.serving_workload(seed=4)
    q = sw.queries
    pool = [Sequences(q.ids[i:i + 1].copy(), np.array([0, q.offsets[i + 1] - q.offsets[i]],
                                                         dtype=np.int64),
                      np.ascontiguousarray(q.bases[q.offsets[i]:q.offsets[i + 1]]))
            for i in range(q.n)]
    out = {"workload": "100 Mb genome, 5% interspersed repeats (2-8 kb families, 1-3% div) "
                       "indexed as 1 Mb pieces, k=15; single-read requests, lengths log-uniform "
                       "1-100 kb, 1% or 8% error 50/50, Poisson arrivals",
           "budget_bytes": 40 << 30, "workers": args.serve_workers,
           "max_batch_bases": args.serve_batch_bases, "rates": []}
    with CudaBackend(device=device, memory_budget_bytes=40 << 30) as be:
        t = time.perf_counter()
        be.build_index(sw.targets, sw.k, sw.min_freq, sw.max_freq)
        out["index_build_s"] = round(time.perf_counter() - t, 3)
        p = OverlapParams.make(**sw.params)
        # plain path: one read per call
        lat = []
        for s in pool[:5]:
            be.overlaps(s, p)
        t = time.perf_counter()
        nb = 0
        for s in pool[:args.plain_sample or 100]:
            t1 = time.perf_counter()
            be.overlaps(s, p)
            lat.append(time.perf_counter() - t1)
            nb += int(s.offsets[-1])
        plain_s = time.perf_counter() - t
        lat_ms = sorted(1000 * x for x in lat)
        out["plain"] = {"read_bases_per_s": nb / plain_s, "p50_ms": lat_ms[len(lat_ms) // 2],
                        "p99_ms": lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))]}
        best = 0.0
        with CudaServer(be, p, workers=args.serve_workers,
                        max_batch_bases=args.serve_batch_bases) as srv:
            for s in pool[:20]:
                srv.poll(srv.submit(s), -1)
            for rate in args.serve_rates:
                n = max(10, min(int(rate * args.serve_seconds), 50_000))
                rng = np.random.default_rng(int(rate))
                arrive = np.cumsum(rng.exponential(1.0 / rate, n))
                t_sub = np.zeros(n)
                t_done = np.zeros(n)
                nbases = np.zeros(n)
                tq: queue.Queue = queue.Queue()
                b0 = srv.stats()

                failed: list = []

                done_at: dict = {}

                def poller():
                    # requests in completion order (batches of the two workers
                    # finish out of submission order)
                    for _ in range(n):
                        try:
                            tk, _rows = srv.poll_any(-1)
                        except Exception as e:  # recorded; the rate reports it
                            failed.append(str(e))
                            continue
                        done_at[tk] = time.perf_counter()

                th = threading.Thread(target=poller)
                th.start()
                t0 = time.perf_counter()
                for i in range(n):
                    wait = arrive[i] - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(wait)
                    s = pool[i % len(pool)]
                    t_sub[i] = time.perf_counter()
                    tq.put((i, srv.submit(s)))
                    nbases[i] = s.offsets[-1]
                th.join()
                while not tq.empty():
                    i, tk = tq.get()
                    t_done[i] = done_at.get(tk, np.nan)
                b1 = srv.stats()
                if failed:
                    out["rates"].append({"offered_reads_per_s": rate, "requests": n,
                                         "failed": len(failed), "first_error": failed[0]})
                    continue
                lat = np.sort(1000 * (t_done - t_sub))
                span = t_done.max() - t_sub[0]
                thr = float(nbases.sum() / span)
                best = max(best, thr)
                out["rates"].append({
                    "offered_reads_per_s": rate, "requests": n,
                    "submitted_reads_per_s": round(n / max(t_sub[-1] - t_sub[0], 1e-9), 1),
                    "p50_ms": float(lat[n // 2]), "p99_ms": float(lat[min(n - 1, int(0.99 * n))]),
                    "read_bases_per_s": thr,
                    "batches": b1["batches"] - b0["batches"]})
        out["served_over_plain"] = best / out["plain"]["read_bases_per_s"]
    return out


STAGES = ["hit generation", "KmerMatch sort", "group prefilter + ext re-sort", "chaining DP",
          "score sort + backtrack + rows"]


def stage_rooflines(names, stage_ms, stage_bytes, peak) -> dict:
    """Achieved algorithmic GB/s and fraction of the measured HBM peak per
    stage, and for hit generation and for chaining (groups + DP + backtrack)
    on their own."""
    def one(ms, by):
        gbs = by / (ms / 1000.0) / 1e9 if ms > 0 else None
        return {"achieved_gbs": gbs, "frac": (gbs / peak) if (gbs and peak) else None}
    out = {n: one(float(stage_ms[i]), float(stage_bytes[i])) for i, n in enumerate(names)}
    out["hit generation (target 0.5)"] = out[names[0]]
    out["chaining (target 0.5)"] = one(float(stage_ms[2:5].sum()), float(stage_bytes[2:5].sum()))
    return out


def _pct(xs, q):
    xs = sorted(xs)
    return xs[min(len(xs) - 1, int(q * len(xs)))] if xs else None


def _plain_pass(gpu, reads, call, sample):
    """One read per call (and per launch sequence) over the first `sample`
    reads: read-bases/s and p50 / p99 latency in ms."""
    from cuflye_gb300.backend import Sequences
    sub = reads.subset(np.arange(min(sample, reads.n)))
    one = [Sequences(np.array([sub.ids[i]], dtype=np.int64),
                     np.array([0, sub.offsets[i + 1] - sub.offsets[i]], dtype=np.int64),
                     np.ascontiguousarray(sub.bases[sub.offsets[i]:sub.offsets[i + 1]]))
           for i in range(sub.n)]
    call(one[0])
    lat = []
    t = time.perf_counter()
    for q in one:
        t1 = time.perf_counter()
        call(q)
        lat.append(1000.0 * (time.perf_counter() - t1))
    return {"read_bases_per_s": sub.total_bases / (time.perf_counter() - t), "reads": sub.n,
            "p50_ms": _pct(lat, 0.5), "p99_ms": _pct(lat, 0.99)}


def extra_configs(args, device: int) -> dict:
    """The other single-GPU configurations of the metric, each batched (all
    reads in one call through the C ABI, host buffers, wall time) and plain
    (one read per call): config 1, plain overlap on a 1 Mb genome at 20x
    (k = 15); config 3, read-to-graph chains of ONT 30x reads against a
    400-edge graph of a 20 Mb genome (k = 15)."""
    from cuflye_gb300 import synth
    from cuflye_gb300.backend import CudaBackend, OverlapParams, R2GParams, Sequences
    out = {}
    if "1" in args.configs:
        wl = synth.plain_overlap()
        p = OverlapParams.make(**wl.params)
        with CudaBackend(device=device, memory_budget_bytes=0) as be:
            be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
            q = Sequences.of(wl.reads)
            be.overlaps(q, p)
            t = time.perf_counter()
            for _ in range(3):
                rows = be.overlaps(q, p)
            wall = (time.perf_counter() - t) / 3
            be.set_batch_queries(1)
            plain = _plain_pass(be, wl.reads, lambda s: be.overlaps(s, p), args.config_plain_sample)
            be.set_batch_queries(0)
        out["1_plain_overlap"] = {
            "workload": "1 Mb uniform genome; reads 20x lognormal(10 kb, 5 kb) in 1-50 kb, "
                        "1/0.5/0.5 % sub/ins/del; k=15", "reads": wl.reads.n,
            "read_bases": wl.reads.total_bases, "rows": len(rows),
            "batched_read_bases_per_s": wl.reads.total_bases / wall, "plain": plain,
            "batched_over_plain": wl.reads.total_bases / wall / plain["read_bases_per_s"]}
    if "3" in args.configs:
        wl = synth.read_to_graph()
        g = wl.graph
        p = OverlapParams.make(**wl.params)
        r = R2GParams.make(**synth.R2G_PARAMS)
        with CudaBackend(device=device, memory_budget_bytes=0) as be:
            be.build_index(g.seqs, wl.k, wl.min_freq, wl.max_freq)
            be.set_graph(g.edge_ids, g.seq_ids, g.left, g.right)
            q = Sequences.of(wl.reads)
            be.read_to_graph(q, p, r)
            t = time.perf_counter()
            rows = be.read_to_graph(q, p, r)
            wall = time.perf_counter() - t
            ms, _ = be.last_timing()
            plain = _plain_pass(be, wl.reads, lambda s: be.read_to_graph(s, p, r),
                                args.config_plain_sample)
        out["3_read_to_graph"] = {
            "workload": "20 Mb genome cut into 400 edges (log-uniform 5-500 kb, 10 % duplicated "
                        "at 0.5 %); ONT 30x lognormal(20 kb, 12 kb) in 1-150 kb, 8 % error; k=15",
            "reads": wl.reads.n, "read_bases": wl.reads.total_bases, "alignment_rows": len(rows),
            "batched_read_bases_per_s": wl.reads.total_bases / wall,
            "device_read_bases_per_s": wl.reads.total_bases / (sum(ms) / 1000.0),
            "plain": plain,
            "batched_over_plain": wl.reads.total_bases / wall / plain["read_bases_per_s"]}
    if "5" in args.configs:
        out["5_scale"] = scale_config(args, device)
    return out


def scale_config(args, device: int) -> dict:
    """Config 5 at a chosen genome length (the configuration is 500 Mb): the
    genome's 10 % repeats and ONT 30x reads as specified, and the 180 GB
    memory budget scaled by the same factor, so the index is built in key
    ranges and the reads stream from pinned host buffers in passes.  One
    warm-up call, then one timed call through the C ABI."""
    from cuflye_gb300 import abi, synth
    from cuflye_gb300.backend import CudaBackend, OverlapParams, Sequences
    scale = args.scale_genome / 500e6
    # sparse error draws: the same error rates, fast enough for 15 Gbp of reads
    wl = synth.scale_ont(seed=6, genome_len=int(args.scale_genome), coverage=30.0,
                         sparse_errors=True)
    budget = int(180e9 * scale)
    p = OverlapParams.make(**wl.params)
    q = Sequences(pinned_like(np.ascontiguousarray(wl.reads.ids, dtype=np.int64)),
                  pinned_like(np.ascontiguousarray(wl.reads.offsets, dtype=np.int64)),
                  pinned_like(np.ascontiguousarray(wl.reads.bases, dtype=np.uint8)))
    with CudaBackend(device=device, memory_budget_bytes=budget) as be:
        t = time.perf_counter()
        stats = be.build_index(wl.reads, wl.k, wl.min_freq, wl.max_freq)
        build_s = time.perf_counter() - t
        ranges = be.last_index_ranges()
        # the warm-up call gives the row count: the timed call writes into a
        # pinned buffer of that size (a short buffer would make it run twice)
        warm = be.overlaps(q, p)
        out = pinned_like(np.zeros(len(warm) + 1024, dtype=abi.OVERLAP_DTYPE))
        t = time.perf_counter()
        rows = be.overlaps(q, p, out=out)
        wall = time.perf_counter() - t
        ms, by = be.last_timing()
        passes = be.last_passes()
        pass_stats = be.last_pass_stats()
        sort_paths = be.last_sort_stats()
        dev_peak = be.memory_stats()[1]
    ms = np.array(ms)
    by = np.array(by, dtype=np.float64)
    bases = float(wl.reads.total_bases)
    return {
        "workload": f"{args.scale_genome / 1e6:g} Mb genome (the 500 Mb configuration at "
                    f"{scale:g} of its length), 10 % repeats (1-20 kb families, 0.5-5 % "
                    "divergence); ONT 30x lognormal(25 kb, 15 kb) in 1-150 kb, 6 % error; k=17",
        "reads": wl.reads.n, "read_bases": int(bases), "rows": len(rows),
        "memory_budget_bytes": budget, "device_peak_bytes": int(dev_peak),
        "index_build_s": round(build_s, 3), "index_key_ranges": ranges,
        "index_positions": stats["positions"], "passes": passes,
        "pass_retries": pass_stats["retries"], "host_alloc_ms": pass_stats["alloc_ms"],
        "sort_paths": sort_paths,
        "batched_read_bases_per_s": bases / wall,
        "device_read_bases_per_s": bases / (float(ms[:5].sum()) / 1000.0),
        "stages_ms": {n: round(float(ms[i]), 3)
                      for i, n in enumerate(STAGES + ["output + D2H", "H2D"])},
        "stage_rooflines": stage_rooflines(STAGES, ms, by, measured_peaks().get("hbm_gbs")),
    }


def shard_reads(lengths, world: int) -> list[np.ndarray]:
    """Length-balanced split of the reads over the ranks: longest first, each
    to the rank with the fewest bases so far (ties to the lower rank); each
    rank's reads in input order."""
    lengths = np.asarray(lengths, dtype=np.int64)
    load = np.zeros(world, dtype=np.int64)
    owner = np.empty(len(lengths), dtype=np.int64)
    for i in np.argsort(-lengths, kind="stable"):
        r = int(np.argmin(load))
        owner[i] = r
        load[r] += lengths[i]
    return [np.flatnonzero(owner == r) for r in range(world)]


def run_ours(args, world, rank, local) -> None:
    from cuflye_gb300 import abi
    from cuflye_gb300.backend import CudaBackend, OverlapParams, Sequences, load_library
    import ctypes

    wl = make_workload(args)
    reads = wl.reads
    params = OverlapParams.make(**wl.params)
    gpu = CudaBackend(device=local, memory_budget_bytes=0)
    t0 = time.perf_counter()
    stats = gpu.build_index(reads, wl.k, wl.min_freq, wl.max_freq)
    index_s = time.perf_counter() - t0
    tune = None
    if args.autotune > 0:
        # the autotuner picks the launch shape on a sample before the timed steps
        t0 = time.perf_counter()
        tune = gpu.autotune(reads.subset(np.arange(min(args.autotune, reads.n))), params)
        tune.update(sample_reads=min(args.autotune, reads.n),
                    seconds=round(time.perf_counter() - t0, 3))
    # this rank's queries (all reads on one GPU; a length-balanced share
    # under torchrun), against the index of all reads
    mine = reads if world == 1 else reads.subset(shard_reads(np.diff(reads.offsets), world)[rank])
    if args.query_sample > 0:
        # profiling cases: the first reads only, against the index of all
        mine = mine.subset(np.arange(min(args.query_sample, mine.n)))
    if args.emission_mode >= 0:
        gpu.set_sorted_emission(args.emission_mode)
    # pinned host inputs / outputs for the end-to-end leg
    seqs = Sequences(pinned_like(np.ascontiguousarray(mine.ids, dtype=np.int64)),
                     pinned_like(np.ascontiguousarray(mine.offsets, dtype=np.int64)),
                     pinned_like(np.ascontiguousarray(mine.bases, dtype=np.uint8)))
    out = pinned_like(np.zeros(max(1024, 256 * mine.n), dtype=abi.OVERLAP_DTYPE))
    L = load_library()
    launches = ctypes.c_uint64()
    for _ in range(args.warmup):
        rows = gpu.overlaps(seqs, params, out=out)
    barrier(world)
    L.cuflye_kernel_launches(ctypes.byref(launches))
    l0 = launches.value
    log = Path(args.clock_log.format(rank=rank)) if args.clock_log else \
        Path(f"/tmp/cuflye_clocks_rank{rank}.csv")
    sampler = ClockSampler(local, log)
    dev_ms, wall_s, stage_tot, bytes_tot = [], [], np.zeros(7), np.zeros(7)
    nrows = 0
    for _ in range(args.steps):
        t = time.perf_counter()
        rows = gpu.overlaps(seqs, params, out=out)
        wall_s.append(time.perf_counter() - t)
        ms, by = gpu.last_timing()
        sort_paths = gpu.last_sort_stats()
        ms = np.array(ms)
        stage_tot += ms
        bytes_tot += np.array(by, dtype=np.float64)
        dev_ms.append(float(ms[:5].sum()))
        nrows = len(rows)
    clocks = sampler.stop()
    L.cuflye_kernel_launches(ctypes.byref(launches))
    launches_step = (launches.value - l0) / args.steps
    barrier(world)
    bases = float(mine.total_bases)
    dev_total = reduce_max(world, sum(dev_ms) / 1000.0)
    wall_total = reduce_max(world, sum(wall_s))
    all_bases = reduce_sum(world, bases * args.steps)
    value = all_bases / dev_total
    e2e = all_bases / wall_total
    # dominant stage roofline (stages 0-4 carry algorithmic bytes)
    names = STAGES
    dom = int(np.argmax(stage_tot[:5]))
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    achieved = bytes_tot[dom] / (stage_tot[dom] / 1000.0) / 1e9
    traffic = None
    tfile = REPO / "profiles" / "ncu_traffic.json"
    if tfile.exists():
        tj = json.loads(tfile.read_text())
        per = tj.get("stages", {}).get(names[dom])
        if per and per.get("dram_bytes_per_hit"):
            traffic = per["dram_bytes_per_hit"] * (bytes_tot[dom] / args.steps) / max(
                1.0, per.get("alg_bytes_per_hit", 1.0))
    # plain path: one read per launch, sample
    plain = None
    lat = []
    if rank == 0 and args.plain_sample > 0:
        sub = reads.subset(np.arange(min(args.plain_sample, reads.n)))
        gpu.set_batch_queries(1)
        one = [Sequences(np.array([sub.ids[i]], dtype=np.int64),
                         np.array([0, sub.offsets[i + 1] - sub.offsets[i]], dtype=np.int64),
                         np.ascontiguousarray(sub.bases[sub.offsets[i]:sub.offsets[i + 1]]))
               for i in range(sub.n)]
        gpu.overlaps(one[0], params)
        t = time.perf_counter()
        for s in one:
            t1 = time.perf_counter()
            gpu.overlaps(s, params)
            lat.append(time.perf_counter() - t1)
        plain_s = time.perf_counter() - t
        gpu.set_batch_queries(0)
        plain = {"value": sub.total_bases / plain_s, "unit": UNIT,
                 "sample": f"first {sub.n} reads, one read per call and per launch sequence",
                 "batched_over_plain": (bases / (sum(wall_s) / len(wall_s))) /
                                       (sub.total_bases / plain_s)}
    cpu = None
    parity = None
    if rank == 0 and world == 1 and args.cpu_sample > 0:
        # the CPU oracle on a sample spread over the workload, timed, and its
        # rows compared with the GPU's rows for the same reads
        m = min(args.cpu_sample, reads.n)
        picks = np.linspace(0, reads.n - 1, m).astype(np.int64)
        idx, _ = oracle_index(wl)
        res, secs = oracle_run(wl, idx, picks)
        sub = reads.subset(picks)
        got = rows_tuples(gpu.overlaps(sub, params))
        exp = oracle_tuples(res)
        sb = int(sub.total_bases)
        cores = os.cpu_count() or 1
        cpu = {"value": sb / secs, "unit": UNIT, "cores": cores, "cpu_model": cpu_model(),
               "kind": "port",
               "sample": f"{m} reads spread evenly over the workload ({sb} bases) against the "
                         f"full index, CPU oracle on {cores} threads"}
        first_diff = next((i for i, (a, b) in enumerate(zip(got, exp)) if a != b),
                          None if len(got) == len(exp) else min(len(got), len(exp)))
        parity = {"reads": m, "rows": len(exp), "gpu_rows": len(got), "equal": got == exp,
                  "first_difference": first_diff,
                  "compared": "every overlap row of the sample, all fields, divergence as "
                              "float bits, GPU (C ABI) vs CPU oracle (libstdc++ sort order)"}
    if rank != 0:
        return
    mean_ms = 1000.0 * dev_total / args.steps
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True,
        "scaling": "strong", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": bench_config(wl),
        "index": {"positions": stats["positions"], "keys": stats["keys"],
                  "build_s": round(index_s, 3)},
        "rows_per_step": nrows,
        "e2e": {"value": e2e, "unit": UNIT,
                "h2d_bytes_per_step": int(seqs.bases.nbytes + seqs.offsets.nbytes +
                                          seqs.ids.nbytes),
                "d2h_bytes_per_step": int(nrows * abi.OVERLAP_DTYPE.itemsize)},
        "gpu_launches": int(round(launches_step * args.steps)),
        "stages_ms_per_step": {n: round(float(stage_tot[i]) / args.steps, 3)
                               for i, n in enumerate(names + ["output + D2H", "H2D"])},
        "sort_paths_per_step": sort_paths,
        "stage_rooflines": stage_rooflines(names, stage_tot, bytes_tot, peak),
        "roofline": {"bound": "hbm", "stage": names[dom], "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if peak else None,
                     "traffic": traffic,
                     "traffic_unit": "DRAM bytes per step of the stage's kernels (ncu bytes per "
                                     "hit from profiles/ncu_traffic.json x hits per step)",
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"
                     if peak else "missing"},
        "clocks": clocks,
    }
    if args.query_sample > 0:
        line["config"]["query_sample"] = int(mine.n)
    if args.emission_mode >= 0:
        line["config"]["emission_mode"] = args.emission_mode
    if plain:
        line["plain"] = plain
        lat_ms = sorted(1000 * x for x in lat)
        line["latency_ms"] = {"p50": lat_ms[len(lat_ms) // 2],
                              "p99": lat_ms[min(len(lat_ms) - 1, int(0.99 * len(lat_ms)))],
                              "mode": "plain path, one read per call through the C ABI"}
    if cpu:
        line["cpu_baseline"] = cpu
        line["parity"] = parity
    line["launch_shape"] = {"shape": gpu.launch_shape(), "autotune": tune}
    gpu.close()
    if args.configs and world == 1:
        line["configs"] = extra_configs(args, local)
    if args.serve_rates and world == 1:
        line["serving"] = serving_run(args, local)
    print(json.dumps(line), flush=True)


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--seed", type=int, default=2)
    ap.add_argument("--genome-len", type=int, default=5_000_000)
    ap.add_argument("--coverage", type=float, default=40.0)
    ap.add_argument("--plain-sample", type=int, default=2000)
    ap.add_argument("--cpu-sample", type=int, default=2000,
                    help="reads of the CPU baseline, also compared row for row with the GPU")
    ap.add_argument("--reference-sample", type=int, default=400,
                    help="reads per step of --impl reference (each step takes the next ones)")
    ap.add_argument("--serve-rates", type=lambda v: [float(x) for x in v.split(",") if x],
                    default=[1000.0, 10000.0, 50000.0],
                    help="offered request rates (reads/s) of the serving run; empty skips it")
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--clock-log", default="",
                    help="where the nvidia-smi clock samples of the timed region go "
                         "({rank} is replaced); default /tmp")
    ap.add_argument("--configs", default="1,3,5",
                    help="other configurations to measure (1: plain 1 Mb, 3: read-to-graph, "
                         "5: scale, at --scale-genome); empty to skip")
    ap.add_argument("--scale-genome", type=int, default=500_000_000,
                    help="genome length of config 5 (the configuration's 500 Mb by default; "
                         "smaller values scale its memory budget too)")
    ap.add_argument("--config-plain-sample", type=int, default=2000)
    ap.add_argument("--serve-workers", type=int, default=2)
    ap.add_argument("--serve-batch-bases", type=int, default=32_000_000,
                    help="most read bases one served batch takes")
    ap.add_argument("--query-sample", type=int, default=0,
                    help="time only this many reads (the first) as queries against the "
                         "index of all reads, for profiling cases (0: all)")
    ap.add_argument("--emission-mode", type=int, default=-1, choices=[-1, 0, 1, 2],
                    help="cuflye_set_sorted_emission mode for the timed calls (-1: the "
                         "library's default)")
    ap.add_argument("--autotune", type=int, default=1500,
                    help="reads in the autotuner's sample, run before the timed steps "
                         "(0: the default launch shape)")
    args = ap.parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
