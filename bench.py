#!/usr/bin/env python3
"""INLJ probe benchmark on GB300 (one JSON line on stdout).

Default workload (the headline): an index-nested-loop join of 2^28 probe keys
drawn Zipf(theta=0.5) with permuted ranks from a 2^26-key uniform build
column (keys in [0, 2^63)), through a 64-key-node B+tree, emitting
(probe row, build position) pairs.  Harmonia, RadixSpline, binary search
and the learned index are measured on the same probes and reported per index.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload inlj|partitioned|star|learned|batch]

A step is one pass of the probe path over the whole probe column.  Inputs
(2 GiB of probes) are larger than the 126 MB L2, so no flush is needed
between steps.  For N > 1 (torchrun) every rank runs the same workload on its
own GPU (independent replicas, no collective on the data path) and the
timing is the max over ranks.

--impl reference times the reference's CPU lookup path (the B+tree
restated in oracle/, the reference's page geometry) on the host cores with
all threads, on a bounded sample of the same workload.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 126 * 1024 * 1024
FALLBACK_HBM_GBS = 6800.0


# ---------------------------------------------------------------------------
# distributed helpers (also exercised by tests with the gloo backend)
# ---------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init_dist(backend: str):
    import torch.distributed as dist

    world, rank, _ = dist_env()
    if world > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend, rank=rank, world_size=world)
    return world, rank


def barrier(world: int, device=None):
    if world > 1:
        import torch.distributed as dist

        if device is not None and device.type == "cuda":
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


def max_over_ranks(value: float, world: int, device=None) -> float:
    """Largest value over all ranks (timing = slowest rank)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []
        self.reader = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.reader:
            self.reader.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, flag in zip(names, parts[5:9]):
                if flag.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def profile_traffic(kernel_tag: str):
    """DRAM bytes per launch from a committed ncu summary (profiles/traffic.txt)."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        with open(path) as f:
            for ln in f:
                ln = ln.strip()
                if ln.startswith(kernel_tag + " "):
                    return float(ln.split()[1])
    except OSError:
        pass
    return None


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def time_steps(fn, steps: int, warmup: int, stream, world: int, device):
    """Run warmup untimed steps, then time exactly `steps` steps with CUDA
    events on `stream`, bracketed by barrier + synchronize; returns ms."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    barrier(world, device)
    torch.cuda.synchronize()
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for _ in range(steps):
        fn()
    end.record(stream)
    torch.cuda.synchronize()
    barrier(world, device)
    torch.cuda.synchronize()
    return start.elapsed_time(end)


def cpu_baseline_btree(h_keys, h_probes, sample: int):
    """The reference's CPU B+tree lookup (oracle restatement, 247/246 page
    geometry) on a bounded sample, all host threads."""
    import numpy as np

    import oracle

    threads = oracle.hardware_threads()
    tree = oracle.BTree(h_keys, 247, 246)
    pr = np.ascontiguousarray(h_probes[:sample])
    tree.lookup(pr[: min(len(pr), 1 << 16)], threads)  # warm
    t0 = time.perf_counter()
    out = tree.lookup(pr, threads)
    dt = time.perf_counter() - t0
    del out
    return {"value": len(pr) / dt, "unit": "probe tuples/s", "cores": threads, "kind": "port",
            "sample": f"{len(pr)} probes of the same Zipf column into the same {len(h_keys)}-key column "
                      f"(oracle B+tree, reference page geometry 247/246), {threads} threads, {dt:.2f} s"}


def gpu_main(args):
    import numpy as np
    import torch

    import gpujoin_gb300 as gj

    world, rank, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        init_dist("nccl")
    device = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(device)
    stream = torch.cuda.current_stream(device)

    n, m = 1 << args.n_log2, 1 << args.m_log2
    keys = gj.generate_sorted_keys(n, gj.DIST_UNIFORM, 1 << 63, seed=args.seed)
    probes = gj.generate_probes(keys, m, theta=args.theta, seed=args.seed + 1)
    torch.cuda.synchronize()

    kinds = [k.strip() for k in args.indexes.split(",") if k.strip()]
    per_index = {}
    headline_ms = None
    pairs = torch.empty(2 * m, dtype=torch.int32, device=device)
    count = torch.zeros(1, dtype=torch.int64, device=device)
    ws_size = __import__("ctypes").c_size_t(0)
    gj.lib().gj_inlj_pairs_workspace_size(m, __import__("ctypes").byref(ws_size))
    ws = torch.empty(ws_size.value, dtype=torch.uint8, device=device)
    headline_index = None
    bytes_per_probe = 8 + 8 + (32 if 8 * n > L2_BYTES else 0)
    clocks = None
    for kind in kinds:
        t_build = time.perf_counter()
        ix = gj.make_index(kind).construct(None, keys)
        torch.cuda.synchronize()
        t_build = time.perf_counter() - t_build

        def step():
            ix.inlj_pairs(probes, pairs, count, ws)

        sampler = None
        if headline_index is None:
            sampler = ClockSampler(device.index)
            sampler.start()
        ms = time_steps(step, args.steps, args.warmup, stream, world, device)
        if sampler is not None:
            clocks = sampler.stop()
        ms = max_over_ranks(ms, world, device)
        got = int(count.item())
        per_index[kind] = {"tuples_per_s": world * m * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                           "pairs": got, "build_s": round(t_build, 3), "index_bytes": ix.memory_consumption()}
        if headline_index is None:
            headline_index, headline_ms, headline_ix = kind, ms, ix
        else:
            ix.free()

    # end-to-end through the public API with host buffers (pinned), headline index
    h_probes = probes.cpu().pin_memory() if args.e2e else None
    e2e = None
    if args.e2e:
        h_pairs = torch.empty(2 * m, dtype=torch.int32).pin_memory()
        d_in = torch.empty_like(probes)

        def e2e_step():
            d_in.copy_(h_probes, non_blocking=True)
            headline_ix.inlj_pairs(d_in, pairs, count, ws)
            h_pairs.copy_(pairs, non_blocking=True)

        e_ms = time_steps(e2e_step, max(2, args.steps // 2), 1, stream, world, device)
        e_ms = max_over_ranks(e_ms, world, device)
        e_steps = max(2, args.steps // 2)
        e2e = {"value": world * m * e_steps / (e_ms / 1e3), "unit": "probe tuples/s", "h2d_bytes_per_step": 8 * m,
               "d2h_bytes_per_step": 8 * m}

    peak, peak_kind = measured_peak()
    per_launch_ms = headline_ms / args.steps
    achieved = bytes_per_probe * m / (per_launch_ms / 1e3) / 1e9
    traffic = profile_traffic(f"inlj_pairs_{headline_index}_n{args.n_log2}_m{args.m_log2}")
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_source": f"{peak_kind} hbm_gbs (copy, burst)",
                "bytes_per_probe": bytes_per_probe}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        h_keys = keys.cpu().numpy().view(np.uint64)
        hp = probes[: args.cpu_sample].cpu().numpy().view(np.uint64)
        cpu = cpu_baseline_btree(h_keys, hp, args.cpu_sample)

    value = per_index[headline_index]["tuples_per_s"]
    line = {
        "metric": f"INLJ probe tuples/s ({headline_index}, 1 GB300 per rank), % of HBM roofline",
        "value": value,
        "unit": "probe tuples/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": headline_ms / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic (seeded device generators)",
        "config": {"workload": f"INLJ pairs: {n} uniform uint64 build keys (2^{args.n_log2}), {m} Zipf(theta="
                               f"{args.theta}) probes (2^{args.m_log2}), permuted ranks, index {headline_index}",
                   "index": headline_index, "build_keys": n, "probes": m, "zipf_theta": args.theta,
                   "output": "(probe row u32, build pos u32) pairs", "l2": "inputs larger than L2 (no flush)",
                   "parallelism": f"replicas x{world}"},
        "per_index": per_index,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": args.steps,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU lookup path on the host cores
# ---------------------------------------------------------------------------
def reference_main(args):
    import numpy as np

    import oracle

    world, rank, _ = dist_env()
    if rank != 0:
        return
    n, m = 1 << args.n_log2, 1 << args.m_log2
    rng = np.random.default_rng(args.seed)
    keys = np.unique(rng.integers(0, 1 << 63, size=n + n // 64, dtype=np.uint64))
    keys = np.sort(rng.choice(keys, size=n, replace=False)) if len(keys) > n else keys
    threads = oracle.hardware_threads()
    sample = min(args.cpu_sample, m)
    probes = oracle.zipf_probes(keys, sample, args.theta, args.seed + 1, threads)
    tree = oracle.BTree(keys, 247, 246)
    for _ in range(args.warmup):
        tree.lookup(probes[: sample // 8], threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        tree.lookup(probes, threads)
    dt = time.perf_counter() - t0
    value = sample * args.steps / dt
    line = {
        "impl": "reference",
        "metric": "INLJ probe tuples/s (btree, 1 GB300 per rank), % of HBM roofline",
        "value": value,
        "unit": "probe tuples/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic (seeded numpy build column, oracle Zipf probes)",
        "config": {"workload": f"INLJ: {n} uniform uint64 build keys (2^{args.n_log2}), Zipf(theta={args.theta}) "
                               f"probes; each step a bounded sample of {sample} of the {m} probes",
                   "index": "btree", "build_keys": n, "probes": m, "zipf_theta": args.theta},
        "cpu_baseline": {"value": value, "unit": "probe tuples/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} probes per step, B+tree with the reference page geometry "
                                   f"(247/246), restated in oracle/oracle.c, {threads} threads"},
        "e2e": {"value": value, "unit": "probe tuples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=["inlj"], default="inlj")
    ap.add_argument("--n-log2", type=int, default=26)
    ap.add_argument("--m-log2", type=int, default=28)
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--indexes", default="btree,harmonia,radix_spline,binary_search,learned")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--cpu-sample", type=int, default=1 << 22)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    return ap.parse_args(argv)


def main(argv=None):
    args = parse_args(argv)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_main(args)
    else:
        gpu_main(args)


if __name__ == "__main__":
    main()
