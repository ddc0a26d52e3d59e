#!/usr/bin/env python3
"""INLJ probe benchmark on GB300 (one JSON line on stdout).

Default workload (the headline): an index-nested-loop join of 2^28 probe keys
drawn Zipf(theta=0.5) with permuted ranks from a 2^26-key uniform build
column (keys in [0, 2^63)), through the library's default B+tree (inner
nodes of one 32-byte sector, 15 delta-coded separators; leaves of one
sector of the column), emitting (probe row, build position) pairs.  The
B+tree with 64-key uint64 inner nodes (btree_w64, the reference's node
width), Harmonia, RadixSpline, binary search, the learned index and the hash
index are measured on the same probes and reported per index; for the
B+tree, binary search and Harmonia the reference's own device lookups
(compiled from its headers into oracle/_ref/refgpu.cubin, launched as its
lookup_kernel) are timed beside this library's lookup on the same data.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload inlj|partitioned|star|learned|batch]

A step is one pass of the probe path over the whole probe column.  Inputs
(2 GiB of probes) are larger than the L2, so no flush is needed
between steps.  For N > 1 (torchrun) every rank runs the same workload on its
own GPU (independent replicas, no collective on the data path) and the
timing is the max over ranks.

The default line also carries "configurations", the other configurations of the
measurement, each checked against the oracle: the B+tree at Zipf theta 0 and
1.0, the partitioned INLJ (2^29 probes into 2^28 keys), the learned index
beside binary search and RadixSpline (2^27 keys, three distributions), the
star-join aggregate and the CPU lookup at 1 and all host threads
(--no-extras leaves them out).

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
ROOT_NAMES = {0: "linear", 1: "mlp", 3: "segments"}  # learned-index root kinds


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


def reference_gpu_lookup(ref, kind, ix, keys, h_keys, probes, out, expect, steps, warmup, stream, world, device):
    """Times the reference's own device lookup of `kind` (oracle/ref_gpu.py:
    its binary_search_index / btree / harmonia_tree lookups compiled from its
    headers) and this library's lookup (gj_index_lookup, the same u32
    positions; for binary search and Harmonia also the warp-collective
    gj_index_lookup_cooperative with the reference's 16-lane groups) on the
    same index data and probes; every output is compared with the oracle's
    positions."""
    import torch

    import gpujoin_gb300 as gj
    from oracle import ref_gpu

    m = probes.numel()
    if kind == "harmonia":
        view, keep = ref.padded_harmonia(ref_gpu.harmonia_view(gj, ix))
        run_ref = lambda: ref.harmonia(view, probes, out, stream)  # noqa: E731
    elif kind == "btree":
        # the reference's own tree (246-separator 4 KB pages, 247-key leaves)
        # over the same column
        root, keep = ref.btree_pages(keys, h_keys)
        run_ref = lambda: ref.btree(root, keys, probes, out, stream)  # noqa: E731
    else:
        run_ref = lambda: ref.binary_search(keys, probes, out, stream)  # noqa: E731
    res = {}
    arms = [("reference_kernel", run_ref), ("gb300_lookup", lambda: ix.lookup(probes, out=out))]
    if kind in ("harmonia", "binary_search"):
        # the same warp-collective protocol as the reference's (16-lane groups)
        arms.append(("gb300_warp_cooperative_16", lambda: ix.lookup_cooperative(probes, 4, out=out)))
    for arm, fn in arms:
        out.fill_(0)
        ms = max_over_ranks(time_steps(fn, steps, warmup, stream, world, device), world, device)
        mism = None
        if expect is not None:
            mism = int((out != expect).sum().item())
        res[arm] = {"tuples_per_s": world * m * steps / (ms / 1e3), "ms_per_step": ms / steps, "mismatches": mism}
    res["speedup"] = round(res["gb300_lookup"]["tuples_per_s"] / res["reference_kernel"]["tuples_per_s"], 2)
    torch.cuda.synchronize()
    return res


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


# ---------------------------------------------------------------------------
# parity against the oracle, outside every timed region
# ---------------------------------------------------------------------------
def oracle_positions(h_keys, h_probes):
    """(lower bound, exact) oracle positions of every probe, all host threads
    (the oracle's B+tree restatement; equal to its binary search)."""
    import oracle

    return oracle.fast_positions(h_keys, h_probes, oracle.hardware_threads())


def check_pairs(pairs, count, expect, ordered=True):
    """Compare GPU join pairs with the oracle's positions per probe row
    (expect: int32 device tensor, -1 = no match).  ordered: pairs in probe
    order; otherwise as a set (partitioned pairs).  Device-side compare."""
    import torch

    got = int(count.item())
    rows = torch.nonzero(expect != -1).squeeze(1)
    n_exp = rows.numel()
    if got != n_exp:
        return {"checked": n_exp, "mismatches": max(abs(got - n_exp), 1), "count": got, "expected_count": n_exp}
    p = pairs[: 2 * got].view(-1, 2)
    if ordered:
        bad = int(((p[:, 0].long() != rows) | (p[:, 1] != expect[rows])).sum())
    else:
        by_row = torch.full_like(expect, -1)
        by_row[p[:, 0].long()] = p[:, 1]
        bad = int((by_row != expect).sum())
    return {"checked": got, "mismatches": bad}


def check_pairs_sample(pairs, count, m, h_keys, h_probes, sample, seed, semantics="exact"):
    """Partitioned pairs of m probes against the oracle on a seeded sample of
    probe rows (plus the pair count): the pairs are gathered by row on the
    device, the oracle searches the sampled rows on the host."""
    import numpy as np
    import torch

    import oracle

    got = int(count.item())
    p = pairs[: 2 * got].view(-1, 2)
    by_row = torch.full((m,), -1, dtype=torch.int32, device=pairs.device)
    by_row[p[:, 0].long()] = p[:, 1]
    rng = np.random.default_rng(seed)
    rows = rng.integers(0, m, size=min(sample, m))  # with replacement: a row drawn twice is checked twice
    lb, ex = oracle.fast_positions(h_keys, h_probes[rows], oracle.hardware_threads())
    want = (ex if semantics == "exact" else lb).view(np.int32)
    have = by_row[torch.from_numpy(rows).to(pairs.device)].cpu().numpy()
    matched_rows = int((by_row != -1).sum())
    return {"checked": int(len(rows)), "mismatches": int(np.count_nonzero(have != want)), "count": got,
            "rows_with_a_pair": matched_rows, "sample": f"{len(rows)} seeded probe rows of {m} + the pair count"}


EXACT_KINDS = ("btree", "harmonia", "hash")  # position of an equal key, else none


def index_params(args, kind):
    """Build parameters given on the command line for an index kind."""
    p = {}
    if kind == "btree":
        if args.btree_node_keys:
            p["btree_node_keys"] = args.btree_node_keys
        if args.btree_leaf_keys:
            p["btree_leaf_keys"] = args.btree_leaf_keys
        if args.btree_start_bits:
            p["btree_start_bits"] = args.btree_start_bits
    if kind == "harmonia" and args.btree_start_bits:
        p["btree_start_bits"] = args.btree_start_bits  # Harmonia's start table shares the parameter
    return p


def gpu_setup():
    import torch

    world, rank, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        init_dist("nccl")
    device = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(device)
    return world, rank, device, torch.cuda.current_stream(device)


def gpu_main(args):
    world, rank, device, stream = gpu_setup()
    fn = {"inlj": inlj_workload, "partitioned": partitioned_workload, "star": star_workload,
          "learned": learned_workload, "batch": batch_workload, "host_index": host_index_workload,
          "orderings": orderings_workload}[args.workload]
    line = fn(args, world, rank, device, stream)
    if rank == 0:
        print(json.dumps(line), flush=True)


def random_sector_rate(device, stream, n_sectors=1 << 26, loads=1 << 28, reps=5):
    """Random 32-byte sector reads per second over a 2 GiB buffer (larger than
    L2), CUDA events, best of reps, with the default L2 fill and with the
    64-byte fill the probe kernels' scattered loads ask for
    (gj_calibrate_random_sectors)."""
    import ctypes

    import torch

    import gpujoin_gb300 as gj

    buf = torch.randint(0, 1 << 62, (4 * n_sectors,), dtype=torch.int64, device=device)
    words = ctypes.c_uint64(0)
    gj._check(gj.lib().gj_calibrate_sink_words(ctypes.byref(words)))
    sink = torch.empty(words.value, dtype=torch.int64, device=device)
    out = {"buffer_bytes": 32 * n_sectors, "loads": loads}
    for fill64, name in ((0, "default_fill"), (1, "fill_64B")):
        best = None
        for r in range(reps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            gj._check(gj.lib().gj_calibrate_random_sectors(buf.data_ptr(), n_sectors, loads, 12345 + r, fill64,
                                                          sink.data_ptr(), stream.cuda_stream))
            b.record(stream)
            torch.cuda.synchronize()
            t = a.elapsed_time(b)
            if r and (best is None or t < best):
                best = t
        out[name] = {"sectors_per_s": loads / (best / 1e3), "ms": round(best, 3)}
    del buf, sink
    torch.cuda.empty_cache()
    return out


def cpu_baselines(h_keys, h_probes, one_sample, all_sample):
    """The reference's CPU lookup paths (restated in oracle/oracle.c, pinned
    to the reference's own headers by the golden fixtures) on the host cores:
    std::lower_bound (binary_search_index's semantics), the branch-free lower
    bound (src/bf_search.cpp:34-47), Harmonia's host lookup
    (src/harmonia.cuh:640-668) and the clustered B+tree with the reference's
    page geometry -- each at 1 thread (as the reference runs them,
    src/tpch/cpu_bench.cpp:31,37) and at all host threads, on bounded samples
    of the same probes."""
    import oracle

    threads = oracle.hardware_threads()
    bt = oracle.BTree(h_keys, 247, 246)
    hm = oracle.Harmonia(h_keys)
    methods = (("lower_bound", lambda pr, t: oracle.bs_lookup(h_keys, pr, t)),
               ("branch_free_lower_bound", lambda pr, t: oracle.bs_lookup(h_keys, pr, t, branch_free=True)),
               ("harmonia", lambda pr, t: hm.lookup(pr, t)),
               ("btree", lambda pr, t: bt.lookup(pr, t)))
    out = {"cores": threads, "kind": "port", "unit": "probe tuples/s"}
    for name, f in methods:
        row = {}
        for t, sample in ((1, one_sample), (threads, all_sample)):
            pr = h_probes[:sample]
            f(pr[:4096], t)  # warm
            t0 = time.perf_counter()
            f(pr, t)
            dt = time.perf_counter() - t0
            row[f"threads_{t}"] = {"value": len(pr) / dt, "probes": int(len(pr)), "seconds": round(dt, 3)}
        out[name] = row
    return out


def other_configurations(args, world, device, stream, keys, h_keys, h_probes):
    """The other configurations of the INLJ measurement, each checked against
    the oracle: the same B+tree at Zipf theta 0 and 1.0; the partitioned INLJ
    of 2^29 Zipf(0.5) probes into a 2^28-key index (autotuned fanout), and on
    the headline's 2^26 keys and 2^28 probes; the
    learned index against binary search and RadixSpline (2^27 keys x three
    distributions, 2^28 probes with 5% absent keys); the star-join aggregate;
    and the reference's CPU lookup paths at 1 and all host threads."""
    import numpy as np
    import torch

    import gpujoin_gb300 as gj
    import oracle

    extras = {}
    n, m = keys.numel(), h_probes.shape[0]
    steps = max(3, min(args.steps, args.extra_steps))

    t0 = time.perf_counter()
    per_theta = {}
    ix = gj.btree_index().construct(None, keys)
    pairs = torch.empty(2 * m, dtype=torch.int32, device=device)
    count = torch.zeros(1, dtype=torch.int64, device=device)
    import ctypes

    wsz = ctypes.c_size_t(0)
    gj.lib().gj_inlj_pairs_workspace_size(m, ctypes.byref(wsz))
    ws = torch.empty(wsz.value, dtype=torch.uint8, device=device)
    for theta in (0.0, 1.0):
        probes = gj.generate_probes(keys, m, theta=theta, seed=args.seed + 1)
        ms = time_steps(lambda: ix.inlj_pairs(probes, pairs, count, ws), steps, args.warmup, stream, world, device)
        parity = None
        if not args.no_parity:
            parity = check_pairs_sample(pairs, count, m, h_keys, probes.cpu().numpy().view(np.uint64),
                                        args.parity_sample, args.seed + 9, "exact")
        per_theta[str(theta)] = {"tuples_per_s": m * steps / (ms / 1e3), "ms_per_step": ms / steps,
                                 "pairs": int(count.item()), "parity": parity}
        del probes
    ix.free()
    del pairs, ws
    torch.cuda.empty_cache()
    extras["per_theta"] = dict(per_theta, index="btree (default build)", theta_0_5="the headline",
                               seconds=round(time.perf_counter() - t0, 1))

    t0 = time.perf_counter()
    extras["partitioned"] = partitioned_measure(args, world, device, stream, 28, 29, steps, "btree")
    extras["partitioned"]["seconds"] = round(time.perf_counter() - t0, 1)

    # the partitioned INLJ on the headline's data (2^26 keys, 2^28 Zipf(0.5)
    # probes): the same set of pairs as the headline, grouped by partition
    # tile instead of in probe order
    t0 = time.perf_counter()
    extras["partitioned_headline_data"] = partitioned_measure(args, world, device, stream, 26, 28, steps, "btree",
                                                              sample_clocks=False)
    extras["partitioned_headline_data"]["seconds"] = round(time.perf_counter() - t0, 1)

    t0 = time.perf_counter()
    results, parity = learned_measure(args, world, device, stream, 27, 28, 3, quick=True)
    extras["learned"] = {"results": results, "parity": parity, "seconds": round(time.perf_counter() - t0, 1),
                         "config": "2^27 keys x {uniform, lognormal(0,2) x 2^60, 1024 clusters}, 2^28 probes "
                                   "(5% absent), 3 timed steps each"}

    t0 = time.perf_counter()
    n_fact, n_dim, lo, hi = 6_000_000, 200_000, 1000, 1030
    dim_keys, flag, fk, date, price, disc = star_inputs(n_fact, n_dim, args.seed, device)
    six = gj.btree_index().construct(None, dim_keys)
    sout = torch.zeros(2, dtype=torch.int64, device=device)
    ms = time_steps(lambda: gj.star_join_sum(six, fk, date, price, disc, flag, lo, hi, sout), steps, args.warmup,
                    stream, world, device)
    got = sout.cpu().numpy()
    h = [t.cpu().numpy() for t in (fk, date, price, disc, dim_keys, flag)]
    c0 = time.perf_counter()
    num, den = oracle.star_join(h[0].view(np.uint32), h[1].view(np.uint32), h[2], h[3], h[4].view(np.uint64), h[5],
                                lo, hi)
    cpu_s = time.perf_counter() - c0
    sout2 = torch.zeros(2, dtype=torch.int64, device=device)
    ms_sorted = time_steps(lambda: gj.star_join_sum(six, fk, date, price, disc, flag, lo, hi, sout2,
                                                    sorted_batches=True), steps, args.warmup, stream, world, device)
    got2 = sout2.cpu().numpy()
    extras["star"] = {"fact_rows_per_s": n_fact * steps / (ms / 1e3), "latency_us": ms / steps * 1e3,
                      "sums": [int(got[0]), int(got[1])], "oracle_sums": [num, den],
                      "exact": bool(int(got[0]) == num and int(got[1]) == den),
                      "sorted_batches": {"fact_rows_per_s": n_fact * steps / (ms_sorted / 1e3),
                                         "latency_us": ms_sorted / steps * 1e3,
                                         "exact": bool(int(got2[0]) == num and int(got2[1]) == den),
                                         "order": "gj_star_join_sum_sorted (ij_pbws: buffered, key-sorted batches)"},
                      "cpu_query_14_part_build_1_thread_rows_per_s": n_fact / cpu_s,
                      "config": "6M fact rows, 200k dimension rows (B+tree), 30-day window of 2556 days"}
    six.free()

    t0 = time.perf_counter()
    extras["cpu_baselines"] = cpu_baselines(h_keys, h_probes, args.cpu_one_sample, args.cpu_all_sample)
    extras["cpu_baselines"]["seconds"] = round(time.perf_counter() - t0, 1)
    return extras


def inlj_workload(args, world, rank, device, stream):
    import numpy as np
    import torch

    import gpujoin_gb300 as gj

    n, m = 1 << args.n_log2, 1 << args.m_log2
    keys = gj.generate_sorted_keys(n, gj.DIST_UNIFORM, 1 << 63, seed=args.seed)
    probes = gj.generate_probes(keys, m, theta=args.theta, seed=args.seed + 1)
    torch.cuda.synchronize()

    kinds = [k.strip() for k in args.indexes.split(",") if k.strip()]
    per_index = {}
    # oracle positions of every probe (host threads, outside the timed
    # regions), on the device for the comparisons
    # (rank 0 only: the replicas' inputs are the same)
    h_keys = keys.cpu().numpy().view(np.uint64)
    h_probes = probes.cpu().numpy().view(np.uint64)
    expect, oracle_s = None, 0.0
    if rank == 0 and not args.no_parity:
        t_or = time.perf_counter()
        lb, ex = oracle_positions(h_keys, h_probes)
        expect = {"lower_bound": torch.from_numpy(lb.view(np.int32)).to(device),
                  "exact": torch.from_numpy(ex.view(np.int32)).to(device)}
        del lb, ex
        oracle_s = time.perf_counter() - t_or
    headline_ms = None
    pairs = torch.empty(2 * m, dtype=torch.int32, device=device)
    count = torch.zeros(1, dtype=torch.int64, device=device)
    ws_size = __import__("ctypes").c_size_t(0)
    gj.lib().gj_inlj_pairs_workspace_size(m, __import__("ctypes").byref(ws_size))
    ws = torch.empty(ws_size.value, dtype=torch.uint8, device=device)
    headline_index = None
    ref_kernels = None
    bytes_per_probe = 8 + 8 + (32 if 8 * n > L2_BYTES else 0)
    clocks = None
    for entry in kinds:
        # "btree_w64": the B+tree with 64-key uint64 inner nodes (the node
        # width of the INLJ configuration as written)
        kind, params = entry, index_params(args, entry)
        if entry == "btree_w64":
            kind, params = "btree", {"btree_node_keys": 64}
        t_build = time.perf_counter()
        ix = gj.make_index(kind, **params).construct(None, keys)
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
        sem = "exact" if kind in EXACT_KINDS else "lower_bound"
        if kind == "no_op":
            sem = None
        parity = None
        if expect is not None:
            parity = check_pairs(pairs, count, expect[sem]) if sem else {"checked": m, "mismatches": int(got != 0)}
        per_index[entry] = {"tuples_per_s": world * m * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                            "pairs": got, "build_s": round(t_build, 3), "index_bytes": ix.memory_consumption(),
                            "params": params or "default build",
                            "parity": dict(parity, semantics=sem, oracle="all probes") if parity else None}
        if (entry in ("btree", "harmonia", "binary_search") and rank == 0 and world == 1
                and not args.no_reference_gpu):
            # the reference's own device lookup on the same index data
            try:
                if ref_kernels is None:
                    from oracle import ref_gpu

                    ref_kernels = ref_gpu.ReferenceKernels()
                per_index[entry]["reference_gpu"] = reference_gpu_lookup(
                    ref_kernels, kind, ix, keys, h_keys, probes, pairs[m:], None if expect is None else expect[sem],
                    max(3, min(args.steps, args.extra_steps)), args.warmup, stream, world, device)
            except (OSError, RuntimeError) as e:
                per_index[entry]["reference_gpu"] = {"unavailable": str(e)}
        if headline_index is None:
            headline_index, headline_ms, headline_ix = kind, ms, ix
        else:
            ix.free()

    # End to end through the public API with host buffers (pinned): the
    # host-buffer entry point reads the probes from host memory and writes
    # the pairs and their count back inside its kernels (NVLink-C2C), so every
    # step moves 8 B per probe to the device and 8 B per pair back.  For
    # comparison, the explicit-copy form: pinned copy in, device call, copy out.
    e2e = None
    if args.e2e:
        h_probes = probes.cpu().pin_memory()
        h_pairs = torch.empty(2 * m, dtype=torch.int32).pin_memory()
        h_count = torch.zeros(1, dtype=torch.int64).pin_memory()
        hw = __import__("ctypes").c_size_t(0)
        gj.lib().gj_inlj_pairs_host_workspace_size(m, __import__("ctypes").byref(hw))
        hws = torch.empty(hw.value, dtype=torch.uint8, device=device)
        e_steps = max(2, args.steps // 2)
        e_ms = time_steps(lambda: headline_ix.inlj_pairs_host(h_probes, h_pairs, h_count, hws), e_steps, args.warmup, stream,
                          world, device)
        e_ms = max_over_ranks(e_ms, world, device)
        assert int(h_count[0]) == per_index[headline_index]["pairs"]
        d_in = torch.empty_like(probes)

        def copy_step():
            d_in.copy_(h_probes, non_blocking=True)
            headline_ix.inlj_pairs(d_in, pairs, count, ws)
            h_pairs.copy_(pairs, non_blocking=True)

        c_ms = time_steps(copy_step, e_steps, args.warmup, stream, world, device)
        c_ms = max_over_ranks(c_ms, world, device)
        # the same pairs in the order their tiles finish (no tile waits for
        # its predecessors' counts), checked as a set against the oracle;
        # and the same from device buffers (gj_inlj_pairs_unordered)
        u_ms = time_steps(lambda: headline_ix.inlj_pairs_host(h_probes, h_pairs, h_count, hws, ordered=False),
                          e_steps, args.warmup, stream, world, device)
        u_ms = max_over_ranks(u_ms, world, device)
        u_count = int(h_count[0])
        assert u_count == per_index[headline_index]["pairs"]
        u_parity = None
        if expect is not None:
            d_p = h_pairs[: 2 * u_count].to(device).view(-1, 2)
            by_row = torch.full((m,), -1, dtype=torch.int32, device=device)
            by_row[d_p[:, 0].long()] = d_p[:, 1]
            sem = "exact" if headline_index in EXACT_KINDS else "lower_bound"
            u_parity = {"checked": m, "mismatches": int((by_row != expect[sem]).sum().item()),
                        "semantics": sem + ", pairs as a set (rows placed by row id)"}
            del d_p, by_row
        d_ms = time_steps(lambda: headline_ix.inlj_pairs(probes, pairs, count, ws, ordered=False), args.steps,
                          args.warmup, stream, world, device)
        d_ms = max_over_ranks(d_ms, world, device)
        d_count = int(count.item())
        d_parity = None
        if expect is not None:
            d_p = pairs[: 2 * d_count].view(-1, 2)
            by_row = torch.full((m,), -1, dtype=torch.int32, device=device)
            by_row[d_p[:, 0].long()] = d_p[:, 1]
            d_parity = {"checked": m, "mismatches": int((by_row != expect[sem]).sum().item())}
            del d_p, by_row
        e2e = {"value": world * m * e_steps / (e_ms / 1e3), "unit": "probe tuples/s", "h2d_bytes_per_step": 8 * m,
               "d2h_bytes_per_step": 8 * m + 8, "api": "gj_inlj_pairs_host (pinned host probes, pairs and count)",
               "explicit_copies_value": world * m * e_steps / (c_ms / 1e3),
               "unordered": {"value": world * m * e_steps / (u_ms / 1e3),
                             "api": "gj_inlj_pairs_host_unordered (the same pairs, tiles in the order they finish)",
                             "pairs": u_count, "parity": u_parity,
                             "device_buffers": {"value": world * m * args.steps / (d_ms / 1e3),
                                                "ms_per_step": d_ms / args.steps,
                                                "api": "gj_inlj_pairs_unordered (device buffers)",
                                                "pairs": d_count, "parity": d_parity}}}

    # Roofline of the dominant kernel.  A pairs step is two launches: the
    # search pass (k_lookup: probe key in, one 32-byte leaf sector, u32
    # position out to the upper half of the pairs buffer) and the ordered
    # compaction (u32 in, 8-byte pair out).  The search pass is timed on its
    # own here -- the same kernel on the same probes and output location, CUDA
    # events on the same stream; its algorithmic bytes are 8 + 32 + 4 per probe.
    peak, peak_kind = measured_peak()
    lookup_bytes_per_probe = bytes_per_probe - 4
    lookup_ms = time_steps(lambda: headline_ix.lookup(probes, out=pairs[m:]), args.steps, args.warmup, stream, world,
                           device)
    lookup_ms = max_over_ranks(lookup_ms, world, device) / args.steps
    achieved = lookup_bytes_per_probe * m / (lookup_ms / 1e3) / 1e9
    traffic = profile_traffic(f"k_lookup_{headline_index}_n{args.n_log2}_m{args.m_log2}")
    step_ms = headline_ms / args.steps
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_source": f"{peak_kind} hbm_gbs (copy, burst)",
                "kernel": f"k_lookup<{headline_index}> (search pass of the pairs step)",
                "kernel_ms": round(lookup_ms, 4), "kernel_share_of_step": round(lookup_ms / step_ms, 3),
                "bytes_per_probe": lookup_bytes_per_probe,
                "step_bytes_per_probe": bytes_per_probe,
                "step_achieved": round(bytes_per_probe * m / (step_ms / 1e3) / 1e9, 1)}
    # index path: the L2 sectors the search pass reads per probe (ncu,
    # lts__t_sectors_srcunit_tex_op_read at 2^24 probes of the same index),
    # times 32 B, over the live kernel time
    l2_sectors = profile_traffic(f"l2_read_sectors_per_probe_k_lookup_{headline_index}_n{args.n_log2}")
    if l2_sectors:
        path_gbs = l2_sectors * 32 * m / (lookup_ms / 1e3) / 1e9
        roofline["index_path"] = {"l2_sectors_per_probe": l2_sectors, "bytes_per_probe": round(l2_sectors * 32, 1),
                                  "l2_to_sm_gbs": round(path_gbs, 1),
                                  "note": "L2-to-SM bytes of the search pass (ncu sectors x 32 B over the live "
                                          "kernel time); most index reads are L2 hits"}
    # the second roofline of scattered probes: each needs at least one random
    # 32-byte sector of a column larger than L2, so probes/s <= random
    # sectors/s (measured here, same buffer size class, same 64-byte fill)
    if 8 * n > L2_BYTES and not args.no_calibration:
        cal = random_sector_rate(device, stream)
        peak_sectors = cal["fill_64B"]["sectors_per_s"]
        probes_per_s = m / (lookup_ms / 1e3)
        roofline["random_sector"] = {"bound": "random 32-byte sector reads", "sectors_per_probe": 1,
                                     "achieved": round(probes_per_s / 1e9, 3), "peak": round(peak_sectors / 1e9, 3),
                                     "unit": "G sectors/s", "frac": round(probes_per_s / peak_sectors, 4),
                                     "calibration": cal,
                                     "peak_source": "gj_calibrate_random_sectors in this run (2 GiB buffer, "
                                                    "64-byte L2 fill, best of 5)"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_btree(h_keys, h_probes[: args.cpu_sample], args.cpu_sample)
    parity_all = {k: v["parity"] for k, v in per_index.items() if v.get("parity")}

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
        "parity": {"checked": sum(v["checked"] for v in parity_all.values()),
                   "mismatches": sum(v["mismatches"] for v in parity_all.values()),
                   "per_index": {k: v["mismatches"] for k, v in parity_all.items()},
                   "oracle": "oracle/oracle.c B+tree restatement (lower bound; exact = equal key), every probe",
                   "oracle_s": round(oracle_s, 2)},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": 2 * args.steps,
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_extras:
        headline_ix.free()
        del pairs, ws, expect
        torch.cuda.empty_cache()
        t0 = time.perf_counter()
        line["configurations"] = other_configurations(args, world, device, stream, keys, h_keys, h_probes)
        line["configurations"]["seconds"] = round(time.perf_counter() - t0, 1)
    return line


# ---------------------------------------------------------------------------
# further workloads (run with --workload; the default line is inlj)
# ---------------------------------------------------------------------------
def _base_line(args, world, metric, value, unit, ms_per_step, workload, extra):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic (seeded device generators)",
            "config": {"workload": workload, "parallelism": f"replicas x{world}"}}
    line.update(extra)
    return line


def partitioned_measure(args, world, device, stream, n_log2, m_log2, steps, kind="btree", sample_clocks=True):
    """Partitioned INLJ of 2^m_log2 Zipf(theta) probes into a 2^n_log2-key
    index: fanout and window from the library's autotuner (unless given),
    timed steps, pairs checked against the oracle on a seeded sample of probe
    rows, and the unpartitioned pairs on the same probes for comparison."""
    import ctypes

    import numpy as np
    import torch

    import gpujoin_gb300 as gj

    n, m = 1 << n_log2, 1 << m_log2
    keys = gj.generate_sorted_keys(n, gj.DIST_UNIFORM, 1 << args.key_bits, seed=args.seed)
    probes = gj.generate_probes(keys, m, theta=args.theta, seed=args.seed + 1)
    pairs = torch.empty(2 * m, dtype=torch.int32, device=device)
    count = torch.zeros(1, dtype=torch.int64, device=device)
    params = index_params(args, kind)
    ix = gj.make_index(kind, **params).construct(None, keys)
    # the partition directory is part of the index (built once, like the
    # B+tree's start table), outside the timed steps
    t_prep = time.perf_counter()
    ix.prepare_partitioned()
    prep_s = time.perf_counter() - t_prep
    tune = None
    if args.radix_bits and args.window:
        bits, window = args.radix_bits, min(args.window, m)
    else:
        bits, window, tuned_ms = gj.autotune_partitioned(ix, probes)
        tune = {"radix_bits": bits, "window": window, "ms": round(tuned_ms, 3),
                "candidates": "fanout 2^5..2^12 x window {m, m/4, m/16}"}
    need = ctypes.c_size_t()
    gj._check(gj.lib().gj_partitioned_inlj_workspace_size(ix.handle, window, bits, ctypes.byref(need)))
    ws = torch.empty(need.value, dtype=torch.uint8, device=device)

    def step():
        gj._check(gj.lib().gj_partitioned_inlj(ix.handle, probes.data_ptr(), m, window, bits, None,
                                                pairs.data_ptr(), count.data_ptr(), ws.data_ptr(), ws.numel(),
                                                stream.cuda_stream))

    sampler = ClockSampler(device.index) if sample_clocks else None
    if sampler:
        sampler.start()
    ms = time_steps(step, steps, args.warmup, stream, world, device)
    clocks = sampler.stop() if sampler else None
    ms = max_over_ranks(ms, world, device)
    got = int(count.item())
    parity = None
    if not args.no_parity:
        sem = "exact" if kind in EXACT_KINDS else "lower_bound"
        parity = check_pairs_sample(pairs, count, m, keys.cpu().numpy().view(np.uint64),
                                    probes.cpu().numpy().view(np.uint64), args.parity_sample, args.seed + 7, sem)
        parity["semantics"] = sem
    # the same probes through the unpartitioned pairs kernel, for comparison
    pw = ctypes.c_size_t()
    gj.lib().gj_inlj_pairs_workspace_size(m, ctypes.byref(pw))
    pws = torch.empty(pw.value, dtype=torch.uint8, device=device)
    plain_steps = max(2, steps // 2)
    plain_ms = time_steps(lambda: ix.inlj_pairs(probes, pairs, count, pws), plain_steps, 1, stream, world,
                          device) / plain_steps
    per_step = ms / steps
    bpp = 8 + 12 + 12 + 8 + 8.0 * n / m
    peak, peak_kind = measured_peak()
    achieved = bpp * m / (per_step / 1e3) / 1e9
    out = {"tuples_per_s": world * m * steps / (ms / 1e3), "ms_per_step": per_step, "build_keys": n, "probes": m,
           "zipf_theta": args.theta, "index": kind, "params": params or "default build",
           "directory_build_s": round(prep_s, 3), "radix_bits": bits,
           "window": window, "pairs": got, "autotune": tune, "parity": parity,
           "plain_pairs_ms_per_step": plain_ms, "plain_pairs_tuples_per_s": m / (plain_ms / 1e3),
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "bytes_per_probe": bpp,
                        "peak_source": f"{peak_kind} hbm_gbs (copy, burst)"},
           "launches_per_step": 3 + ((m + window - 1) // window) * 8, "clocks": clocks}
    # The probe pass reads its index slices from L2 (a partition's directory
    # and column slice stay resident while its probes run), one random
    # 32-byte sector per request; so its floor is the L2 rate of random
    # sector reads (calibrated here over a 32 MB buffer) times the L2 read
    # requests per probe that ncu counts (profiles/traffic.txt).
    if not args.no_calibration and n_log2 >= 24:
        req = profile_traffic(f"l2_read_requests_per_probe_k_part_probe_n{n_log2}")
        cal = random_sector_rate(device, stream, n_sectors=1 << 20, loads=1 << 28, reps=3)
        rate = cal["default_fill"]["sectors_per_s"]
        out["probe_l2_floor"] = {"l2_random_sectors_per_s": round(rate / 1e9, 1), "unit": "G sectors/s",
                                 "calibration_buffer_bytes": cal["buffer_bytes"],
                                 "l2_read_requests_per_probe": req,
                                 "probe_ms_floor": round(req * m / rate * 1e3, 3) if req else None}
        # The step against the roofline of what bounds each of its parts:
        # the partition passes stream 8 + 20 B per probe at HBM peak; the
        # probe pass needs its L2 random-sector reads (above) or its 12 + 8 B
        # per probe of streaming at HBM peak, whichever takes longer.
        if req:
            part_ms = 28.0 * m / (peak * 1e9) * 1e3
            probe_ms = max(req * m / rate * 1e3, 20.0 * m / (peak * 1e9) * 1e3)
            floor = part_ms + probe_ms
            out["roofline_sector"] = {
                "bound": "hbm (histogram + scatter) + L2 random 32-byte sectors (probe pass)",
                "floor_ms": round(floor, 3), "partition_ms_floor": round(part_ms, 3),
                "probe_ms_floor": round(probe_ms, 3), "achieved_ms": round(per_step, 3),
                "frac": round(floor / per_step, 4),
                "peaks": f"{peak_kind} hbm_gbs {peak} GB/s; L2 random sectors {rate / 1e9:.1f} G/s (calibrated now)"}
    ix.free()
    del keys, probes, pairs, ws, pws
    torch.cuda.empty_cache()
    return out


def partitioned_workload(args, world, rank, device, stream):
    """Partitioned INLJ at out-of-L2 scale: 2^28-key index, 2^29 Zipf(0.5)
    probes, range partition with an autotuned fanout (2^5..2^12) and window."""
    n_log2, m_log2 = args.n_log2, args.m_log2
    kind = args.indexes.split(",")[0]
    r = partitioned_measure(args, world, device, stream, n_log2, m_log2, args.steps, kind)
    return _base_line(
        args, world, "partitioned INLJ probe tuples/s (1 GB300 per rank), % of HBM roofline",
        r["tuples_per_s"], "probe tuples/s", r["ms_per_step"],
        f"partitioned INLJ: {r['build_keys']} uniform uint64 keys (2^{n_log2}), {r['probes']} Zipf({args.theta}) "
        f"probes (2^{m_log2}), {kind}, range partition 2^{r['radix_bits']}, window {r['window']}",
        {"partitioned": r, "parity": r["parity"], "roofline": dict(r["roofline"], traffic=None),
         "gpu_launches": args.steps * r["launches_per_step"], "clocks": r["clocks"], "cpu_baseline": None,
         "e2e": None})


def host_memory_available() -> int:
    """MemAvailable of /proc/meminfo in bytes (0 when unknown)."""
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def link_read_gbs(device, stream) -> float:
    """Pinned host -> HBM copy bandwidth (1 GiB, best of 5): the NVLink-C2C
    read peak the host-memory index is measured against."""
    import torch

    h = torch.empty(1 << 27, dtype=torch.int64).pin_memory()
    d = torch.empty(1 << 27, dtype=torch.int64, device=device)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    best = None
    for _ in range(6):
        a.record(stream)
        d.copy_(h, non_blocking=True)
        b.record(stream)
        torch.cuda.synchronize()
        t = a.elapsed_time(b)
        best = t if best is None or t < best else best
    del h, d
    return (8 << 27) / (best / 1e3) / 1e9


def host_index_workload(args, world, rank, device, stream):
    """Index resident in pinned Grace memory, read by the probe kernels over
    NVLink-C2C -- the GB300 form of the reference's index in host memory over
    NVLink 2.0 (src/index_lookup_config.hpp:52-66).  The column and the index
    live on the host, probes and pairs in HBM; the same data with the index in
    HBM runs beside it.  Column sizes that would take more than a quarter of
    the host's available memory are skipped."""
    import ctypes

    import torch

    import gpujoin_gb300 as gj

    m = 1 << args.m_log2
    kind = args.indexes.split(",")[0]
    params = index_params(args, kind)
    avail = host_memory_available()
    link = link_read_gbs(device, stream)
    pairs = torch.empty(2 * m, dtype=torch.int32, device=device)
    count = torch.zeros(1, dtype=torch.int64, device=device)
    wsz = ctypes.c_size_t(0)
    gj.lib().gj_inlj_pairs_workspace_size(m, ctypes.byref(wsz))
    ws = torch.empty(wsz.value, dtype=torch.uint8, device=device)
    sizes, head = {}, None
    for nl in [int(x) for x in args.host_n_log2.split(",")]:
        n = 1 << nl
        if avail and 8 * n * 1.25 > avail // 4:
            sizes[f"2^{nl}"] = {"skipped": f"{8 * n} B column against {avail} B of available host memory"}
            continue
        keys = gj.generate_sorted_keys(n, gj.DIST_UNIFORM, 1 << 63, seed=args.seed)
        probes = gj.generate_probes(keys, m, theta=args.theta, seed=args.seed + 1)
        h_keys = torch.empty(n, dtype=torch.int64, pin_memory=True)
        h_keys.copy_(keys)
        torch.cuda.synchronize()
        row = {}
        # host: column and index in Grace memory (the reference's setting);
        # column_host: column in Grace memory, inner levels in HBM; device: HBM
        for placement in ("host", "column_host", "device"):
            if placement == "host":
                ix = gj.make_index(kind, index_memory=gj.INDEX_MEMORY_HOST, **params).construct(None, h_keys)
            elif placement == "column_host":
                ix = gj.make_index(kind, **params).construct(None, h_keys)
            else:
                ix = gj.make_index(kind, **params).construct(None, keys)
            ms = time_steps(lambda: ix.inlj_pairs(probes, pairs, count, ws), args.steps, args.warmup, stream,
                            world, device)
            ms = max_over_ranks(ms, world, device)
            row[placement] = {"tuples_per_s": world * m * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                              "pairs": int(count.item()), "index_bytes": ix.memory_consumption(),
                              "host_index_bytes": ix.host_memory()}
            ix.free()
        row["same_pairs"] = row["host"]["pairs"] == row["device"]["pairs"] == row["column_host"]["pairs"]
        sizes[f"2^{nl}"] = row
        head = head or (nl, row)
        del keys, probes, h_keys
        torch.cuda.empty_cache()
    if head is None:
        return {"metric": "INLJ probe tuples/s, index in host memory", "unavailable": "no column size fits"}
    nl, row = head
    per_step = row["column_host"]["ms_per_step"]
    # over the link per probe: the column sector that holds the answer (the
    # inner levels stay in HBM / L2)
    link_bytes = 32
    achieved = link_bytes * m / (per_step / 1e3) / 1e9
    return _base_line(
        args, world, f"INLJ probe tuples/s ({kind}, column in Grace memory over NVLink-C2C, 1 GB300 per rank)",
        row["column_host"]["tuples_per_s"], "probe tuples/s", per_step,
        f"INLJ pairs, 2^{nl}-key column in pinned host memory, index levels in HBM, {m} Zipf({args.theta}) "
        f"probes in HBM (sizes: column and index in host memory / column in host memory / all in HBM)",
        {"host_index": {"index": kind, "params": params, "sizes": sizes, "host_memory_available": avail},
         "roofline": {"bound": "nvlink-c2c", "achieved": round(achieved, 1), "peak": round(link, 1), "unit": "GB/s",
                      "frac": round(achieved / link, 4), "traffic": None, "link_bytes_per_probe": link_bytes,
                      "peak_source": "pinned host-to-device copy measured in this run"},
         "gpu_launches": 2 * args.steps, "cpu_baseline": None, "e2e": None})


def orderings_workload(args, world, rank, device, stream):
    """Probe order as an autotuner choice (the reference's block-wise sorted
    lookups, src/index_lookup_common.cuh:398-549): INLJ pairs of 2^m_log2
    probes into 2^n_log2 keys in probe order, from sorted tiles and
    range-partitioned (one window, default fanout, directory kept with the
    index), over Zipf theta 0 (uniform), 0.5 and 1.0, with the autotuner's
    pick."""
    import ctypes

    import torch

    import gpujoin_gb300 as gj

    n, m = 1 << args.n_log2, 1 << args.m_log2
    kind = args.indexes.split(",")[0]
    keys = gj.generate_sorted_keys(n, gj.DIST_UNIFORM, 1 << 63, seed=args.seed)
    ix = gj.make_index(kind, **index_params(args, kind)).construct(None, keys)
    pairs = torch.empty(2 * m, dtype=torch.int32, device=device)
    count = torch.zeros(1, dtype=torch.int64, device=device)
    wsz = ctypes.c_size_t(0)
    gj.lib().gj_inlj_pairs_workspace_size(m, ctypes.byref(wsz))
    ws = torch.empty(wsz.value, dtype=torch.uint8, device=device)
    ix.prepare_partitioned()
    pwsz = ctypes.c_size_t(0)
    gj._check(gj.lib().gj_partitioned_inlj_workspace_size(ix.handle, m, 0, ctypes.byref(pwsz)))
    pws = torch.empty(pwsz.value, dtype=torch.uint8, device=device)

    def partitioned(probes, pairs, count, ws):
        gj._check(gj.lib().gj_partitioned_inlj(ix.handle, probes.data_ptr(), m, m, 0, None, pairs.data_ptr(),
                                                count.data_ptr(), pws.data_ptr(), pws.numel(), stream.cuda_stream))

    names = {gj.ORDER_PROBE: "probe", gj.ORDER_SORTED_TILES: "sorted_tiles", gj.ORDER_PARTITIONED: "partitioned"}
    thetas, head = {}, None
    for theta in (0.0, 0.5, 1.0):
        probes = gj.generate_probes(keys, m, theta=theta, seed=args.seed + 1)
        row = {}
        for name, fn in (("probe", ix.inlj_pairs), ("sorted_tiles", ix.inlj_pairs_sorted),
                         ("partitioned", partitioned)):
            ms = time_steps(lambda: fn(probes, pairs, count, ws), args.steps, args.warmup, stream, world, device)
            ms = max_over_ranks(ms, world, device)
            row[name] = {"tuples_per_s": world * m * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                         "pairs": int(count.item())}
        pick, _ = ix.autotune_ordering(probes)
        row["autotune"] = names[pick]
        row["same_pairs"] = row["probe"]["pairs"] == row["sorted_tiles"]["pairs"] == row["partitioned"]["pairs"]
        thetas[str(theta)] = row
        if theta == args.theta:
            head = row
        del probes
    head = head or thetas["0.5"]
    best = head[head["autotune"]]
    return _base_line(
        args, world, f"INLJ probe tuples/s ({kind}, autotuned probe order, 1 GB300 per rank)", best["tuples_per_s"],
        "probe tuples/s", best["ms_per_step"],
        f"INLJ pairs: {n} uniform uint64 build keys, {m} Zipf probes (theta 0, 0.5, 1.0), probe order vs "
        f"block-wise sorted tiles of 1024 vs range-partitioned",
        {"orderings": {"index": kind, "thetas": thetas}, "gpu_launches": None, "cpu_baseline": None, "e2e": None})


def star_inputs(n_fact, n_dim, seed, device):
    import torch

    g = torch.Generator(device="cpu")
    g.manual_seed(seed)
    dim_keys = torch.arange(1, n_dim + 1, dtype=torch.int64)
    flag = torch.zeros(n_dim, dtype=torch.uint8)
    flag[torch.randperm(n_dim, generator=g)[: n_dim // 6]] = 1
    fk = torch.randint(1, n_dim + 1, (n_fact,), generator=g, dtype=torch.int32)
    date = torch.randint(0, 2556, (n_fact,), generator=g, dtype=torch.int32)
    price = torch.randint(90000, 10500001, (n_fact,), generator=g, dtype=torch.int64)
    disc = torch.randint(0, 11, (n_fact,), generator=g, dtype=torch.int64)
    return [t.to(device) for t in (dim_keys, flag, fk, date, price, disc)]


def star_workload(args, world, rank, device, stream):
    """Star-join aggregate: 6M fact rows, 200k-row dimension indexed by a
    B+tree, 30-day date window, exact int64 sums."""
    import numpy as np
    import torch

    import gpujoin_gb300 as gj
    import oracle

    n_fact, n_dim, lo, hi = 6_000_000, 200_000, 1000, 1030
    dim_keys, flag, fk, date, price, disc = star_inputs(n_fact, n_dim, args.seed, device)
    ix = gj.btree_index().construct(None, dim_keys)
    out = torch.zeros(2, dtype=torch.int64, device=device)
    sorted_batches = args.star_order == "sorted"
    ms = time_steps(lambda: gj.star_join_sum(ix, fk, date, price, disc, flag, lo, hi, out,
                                             sorted_batches=sorted_batches), args.steps, args.warmup,
                    stream, world, device)
    ms = max_over_ranks(ms, world, device)
    got = out.cpu().numpy()
    num, den = oracle.star_join(fk.cpu().numpy().view(np.uint32), date.cpu().numpy().view(np.uint32),
                                price.cpu().numpy(), disc.cpu().numpy(), dim_keys.cpu().numpy().view(np.uint64),
                                flag.cpu().numpy(), lo, hi)
    per_step = ms / args.steps
    bytes_per_row = 4 + (30 / 2556) * (4 + 8 + 8 + 32)
    peak, peak_kind = measured_peak()
    achieved = bytes_per_row * n_fact / (per_step / 1e3) / 1e9
    return _base_line(
        args, world, "star-join fact rows/s (1 GB300 per rank)", world * n_fact * args.steps / (ms / 1e3),
        "fact rows/s", per_step,
        f"star join: {n_fact} fact rows, {n_dim} dimension rows (B+tree), 30-day window of 2556 days"
        + (", rows buffered and probed in key-sorted batches" if sorted_batches else ""),
        {"star": {"sums": [int(got[0]), int(got[1])], "oracle_sums": [num, den],
                  "exact": bool(int(got[0]) == num and int(got[1]) == den), "latency_us": per_step * 1e3},
         "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                      "frac": round(achieved / peak, 4), "traffic": None, "bytes_per_row": bytes_per_row,
                      "peak_source": f"{peak_kind} hbm_gbs (copy, burst)"},
         "gpu_launches": args.steps, "cpu_baseline": None, "e2e": None})


def learned_measure(args, world, device, stream, n_log2, m_log2, steps, quick):
    """Learned index against binary search and RadixSpline at exact outputs:
    2^27 keys from three distributions, 2^28 uniformly sampled probes with 5%
    absent keys, lower-bound positions.  The learned index runs as its
    default build (column-sized leaves, root chosen per column), at 2^14
    leaves (root chosen per column, and the 2x32 MLP root alone) and at 2^16
    leaves (the top of the 2^12-2^16 range); RadixSpline at its default error
    32 and at each learned model's recorded error bound.  Every index's
    positions are compared with the oracle on a seeded sample of probe rows
    plus every absent key, and in full with the GPU binary search."""
    import numpy as np
    import torch

    import gpujoin_gb300 as gj

    n, m = 1 << n_log2, 1 << m_log2
    results = {}
    out = torch.empty(m, dtype=torch.int32, device=device)
    ref = torch.empty(m, dtype=torch.int32, device=device)
    leaves = {"learned_leaves": args.learned_leaves} if args.learned_leaves else {}
    configs = (("binary_search", "binary_search", {}), ("radix_spline", "radix_spline", {}),
               ("learned", "learned", dict(leaves)),
               ("learned_2^14_leaves", "learned", {"learned_leaves": 1 << 14}),
               ("learned_mlp_2^14_leaves", "learned", {"learned_root": gj.LEARNED_ROOT_MLP, "learned_leaves": 1 << 14}),
               ("learned_2^16_leaves", "learned", {"learned_leaves": 1 << 16}),
               ("learned_mlp", "learned", {"learned_root": gj.LEARNED_ROOT_MLP, **leaves}),
               ("learned_segments", "learned", {"learned_root": gj.LEARNED_ROOT_SEGMENTS, **leaves}),
               ("learned_linear", "learned", {"learned_root": gj.LEARNED_ROOT_LINEAR, **leaves}))
    if quick:
        configs = configs[:6]
    parity_total = {"checked": 0, "mismatches": 0}
    for dist_name, dist in (("uniform", gj.DIST_UNIFORM), ("lognormal", gj.DIST_LOGNORMAL),
                            ("clusters", gj.DIST_CLUSTERS)):
        keys = gj.generate_sorted_keys(n, dist, 1 << 63, seed=args.seed + dist)
        probes = gj.generate_probes(keys, m, theta=0.0, absent_fraction=0.05, seed=args.seed + 10 + dist)
        row = {}
        bs = gj.binary_search_index().construct(None, keys)
        bs.lookup(probes, ref)
        bs.free()
        # rows checked against the oracle: a seeded sample plus every absent key
        present = (ref != -1) & (keys[ref.clamp(min=0).long()] == probes)
        absent_rows = torch.nonzero(~present).squeeze(1).cpu().numpy()
        rng = np.random.default_rng(args.seed + 20 + dist)
        rows = np.concatenate([rng.integers(0, m, size=min(args.parity_sample, m)), absent_rows])
        h_keys = keys.cpu().numpy().view(np.uint64)
        h_sel = probes[torch.from_numpy(rows).to(device)].cpu().numpy().view(np.uint64)
        want_lb, _ = oracle_positions(h_keys, h_sel)
        d_rows = torch.from_numpy(rows).to(device)
        d_want = torch.from_numpy(want_lb.view(np.int32)).to(device)
        del h_keys, h_sel

        def judge(entry):
            bad = int((out[d_rows] != d_want).sum())
            parity_total["checked"] += len(rows)
            parity_total["mismatches"] += bad
            entry["parity"] = {"checked": int(len(rows)), "mismatches": bad, "absent_rows": int(len(absent_rows))}
            entry["equals_gpu_binary_search"] = bool(torch.equal(out, ref))

        for name, kind, kw in configs:
            t0 = time.perf_counter()
            ix = gj.make_index(kind, **kw).construct(None, keys)
            torch.cuda.synchronize()
            build_s = time.perf_counter() - t0
            ms = time_steps(lambda: ix.lookup(probes, out), steps, args.warmup, stream, world, device)
            entry = {"tuples_per_s": m * steps / (ms / 1e3), "ms_per_step": ms / steps,
                     "build_s": round(build_s, 3), "index_bytes": ix.memory_consumption(), "params": kw or "default"}
            judge(entry)
            if kind == "learned":
                me, mw = ix.stats()
                entry.update({"max_error": me, "mean_window": round(mw, 2),
                              "root": ROOT_NAMES[ix.root_kind()]})
            row[name] = entry
            ix.free()
        # RadixSpline at the learned models' recorded error bounds (equal epsilon)
        lnames = [n for n in ("learned", "learned_2^14_leaves", "learned_2^16_leaves") if n in row]
        for lname in lnames:
            eps = int(min(row[lname]["max_error"], (1 << 31) - 1))
            ix = gj.radix_spline_index(rs_max_error=max(eps, 1)).construct(None, keys)
            ms = time_steps(lambda: ix.lookup(probes, out), steps, args.warmup, stream, world, device)
            entry = {"tuples_per_s": m * steps / (ms / 1e3), "ms_per_step": ms / steps, "max_error": eps,
                     "index_bytes": ix.memory_consumption()}
            judge(entry)
            row[f"radix_spline_eps_of_{lname}"] = entry
            ix.free()
        for lname in lnames:
            row[f"{lname}_beats"] = {k: row[lname]["tuples_per_s"] > row[k]["tuples_per_s"]
                                     for k in ("binary_search", "radix_spline", f"radix_spline_eps_of_{lname}")}
        results[dist_name] = row
        del keys, probes, present, d_rows, d_want
    torch.cuda.empty_cache()
    return results, dict(parity_total, oracle="oracle lower bound on sampled + absent rows")


def learned_workload(args, world, rank, device, stream):
    n_log2 = args.n_log2
    results, parity = learned_measure(args, world, device, stream, n_log2, args.m_log2, args.steps, args.learned_quick)
    head = results["uniform"]["learned"]
    n, m = 1 << n_log2, 1 << args.m_log2
    return _base_line(
        args, world, "learned-index probe tuples/s (1 GB300 per rank), exact lower bounds",
        world * head["tuples_per_s"], "probe tuples/s", head["ms_per_step"],
        f"learned vs plain: {n} keys (2^{n_log2}) x 3 distributions, {m} probes (2^{args.m_log2}) with 5% absent",
        {"learned": results, "parity": parity, "roofline": None, "gpu_launches": args.steps, "cpu_baseline": None,
         "e2e": None})


def batch_workload(args, world, rank, device, stream):
    """Batched lookup stream: 8 indexes (B+tree, Harmonia, RadixSpline,
    learned; 2^20..2^27 uniform or lognormal keys), 4096 batches of lognormal
    size in [1k, 16M] drawn Zipf(0.8) against their index, admitted in rounds
    by an HBM budget.  Each round is a plan run as one persistent kernel
    replayed from a CUDA graph (tile shape autotuned on the first round),
    against the same batches issued one kernel launch at a time."""
    import numpy as np
    import torch

    import gpujoin_gb300 as gj

    rng = np.random.default_rng(args.seed)
    specs = [("btree", 27, 0), ("harmonia", 26, 0), ("radix_spline", 25, 1), ("learned", 24, 1),
             ("btree", 23, 1), ("harmonia", 22, 0), ("radix_spline", 21, 0), ("learned", 20, 0)]
    indexes, cols = [], []
    for i, (kind, lg, dist) in enumerate(specs):
        keys = gj.generate_sorted_keys(1 << lg, dist, 1 << 63, seed=args.seed + 100 + i)
        indexes.append(gj.make_index(kind).construct(None, keys))
        cols.append(keys)
    nb = 4096
    sizes = np.clip(np.exp(rng.normal(np.log(65536), 1.6, nb)), 1000, 16 << 20).astype(np.int64)
    which = rng.integers(0, len(specs), nb).astype(np.uint32)
    budget = 2 << 30  # probe bytes admitted per round
    rounds, cur, cur_bytes = [], [], 0
    for b in range(nb):
        if cur and cur_bytes + 8 * sizes[b] > budget:
            rounds.append(cur)
            cur, cur_bytes = [], 0
        cur.append(b)
        cur_bytes += 8 * int(sizes[b])
    rounds.append(cur)
    max_round = max(int(sizes[r].sum()) for r in rounds)
    probes = torch.empty(max_round, dtype=torch.int64, device=device)
    out = torch.empty(max_round, dtype=torch.int32, device=device)
    done = torch.zeros(nb + 1, dtype=torch.int64, device=device)
    total = int(sizes.sum())
    tiles = None
    res = {"persistent_graph": {"ms": 0.0, "lat": []}, "per_launch": {"ms": 0.0, "lat": []}}
    launches = 0
    for ri, r in enumerate(rounds):
        bs = sizes[r]
        offs = np.concatenate([[0], np.cumsum(bs)[:-1]]).astype(np.uint64)
        for j, b in enumerate(r):
            probes[int(offs[j]): int(offs[j] + bs[j])] = gj.generate_probes(cols[which[b]], int(bs[j]), theta=0.8,
                                                                           seed=args.seed + int(b))
        plan = gj.batch_plan(indexes, which[r], offs, bs, tile_items=tiles or 0)
        if tiles is None:
            tiles, _ = plan.autotune(probes, out)
        for key, mode, graph in (("persistent_graph", 0, True), ("per_launch", 1, False)):
            run = plan.run_graph if graph else plan.run
            d = done[: len(r) + 1]
            for _ in range(max(1, args.warmup)):
                run(probes, out, mode, d)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            run(probes, out, mode, d)
            e1.record(stream)
            torch.cuda.synchronize()
            res[key]["ms"] += e0.elapsed_time(e1)
            t = d.cpu().numpy().astype(np.int64)
            res[key]["lat"].extend(((t[: len(r)] - t[len(r)]) / 1e3).tolist())
            launches += 1 if mode == 0 else len(r)
        plan.free()
    summary = {}
    for key, v in res.items():
        lat = np.array(v["lat"])
        summary[key] = {"tuples_per_s": total / (v["ms"] / 1e3), "ms_total": round(v["ms"], 3),
                        "p50_batch_latency_us": round(float(np.percentile(lat, 50)), 1),
                        "p99_batch_latency_us": round(float(np.percentile(lat, 99)), 1)}
    summary["tile_items"] = tiles
    summary["rounds"] = len(rounds)
    head = summary["persistent_graph"]
    return _base_line(
        args, world, "batched lookup stream probe tuples/s (1 GB300 per rank)", world * head["tuples_per_s"],
        "probe tuples/s", head["ms_total"],
        f"batched stream: 8 indexes (2^20..2^27 keys), {nb} batches, {total} probes, {len(rounds)} admission rounds "
        f"of <= 2 GiB of probes; latency = batch completion - round start",
        {"batch": summary, "roofline": None, "gpu_launches": launches, "cpu_baseline": None, "e2e": None})


def reference_main(args):
    import numpy as np

    import oracle

    world, rank, _ = dist_env()
    if rank != 0:
        return
    n, m = 1 << args.n_log2, 1 << args.m_log2
    rng = np.random.default_rng(args.seed)
    # n unique sorted uniform keys: draw a few extra, sort, drop repeats, then
    # drop a seeded random subset of the surplus (keeps the order sorted)
    keys = np.sort(rng.integers(0, 1 << 63, size=n + n // 64, dtype=np.uint64))
    keys = keys[np.concatenate([[True], keys[1:] != keys[:-1]])]
    if len(keys) > n:
        drop = rng.choice(len(keys), size=len(keys) - n, replace=False)
        keep = np.ones(len(keys), dtype=bool)
        keep[drop] = False
        keys = keys[keep]
    threads = oracle.hardware_threads()
    sample = min(args.ref_sample, m)
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
    ap.add_argument("--workload", choices=["inlj", "partitioned", "star", "learned", "batch", "host_index",
                                           "orderings"], default="inlj")
    ap.add_argument("--host-n-log2", default="26,28", help="host_index: column sizes (log2 keys)")
    ap.add_argument("--n-log2", type=int, default=None,
                    help="build keys (log2); default 26, 28 for partitioned, 27 for learned")
    ap.add_argument("--m-log2", type=int, default=None,
                    help="probes (log2); default 28, 29 for partitioned")
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--indexes", default="btree,harmonia,radix_spline,binary_search,learned,hash,btree_w64")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--cpu-sample", type=int, default=1 << 28,
                    help="probes of the CPU baseline leg (one timed pass; about 6 s on 16 Grace cores)")
    ap.add_argument("--ref-sample", type=int, default=1 << 25,
                    help="probes per step of --impl reference (all host threads)")
    ap.add_argument("--btree-node-keys", type=int, default=0, help="B+tree inner node width (0 = library default)")
    ap.add_argument("--btree-start-bits", type=int, default=0,
                    help="B+tree start table bits (0 = library default)")
    ap.add_argument("--btree-leaf-keys", type=int, default=0, help="B+tree leaf width (0 = library default)")
    ap.add_argument("--learned-leaves", type=int, default=0, help="learned: leaf models (0 = library default)")
    ap.add_argument("--radix-bits", type=int, default=0, help="partitioned: fanout bits (0 = autotune)")
    ap.add_argument("--key-bits", type=int, default=63,
                    help="partitioned: build keys drawn from [0, 2^bits) (default 63, the INLJ configuration)")
    ap.add_argument("--window", type=int, default=0, help="partitioned: window size in probes (0 = autotune)")
    ap.add_argument("--parity-sample", type=int, default=1 << 25,
                    help="probe rows checked against the oracle where not every probe is checked")
    ap.add_argument("--learned-quick", action="store_true",
                    help="learned: only binary search, RadixSpline and the learned builds at both leaf counts")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle checks (timing runs)")
    ap.add_argument("--no-calibration", action="store_true", help="inlj: skip the random-sector calibration")
    ap.add_argument("--star-order", choices=["probe", "sorted"], default="probe",
                    help="star: fact-row order of the lookups (sorted = buffered, key-sorted batches)")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="inlj: skip timing the reference's own device lookups (oracle/_ref/refgpu.cubin)")
    ap.add_argument("--no-extras", action="store_true",
                    help="inlj: only the headline (no partitioned / learned / theta / star / CPU sections)")
    ap.add_argument("--extra-steps", type=int, default=5, help="timed steps of each extra section")
    ap.add_argument("--cpu-one-sample", type=int, default=1 << 20, help="CPU baselines: probes at 1 thread")
    ap.add_argument("--cpu-all-sample", type=int, default=1 << 24, help="CPU baselines: probes at all threads")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    return ap.parse_args(argv)


# (build keys, probes) as log2 per workload when not given
SIZES = {"partitioned": (28, 29), "learned": (27, 28)}


def resolve_sizes(args):
    """Fill in the build and probe sizes a workload runs at when not given
    (the reference arm runs the INLJ sizes)."""
    n_def, m_def = SIZES.get(args.workload, (26, 28)) if args.impl != "reference" else (26, 28)
    if args.n_log2 is None:
        args.n_log2 = n_def
    if args.m_log2 is None:
        args.m_log2 = m_def
    return args


def main(argv=None):
    args = resolve_sizes(parse_args(argv))
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_main(args)
    else:
        gpu_main(args)


if __name__ == "__main__":
    main()
