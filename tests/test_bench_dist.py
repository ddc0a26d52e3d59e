"""Host-side logic of bench.py's N > 1 path on CPU: two gloo ranks agree on
the slowest rank's time (replicas, timing = max over ranks), and the
reference arm runs on rank 0 only."""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, results):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    w, r = bench.init_dist("gloo")
    bench.barrier(w)
    slowest = bench.max_over_ranks(10.0 + 5.0 * rank, w)
    results[rank] = slowest
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as mgr:
        results = mgr.dict()
        mp.spawn(_rank_main, args=(world, port, results), nprocs=world, join=True)
        assert dict(results) == {0: 15.0, 1: 15.0}


def test_reference_arm_rank_nonzero_does_no_work(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.reference_main(bench.parse_args(["--impl", "reference", "--n-log2", "12", "--m-log2", "14"]))
    assert buf.getvalue() == ""


def test_reference_arm_line(monkeypatch, orc):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.delenv("RANK", raising=False)
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.reference_main(bench.parse_args(["--impl", "reference", "--n-log2", "14", "--m-log2", "16",
                                               "--cpu-sample", "4096", "--steps", "3"]))
    line = json.loads(buf.getvalue().strip())
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_bench_defines_each_function_once():
    import ast
    import collections
    import os

    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py")
    tree = ast.parse(open(path).read())
    names = collections.Counter(n.name for n in tree.body if isinstance(n, ast.FunctionDef))
    assert not [k for k, v in names.items() if v > 1]


def test_workload_sizes():
    # each workload's default sizes (log2 keys, log2 probes), and explicit sizes kept
    sys.path.insert(0, ROOT)
    import bench

    def sizes(*argv):
        a = bench.resolve_sizes(bench.parse_args(list(argv)))
        return a.n_log2, a.m_log2

    assert sizes() == (26, 28)
    assert sizes("--workload", "partitioned") == (28, 29)
    assert sizes("--workload", "learned") == (27, 28)
    assert sizes("--workload", "orderings") == (26, 28)
    assert sizes("--impl", "reference") == (26, 28)
    assert sizes("--workload", "partitioned", "--n-log2", "26", "--m-log2", "28") == (26, 28)
    assert sizes("--workload", "learned", "--n-log2", "20") == (20, 28)
