"""Reference-style code (index class templates, device_index by value,
cooperative_lookup in the kernel, partitioned_relation<T> with
range_partition / partitioned_lookup, experiment_config and parse_options)
compiled against include/gpujoin/indexes.cuh,
include/gpujoin/partitioned_relation.hpp and libgpujoin.so: it compiles
here, parses the reference's command line, and on a GPU its results equal
the oracle's."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "drop_in", "reference_style_probe.cu")


def build_drop_in(tmpdir) -> str:
    import gpujoin_gb300
    from gpujoin_gb300 import build as gbuild

    gpujoin_gb300.lib()
    out = os.path.join(str(tmpdir), "libdropin.so")
    libdir = os.path.dirname(gpujoin_gb300.LIB_PATH)
    cmd = [gbuild.nvcc(), *gbuild.ARCH, "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", out, "-L", libdir, "-lgpujoin",
           "-Xlinker", "-rpath", "-Xlinker", libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_reference_style_code_compiles(tmp_path, gj):
    lib = ctypes.CDLL(build_drop_in(tmp_path))
    lib.drop_in_type_name.restype = ctypes.c_char_p
    assert lib.drop_in_type_name() == b"btree"


@pytest.mark.gpu
@pytest.mark.parametrize("kind,name", [(0, "btree"), (1, "harmonia"), (2, "binary_search"), (3, "radix_spline"),
                                       (4, "no_op"), (5, "learned")])
def test_reference_style_code_probes(tmp_path, orc, gj, cuda, kind, name):
    import torch

    lib = ctypes.CDLL(build_drop_in(tmp_path))
    lib.drop_in_probe.restype = ctypes.c_int
    lib.drop_in_probe.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                  ctypes.c_uint64, ctypes.c_void_p]
    rng = np.random.default_rng(kind)
    col = np.sort(np.unique(rng.integers(0, 1 << 63, 40000, dtype=np.uint64)))[: 32 * 1200]
    pr = np.concatenate([col[rng.integers(0, len(col), 20000)], rng.integers(0, 1 << 63, 5000, dtype=np.uint64)])
    d_col = torch.from_numpy(col.view(np.int64)).cuda()
    d_pr = torch.from_numpy(pr.view(np.int64)).cuda()
    out = torch.empty(len(pr), dtype=torch.int64, device="cuda")
    rc = lib.drop_in_probe(kind, d_col.data_ptr(), col.ctypes.data, len(col), d_pr.data_ptr(), len(pr), out.data_ptr())
    assert rc == 0
    got = out.cpu().numpy().view(np.uint64)
    if name in ("btree", "harmonia"):
        exp = orc.exact_lookup(col, pr)
    elif name == "no_op":
        exp = np.full(len(pr), 0xFFFFFFFF, dtype=np.uint32)
    else:
        exp = orc.bs_lookup(col, pr)
    exp64 = np.where(exp == 0xFFFFFFFF, np.uint64(0xFFFFFFFFFFFFFFFF), exp.astype(np.uint64))
    np.testing.assert_array_equal(got, exp64)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,name", [(1, "harmonia"), (2, "binary_search")])
@pytest.mark.parametrize("degree", [1, 2, 4, 5])
def test_reference_style_warp_cooperative_lookup(tmp_path, orc, gj, cuda, kind, name, degree):
    # warp_cooperative_lookup<Degree>: the reference's warp-collective
    # protocol (groups of 2^Degree lanes per query, every lane of the warp
    # calling, a partly inactive last warp) with the per-thread results
    import torch

    lib = ctypes.CDLL(build_drop_in(tmp_path))
    lib.drop_in_probe_warp.restype = ctypes.c_int
    lib.drop_in_probe_warp.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                       ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    rng = np.random.default_rng(10 * kind + degree)
    col = np.sort(np.unique(rng.integers(0, 1 << 63, 80000, dtype=np.uint64)))[: 32 * 2000]
    pr = np.concatenate([col[rng.integers(0, len(col), 20000)], rng.integers(0, 1 << 63, 5001, dtype=np.uint64),
                         np.array([0, col[0], col[-1], col[-1] + 1, (1 << 64) - 1], dtype=np.uint64)])
    d_col = torch.from_numpy(col.view(np.int64)).cuda()
    d_pr = torch.from_numpy(pr.view(np.int64)).cuda()
    out = torch.empty(len(pr), dtype=torch.int64, device="cuda")
    rc = lib.drop_in_probe_warp(kind, degree, d_col.data_ptr(), col.ctypes.data, len(col), d_pr.data_ptr(), len(pr),
                                out.data_ptr())
    assert rc == 0
    exp = orc.exact_lookup(col, pr) if name == "harmonia" else orc.bs_lookup(col, pr)
    exp64 = np.where(exp == 0xFFFFFFFF, np.uint64(0xFFFFFFFFFFFFFFFF), exp.astype(np.uint64))
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint64), exp64)


def _parse(lib, args):
    argv = (ctypes.c_char_p * (len(args) + 1))(b"index_lookup", *[a.encode() for a in args])
    out = (ctypes.c_uint64 * 10)()
    approach, index = ctypes.create_string_buffer(32), ctypes.create_string_buffer(32)
    rc = lib.drop_in_parse_options(len(args) + 1, argv, out, approach, index)
    return rc, list(out), approach.value.decode(), index.value.decode()


def test_reference_command_line_parses(tmp_path, gj):
    lib = ctypes.CDLL(build_drop_in(tmp_path))
    lib.drop_in_parse_options.restype = ctypes.c_int
    # the reference's defaults (src/index_lookup_config.hpp:18-34)
    rc, out, approach, index = _parse(lib, [])
    assert rc == 0 and (approach, index) == ("plain", "btree")
    assert out == [1000000, 100000000, 0, 10000, 1, 0, 0, 128, 1250, 11]
    # short and long forms as scripts/bench_join.sh writes them
    rc, out, approach, index = _parse(lib, ["-a", "partitioning", "-i", "harmonia", "-e", "67108864", "-l",
                                            "268435456", "--maxbits=40", "-w", "1048576", "-d", "dense", "-p",
                                            "zipf", "-z", "0.5", "-s", "-b", "256"])
    assert rc == 0 and (approach, index) == ("partitioning", "harmonia")
    assert out == [67108864, 268435456, 40, 1048576, 0, 2, 1, 256, 500, 11]
    assert _parse(lib, ["-h"])[0] == 1
    assert _parse(lib, ["--dataset", "skewed"])[0] == -1
    assert _parse(lib, ["-q"])[0] == -1
    assert _parse(lib, ["-w"])[0] == -1


@pytest.mark.gpu
@pytest.mark.parametrize("kind,bits", [(0, 8), (0, 11), (2, 4)])
def test_reference_style_partitioned_probe(tmp_path, orc, gj, cuda, kind, bits):
    import torch

    lib = ctypes.CDLL(build_drop_in(tmp_path))
    lib.drop_in_partitioned_probe.restype = ctypes.c_int
    lib.drop_in_partitioned_probe.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                              ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p]
    rng = np.random.default_rng(kind * 100 + bits)
    col = np.sort(np.unique(rng.integers(0, 1 << 63, 70000, dtype=np.uint64)))[:65536]
    pr = np.concatenate([col[rng.integers(0, len(col), 30000)], rng.integers(0, 1 << 63, 7000, dtype=np.uint64)])
    d_col = torch.from_numpy(col.view(np.int64)).cuda()
    d_pr = torch.from_numpy(pr.view(np.int64)).cuda()
    out = torch.empty(len(pr), dtype=torch.int32, device="cuda")
    rc = lib.drop_in_partitioned_probe(kind, d_col.data_ptr(), col.ctypes.data, len(col), d_pr.data_ptr(), len(pr),
                                       bits, out.data_ptr())
    assert rc == 0
    got = out.cpu().numpy().view(np.uint32)
    exp = orc.exact_lookup(col, pr) if kind == 0 else orc.bs_lookup(col, pr)
    np.testing.assert_array_equal(got, exp)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,name", [(0, "btree"), (2, "binary_search")])
@pytest.mark.parametrize("approach,window", [("plain", 0), ("bws", 0), ("partitioning", 10000), ("partitioning", 0),
                                             ("auto", 0)])
def test_reference_style_approaches(tmp_path, orc, gj, cuda, kind, name, approach, window):
    # inlj_pairs_by_approach: the reference's approach names give the same
    # set of pairs; "plain" gives them in probe order
    import torch

    lib = ctypes.CDLL(build_drop_in(tmp_path))
    lib.drop_in_approach_pairs.restype = ctypes.c_int
    lib.drop_in_approach_pairs.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_uint64, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                                           ctypes.c_void_p, ctypes.c_void_p]
    rng = np.random.default_rng(kind * 10 + len(approach) + window)
    col = np.sort(np.unique(rng.integers(0, 1 << 63, 70000, dtype=np.uint64)))[:65536]
    pr = np.concatenate([col[rng.integers(0, len(col), 30000)], rng.integers(0, 1 << 63, 7001, dtype=np.uint64)])
    rng.shuffle(pr)
    d_col = torch.from_numpy(col.view(np.int64)).cuda()
    d_pr = torch.from_numpy(pr.view(np.int64)).cuda()
    pairs = torch.empty(2 * len(pr), dtype=torch.int32, device="cuda")
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    rc = lib.drop_in_approach_pairs(kind, approach.encode(), window, d_col.data_ptr(), col.ctypes.data, len(col),
                                    d_pr.data_ptr(), len(pr), pairs.data_ptr(), count.data_ptr())
    assert rc == 0
    c = int(count.item())
    got = pairs[: 2 * c].cpu().numpy().view(np.uint32).reshape(-1, 2)
    exp = orc.exact_lookup(col, pr) if name == "btree" else orc.bs_lookup(col, pr)
    erows, epos = orc.pairs_from_positions(exp)
    if approach == "plain":
        np.testing.assert_array_equal(got[:, 0], erows)
        np.testing.assert_array_equal(got[:, 1], epos)
    order = np.argsort(got[:, 0], kind="stable")
    np.testing.assert_array_equal(got[order, 0], erows)
    np.testing.assert_array_equal(got[order, 1], epos)


def test_reference_style_unknown_approach(tmp_path, gj):
    # an unknown approach name is refused before anything runs on a GPU
    lib = ctypes.CDLL(build_drop_in(tmp_path))
    lib.drop_in_approach_name_known.restype = ctypes.c_int
    lib.drop_in_approach_name_known.argtypes = [ctypes.c_char_p]
    assert [lib.drop_in_approach_name_known(a) for a in (b"plain", b"bws", b"partitioning", b"auto")] == [1] * 4
    assert lib.drop_in_approach_name_known(b"hj") == 0 and lib.drop_in_approach_name_known(b"sorted") == 0
