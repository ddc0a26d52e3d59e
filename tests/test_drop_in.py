"""Reference-style code (index class templates, device_index by value,
cooperative_lookup in the kernel) compiled against include/gpujoin/indexes.cuh
and libgpujoin.so: it compiles here, and on a GPU its results equal the
oracle's."""
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
