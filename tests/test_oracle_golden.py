"""Pin the CPU oracle against fixtures produced by the reference's own code
(tests/golden/make_golden.py runs the reference's search.cuh, btree.cuh and
harmonia.cuh, compiled in place)."""
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _sizes(d, prefix):
    return sorted({int(k.split("_")[1]) for k in d.files if k.startswith(prefix + "_")})


def test_binary_search_matches_reference(orc):
    d = _load("search.npz")
    for n in _sizes(d, "bs"):
        col, pr = d[f"bs_{n}_col"], d[f"bs_{n}_probes"]
        np.testing.assert_array_equal(orc.bs_lookup(col, pr), d[f"bs_{n}_lb"], err_msg=f"n={n}")
        np.testing.assert_array_equal(orc.bs_lookup(col, pr, branch_free=True), d[f"bs_{n}_bf"], err_msg=f"n={n}")


def test_lower_bound_primitives(orc):
    d = _load("search.npz")
    col, pr = d["bs_1000_col"], d["bs_1000_probes"]
    lb = np.searchsorted(col, pr, side="left")
    exp = np.where(lb < len(col), lb, 0xFFFFFFFF).astype(np.uint32)
    np.testing.assert_array_equal(orc.bs_lookup(col, pr), exp)


def test_btree_matches_reference_page_geometry(orc):
    d = _load("btree.npz")
    for n in _sizes(d, "btree"):
        col, pr = d[f"btree_{n}_col"], d[f"btree_{n}_probes"]
        got = orc.BTree(col, 247, 246).lookup(pr)
        np.testing.assert_array_equal(got, d[f"btree_{n}_pos"], err_msg=f"n={n}")


def test_btree_64_key_nodes_same_positions(orc):
    # the product uses 64-key nodes; positions must not depend on node size
    d = _load("btree.npz")
    for n in _sizes(d, "btree"):
        col, pr = d[f"btree_{n}_col"], d[f"btree_{n}_probes"]
        for leaf, inner in ((64, 64), (16, 15), (247, 246)):
            np.testing.assert_array_equal(orc.BTree(col, leaf, inner).lookup(pr), d[f"btree_{n}_pos"],
                                          err_msg=f"n={n} geometry {leaf}/{inner}")


def test_harmonia_matches_reference(orc):
    d = _load("harmonia.npz")
    for n in _sizes(d, "harmonia"):
        col, pr = d[f"harmonia_{n}_col"], d[f"harmonia_{n}_probes"]
        h = orc.Harmonia(col)
        np.testing.assert_array_equal(h.lookup(pr), d[f"harmonia_{n}_pos"], err_msg=f"n={n}")
        keys, children, depth = h.arrays()
        np.testing.assert_array_equal(keys, d[f"harmonia_{n}_keys"], err_msg=f"keys n={n}")
        np.testing.assert_array_equal(children, d[f"harmonia_{n}_children"], err_msg=f"children n={n}")
        assert depth == int(d[f"harmonia_{n}_depth"][0])


def test_harmonia_known_answers(orc):
    # test/test_harmonia.cu:37-55 and test/main.cu:144-164: iota keys, lookup(k) == k
    d = _load("harmonia_kat.npz")
    for key in d.files:
        _, node, n = key.split("_")
        node, n = int(node), int(n)
        col = np.arange(n, dtype=np.uint64)
        expected = d[key]
        if len(expected) == 0:
            # the reference's construct() rejects n % node_size != 0
            with pytest.raises(RuntimeError):
                orc.Harmonia(col, max_keys=node)
            continue
        got = orc.Harmonia(col, max_keys=node).lookup(col)
        np.testing.assert_array_equal(got, expected.astype(np.uint32), err_msg=key)
        np.testing.assert_array_equal(got, np.arange(n, dtype=np.uint32))


def test_exact_semantics_equal_for_btree_and_harmonia(orc):
    d = _load("harmonia.npz")
    for n in _sizes(d, "harmonia"):
        col, pr = d[f"harmonia_{n}_col"], d[f"harmonia_{n}_probes"]
        np.testing.assert_array_equal(orc.exact_lookup(col, pr), d[f"harmonia_{n}_pos"])


def test_radix_spline_returns_exact_lower_bound(orc):
    d = _load("search.npz")
    for n in _sizes(d, "bs"):
        col, pr = d[f"bs_{n}_col"], d[f"bs_{n}_probes"]
        for bits, err in ((18, 32), (4, 1), (10, 0)):
            rs = orc.RadixSpline(col, bits, err)
            np.testing.assert_array_equal(rs.lookup(pr), d[f"bs_{n}_lb"], err_msg=f"n={n} bits={bits} err={err}")


def test_radix_spline_error_bound_on_build_keys(orc):
    rng = np.random.default_rng(5)
    col = np.unique(rng.integers(0, 1 << 63, size=200000, dtype=np.uint64))
    for err in (1, 8, 32):
        rs = orc.RadixSpline(col, 18, err)
        sample = rng.integers(0, len(col), size=5000)
        est = np.array([rs.estimate(int(col[i])) for i in sample])
        assert np.max(np.abs(est - sample)) <= err + 1e-6
