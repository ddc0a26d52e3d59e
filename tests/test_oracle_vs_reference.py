"""Randomised cross-check of the CPU oracle against the reference-built checker
(oracle/_ref, only where the reference tree exists -- skipped elsewhere)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(orc):
    if orc.ref_lib() is None:
        pytest.skip("reference-built checker not available on this host")
    return orc


@pytest.mark.parametrize("n", [32, 96, 1056, 1088, 32 * 1089 + 32 * 7, 32 * 36000])
def test_harmonia_random_sizes(ref, n):
    rng = np.random.default_rng(n)
    col = np.unique(rng.integers(0, 1 << 63, size=n + 64, dtype=np.uint64))[:n]
    assert len(col) == n
    pr = np.concatenate([col[rng.integers(0, n, 4000)], rng.integers(0, 1 << 63, 2000, dtype=np.uint64)])
    np.testing.assert_array_equal(ref.Harmonia(col).lookup(pr), ref.ref_harmonia_lookup(col, pr))
    k1, c1, d1 = ref.Harmonia(col).arrays()
    k2, c2, d2 = ref.ref_harmonia_arrays(col)
    np.testing.assert_array_equal(k1, k2)
    np.testing.assert_array_equal(c1, c2)
    assert d1 == d2


@pytest.mark.parametrize("n", [1, 2, 247, 500, 61009, 61010, 300000])
def test_btree_random_sizes(ref, n):
    rng = np.random.default_rng(n + 7)
    col = np.unique(rng.integers(0, 1 << 63, size=n + 64, dtype=np.uint64))[:n]
    pr = np.concatenate([col[rng.integers(0, n, 4000)], rng.integers(0, 1 << 63, 2000, dtype=np.uint64)])
    np.testing.assert_array_equal(ref.BTree(col).lookup(pr), ref.ref_btree_lookup(col, pr))


@pytest.mark.parametrize("n", [2, 3, 5, 1000, 65537])
def test_search_random_sizes(ref, n):
    rng = np.random.default_rng(n + 11)
    col = np.unique(rng.integers(0, 1 << 40, size=n + 64, dtype=np.uint64))[:n]
    pr = rng.integers(0, 1 << 40, 5000, dtype=np.uint64)
    np.testing.assert_array_equal(ref.bs_lookup(col, pr), ref.ref_bs_lookup(col, pr))
    np.testing.assert_array_equal(ref.bs_lookup(col, pr, branch_free=True), ref.ref_bs_branch_free_lookup(col, pr))
