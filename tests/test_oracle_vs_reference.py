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


@pytest.mark.parametrize("n", [1, 247, 248, 247 * 246, 247 * 246 + 1, 247 * 247 * 3 + 5, 1000003])
def test_btree_page_image_is_the_reference_tree(ref, n):
    # The page image that the GPU timing of the reference's own B+tree lookup
    # runs on (oracle/ref_gpu.py) is the oracle's build written in the
    # reference's page layout; read back breadth first it must be the tree
    # the reference's btree::construct builds: the same nodes, counts, final
    # flags, separators and leaf positions.
    rng = np.random.default_rng(n + 3)
    col = np.unique(rng.integers(0, 1 << 62, size=n + 64, dtype=np.uint64))[:n]
    page, header, keys_off, children_off, inner_keys, leaf_keys = ref.ref_btree_layout()
    assert (page, header, inner_keys, leaf_keys) == (4096, 128, 246, 247)
    pages_base, col_base = 0x7F0000000000, 0x7E0000000000
    image, root = ref.BTree(col, leaf_keys, inner_keys).pages(page, keys_off, children_off, pages_base, col_base)
    ours = ref.btree_canonical_from_pages(image, page, keys_off, children_off, root, pages_base, col_base)
    np.testing.assert_array_equal(ours, ref.ref_btree_canonical(col))


@pytest.mark.parametrize("n", [2, 3, 5, 1000, 65537])
def test_search_random_sizes(ref, n):
    rng = np.random.default_rng(n + 11)
    col = np.unique(rng.integers(0, 1 << 40, size=n + 64, dtype=np.uint64))[:n]
    pr = rng.integers(0, 1 << 40, 5000, dtype=np.uint64)
    np.testing.assert_array_equal(ref.bs_lookup(col, pr), ref.ref_bs_lookup(col, pr))
    np.testing.assert_array_equal(ref.bs_lookup(col, pr, branch_free=True), ref.ref_bs_branch_free_lookup(col, pr))
