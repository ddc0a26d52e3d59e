"""The oracle's fast lower bound (through its B+tree restatement, used for the
large checks of bench.py) equals its plain binary search (which the golden
fixtures pin to the reference's lower_bound), on present and absent keys,
ragged sizes and the extreme keys."""
import numpy as np
import pytest


@pytest.mark.parametrize("n", [1, 2, 3, 246, 247, 248, 60_000, 247 * 246 + 1, 400_003])
def test_btree_lower_bound_equals_binary_search(orc, n):
    rng = np.random.default_rng(n)
    col = np.unique(rng.integers(1, (1 << 64) - 2, size=n + 64, dtype=np.uint64))[:n]
    present = col[rng.integers(0, len(col), size=20_000)]
    absent = rng.integers(0, (1 << 64) - 1, size=20_000, dtype=np.uint64)
    edges = np.array([0, 1, col[0] - 1, col[0], col[-1], col[-1] + 1, (1 << 64) - 1], dtype=np.uint64)
    pr = np.concatenate([present, absent, edges])
    lb = orc.BTree(col, 247, 246).lower_bound(pr, 4)
    np.testing.assert_array_equal(lb, orc.bs_lookup(col, pr))
    flb, fex = orc.fast_positions(col, pr, 4)
    np.testing.assert_array_equal(flb, lb)
    np.testing.assert_array_equal(fex, orc.exact_lookup(col, pr))
