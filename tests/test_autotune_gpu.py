"""Autotuners: the returned configuration is one of the candidates, and the
tuned configuration still gives the oracle's results."""
import numpy as np
import pytest

from test_join_gpu import pairs_of
from test_lookup_gpu import column, from_dev_u32, probes_for, to_dev

pytestmark = pytest.mark.gpu


def test_autotune_btree(orc, gj, cuda):
    import torch

    rng = np.random.default_rng(5)
    col = column(rng, 1 << 16)
    pr = probes_for(rng, col, 1 << 16)
    d_col, d_pr = to_dev(torch, col), to_dev(torch, pr)
    w, l, ms = gj.autotune_btree(d_col, d_pr)
    assert w in (4, 7, 8, 15, 16) and l in (4, 8, 16, 32) and ms > 0
    ix = gj.btree_index(btree_node_keys=w, btree_leaf_keys=l).construct(None, d_col)
    np.testing.assert_array_equal(from_dev_u32(ix.lookup(d_pr)), orc.exact_lookup(col, pr))


def test_autotune_partitioned(orc, gj, cuda):
    import torch

    rng = np.random.default_rng(6)
    col = column(rng, 1 << 17)
    pr = probes_for(rng, col, 1 << 18)
    d_col, d_pr = to_dev(torch, col), to_dev(torch, pr)
    ix = gj.btree_index().construct(None, d_col)
    bits, window, ms = gj.autotune_partitioned(ix, d_pr)
    m = len(pr)
    assert 5 <= bits <= 12 and window in (m, m // 4, m // 16) and ms > 0
    _, prs, cnt = ix.partitioned_inlj(d_pr, window_size=window, radix_bits=bits, positions=False, pairs=True)
    rows, bpos = pairs_of(prs, cnt)
    erows, epos = orc.pairs_from_positions(orc.exact_lookup(col, pr))
    order = np.argsort(rows, kind="stable")
    np.testing.assert_array_equal(rows[order], erows)
    np.testing.assert_array_equal(bpos[order], epos)


def test_autotune_partitioned_btree(orc, gj, cuda):
    import torch

    rng = np.random.default_rng(7)
    col = column(rng, 1 << 17)
    pr = probes_for(rng, col, 1 << 18)
    d_col, d_pr = to_dev(torch, col), to_dev(torch, pr)
    w, lk, bits, window, ms = gj.autotune_partitioned_btree(d_col, d_pr)
    m = len(pr)
    assert (w, lk) in ((4, 4), (4, 8), (4, 16), (7, 4), (15, 4)) and 5 <= bits <= 12 and window in (m, m // 4, m // 16)
    ix = gj.btree_index(btree_node_keys=w, btree_leaf_keys=lk).construct(None, d_col)
    _, prs, cnt = ix.partitioned_inlj(d_pr, window_size=window, radix_bits=bits, positions=False, pairs=True)
    rows, bpos = pairs_of(prs, cnt)
    erows, epos = orc.pairs_from_positions(orc.exact_lookup(col, pr))
    order = np.argsort(rows, kind="stable")
    np.testing.assert_array_equal(rows[order], erows)
    np.testing.assert_array_equal(bpos[order], epos)
