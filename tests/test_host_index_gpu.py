"""Indexes resident in pinned host memory (Grace memory read over NVLink-C2C,
index_memory = GJ_INDEX_MEMORY_HOST): the column and the index's own arrays
live on the host, probes and results in HBM.  Every index kind and probe
operator gives the oracle's results, and the index's arrays really are in
host memory."""
import numpy as np
import pytest

from test_join_gpu import pairs_of
from test_lookup_gpu import column, expected, from_dev_u32, probes_for, to_dev

pytestmark = pytest.mark.gpu


def host_column(torch, col):
    return torch.from_numpy(np.ascontiguousarray(col).view(np.int64)).pin_memory()


@pytest.mark.parametrize("kind", ["binary_search", "btree", "harmonia", "radix_spline", "learned"])
def test_host_index_lookup(orc, gj, cuda, kind):
    import torch

    rng = np.random.default_rng(31)
    col = column(rng, 1 << 18)
    pr = probes_for(rng, col, 1 << 17)
    ix = gj.make_index(kind, index_memory=gj.INDEX_MEMORY_HOST).construct(None, host_column(torch, col))
    assert ix.host_memory() > 0
    got = from_dev_u32(ix.lookup(to_dev(torch, pr)))
    np.testing.assert_array_equal(got, expected(orc, kind, col, pr))


@pytest.mark.parametrize("node_keys,leaf_keys", [(15, 4), (7, 4), (4, 8)])
def test_host_btree_pairs_and_partitioned(orc, gj, cuda, node_keys, leaf_keys):
    import torch

    rng = np.random.default_rng(node_keys)
    col = column(rng, 200003)
    pr = probes_for(rng, col, 300000)
    ix = gj.btree_index(btree_node_keys=node_keys, btree_leaf_keys=leaf_keys,
                        index_memory=gj.INDEX_MEMORY_HOST).construct(None, host_column(torch, col))
    assert ix.host_memory() > 0
    d_pr = to_dev(torch, pr)
    erows, epos = orc.pairs_from_positions(orc.exact_lookup(col, pr))
    out, cnt = ix.inlj_pairs(d_pr)
    rows, pos = pairs_of(out, cnt)
    np.testing.assert_array_equal(rows, erows)
    np.testing.assert_array_equal(pos, epos)
    _, prs, cnt = ix.partitioned_inlj(d_pr, radix_bits=8, positions=False, pairs=True)
    rows, pos = pairs_of(prs, cnt)
    order = np.argsort(rows, kind="stable")
    np.testing.assert_array_equal(rows[order], erows)
    np.testing.assert_array_equal(pos[order], epos)


@pytest.mark.parametrize("kind", ["btree", "radix_spline", "learned"])
def test_host_column_device_index(orc, gj, cuda, kind):
    # column in Grace memory, the index's own arrays (inner levels, spline,
    # models) in HBM
    import torch

    rng = np.random.default_rng(41)
    col = column(rng, 1 << 17)
    pr = probes_for(rng, col, 1 << 16)
    ix = gj.make_index(kind).construct(None, host_column(torch, col))
    assert ix.host_memory() == 0
    got = from_dev_u32(ix.lookup(to_dev(torch, pr)))
    np.testing.assert_array_equal(got, expected(orc, kind, col, pr))


def test_device_index_has_no_host_arrays(gj, cuda):
    import torch

    rng = np.random.default_rng(5)
    col = column(rng, 4096)
    ix = gj.btree_index().construct(None, to_dev(torch, col))
    assert ix.host_memory() == 0


def test_host_index_rejects_bad_placement(gj, cuda):
    import torch

    rng = np.random.default_rng(6)
    col = column(rng, 4096)
    with pytest.raises(gj.GJError):
        gj.btree_index(index_memory=7).construct(None, to_dev(torch, col))
    with pytest.raises(ValueError):
        gj.btree_index().construct(None, torch.from_numpy(col.view(np.int64)))  # pageable host memory
