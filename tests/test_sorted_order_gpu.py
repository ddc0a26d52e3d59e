"""Block-wise sorted probe order (the reference's bws_lookup): lookups give
the plain lookup's positions in probe order, pairs the plain pairs' set
(tile by tile, key order inside a tile), for every index kind, ragged and
skewed probe sets; the ordering autotuner returns one of the two orders."""
import numpy as np
import pytest

from test_join_gpu import pairs_of
from test_lookup_gpu import column, expected, from_dev_u32, probes_for, to_dev

pytestmark = pytest.mark.gpu

KINDS = ["binary_search", "btree", "harmonia", "radix_spline", "learned", "hash", "no_op"]


def skewed_probes(rng, col, m):
    # a few hot keys repeated many times, absent keys, both ends
    hot = col[rng.integers(0, len(col), 16)]
    return np.concatenate([rng.choice(hot, m // 2), probes_for(rng, col, m // 2),
                           np.array([0, (1 << 64) - 1], dtype=np.uint64)]).astype(np.uint64)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("m", [1, 1023, 1025, 4096 * 4 + 7, 200003])
def test_sorted_lookup_matches_oracle(orc, gj, cuda, kind, m):
    import torch

    rng = np.random.default_rng(m + len(kind))
    col = column(rng, 32 * 3001)
    pr = skewed_probes(rng, col, m)[:m]
    ix = gj.make_index(kind).construct(None, to_dev(torch, col))
    got = from_dev_u32(ix.lookup_sorted(to_dev(torch, pr)))
    np.testing.assert_array_equal(got, expected(orc, kind, col, pr), err_msg=f"{kind} m={m}")


@pytest.mark.parametrize("kind", ["btree", "harmonia", "radix_spline", "hash"])
@pytest.mark.parametrize("m", [0, 1, 1024, 3000, 100003])
def test_sorted_pairs_match_oracle(orc, gj, cuda, kind, m):
    import torch

    rng = np.random.default_rng(7 * m + 3)
    col = column(rng, 32 * 1563)
    pr = skewed_probes(rng, col, max(m, 2))[:m]
    ix = gj.make_index(kind).construct(None, to_dev(torch, col))
    out, cnt = ix.inlj_pairs_sorted(to_dev(torch, pr))
    rows, pos = pairs_of(out, cnt)
    erows, epos = orc.pairs_from_positions(expected(orc, kind, col, pr))
    # tile by tile in probe order: every pair's row lies in its tile's range
    assert np.all(np.diff(rows.astype(np.int64) // 1024) >= 0)
    order = np.argsort(rows, kind="stable")
    np.testing.assert_array_equal(rows[order], erows)
    np.testing.assert_array_equal(pos[order], epos)


def test_autotune_ordering(orc, gj, cuda):
    import torch

    rng = np.random.default_rng(12)
    col = column(rng, 1 << 16)
    pr = skewed_probes(rng, col, 1 << 18)
    d_pr = to_dev(torch, pr)
    ix = gj.btree_index().construct(None, to_dev(torch, col))
    order, ms = ix.autotune_ordering(d_pr)
    assert order in (gj.ORDER_PROBE, gj.ORDER_SORTED_TILES, gj.ORDER_PARTITIONED) and ms > 0
    erows, epos = orc.pairs_from_positions(orc.exact_lookup(col, pr))
    # every candidate order gives the same set of pairs
    runs = {gj.ORDER_PROBE: lambda: ix.inlj_pairs(d_pr), gj.ORDER_SORTED_TILES: lambda: ix.inlj_pairs_sorted(d_pr),
            gj.ORDER_PARTITIONED: lambda: ix.partitioned_inlj(d_pr, positions=False, pairs=True)[1:]}
    for o, run in runs.items():
        out, cnt = run()
        rows, pos = pairs_of(out, cnt)
        order_ = np.argsort(rows, kind="stable")
        np.testing.assert_array_equal(rows[order_], erows, err_msg=f"order {o}")
        np.testing.assert_array_equal(pos[order_], epos, err_msg=f"order {o}")
