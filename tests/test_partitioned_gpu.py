"""The partitioned INLJ's directory on the columns that stress it, against
the oracle: a column whose keys crowd into a few buckets (long lower-bound
ranges, searched past the first sectors), a column that is not 32-byte
aligned, columns of a few keys, clustered keys with long gaps (buckets
filled by the prefix maximum), narrower key ranges, a run of consecutive
keys, probes outside the key range, several windows, and the directory
built per call or kept with the index.
Positions must equal the oracle's per probe row, the pairs as a set (their
order across tiles is not fixed)."""
import numpy as np
import pytest

from test_lookup_gpu import column, expected, from_dev_u32, probes_for, to_dev

pytestmark = pytest.mark.gpu

KINDS = ["btree", "binary_search", "radix_spline", "hash", "learned", "no_op"]


def _column(case, rng):
    if case == "wide":
        # 2^19 dense keys in partition 0 (2^17 sectors: too wide for the
        # directory) and 2^19 keys spread over the rest of the range
        dense = np.arange(1000, 1000 + (1 << 19), dtype=np.uint64)
        sparse = np.unique(rng.integers(1 << 40, 1 << 63, size=(1 << 19) + 4096, dtype=np.uint64))[: 1 << 19]
        return np.concatenate([dense, sparse])
    if case == "clusters":
        starts = np.sort(rng.choice(1 << 50, size=64, replace=False).astype(np.uint64)) << np.uint64(10)
        col = np.concatenate([s + np.arange(4096, dtype=np.uint64) * np.uint64(3) for s in starts])
        return np.unique(col)
    if case == "tiny":
        return np.array([5, 17, 1 << 40, (1 << 64) - 2, (1 << 64) - 1], dtype=np.uint64)
    # narrower key ranges (directory buckets a few keys wide), and a run of
    # 3000 consecutive keys inside one bucket among sparse ones
    if case == "range48":
        return column(rng, 100_003, upper=1 << 48)
    if case == "range52":
        return column(rng, 1 << 17, upper=1 << 52)
    if case == "run":
        col = column(rng, 1 << 17, upper=1 << 49)
        return np.unique(np.concatenate([col, np.arange(1 << 40, (1 << 40) + 3000, dtype=np.uint64)]))
    return column(rng, 100_003)  # "unaligned" and "plain"


@pytest.mark.parametrize("prepared", [False, True])
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("case", ["wide", "unaligned", "tiny", "clusters", "range48", "range52", "run"])
def test_partitioned_directory_cases(orc, gj, cuda, kind, case, prepared):
    import torch

    rng = np.random.default_rng(len(case) * 31 + len(kind))
    col = _column(case, rng)
    pr = probes_for(rng, col, 60_000)
    if case == "unaligned":
        d_all = to_dev(torch, np.concatenate([np.array([0], dtype=np.uint64), col]))
        d_col = d_all[1:]  # 8-byte offset: not 32-byte aligned
        assert d_col.data_ptr() % 32 != 0
    else:
        d_col = to_dev(torch, col)
    ix = gj.make_index(kind).construct(None, d_col)
    if prepared:  # the directory kept with the index instead of built per call
        ix.prepare_partitioned()
    exp = expected(orc, kind, col, pr)
    erows, epos = orc.pairs_from_positions(exp)
    # the wide scatter (fanout 2^8 and up), the narrow one (below 2^8), and the
    # default fanout (0: about 2^20 keys a partition, from 2^5)
    for bits, window in ((8, 0), (12, 0), (10, 7777), (5, 0), (6, 20000), (0, 0)):
        pos, prs, cnt = ix.partitioned_inlj(to_dev(torch, pr), window_size=window, radix_bits=bits, positions=True,
                                            pairs=True)
        got = from_dev_u32(pos)
        bad = np.nonzero(got != exp)[0]
        assert len(bad) == 0, f"{kind}/{case}/2^{bits}: {len(bad)} positions differ, rows {bad[:5]}"
        c = int(cnt.item())
        a = prs[: 2 * c].cpu().numpy().view(np.uint32).reshape(-1, 2)
        order = np.argsort(a[:, 0], kind="stable")
        np.testing.assert_array_equal(a[order, 0], erows, err_msg=f"{kind}/{case}/2^{bits}")
        np.testing.assert_array_equal(a[order, 1], epos, err_msg=f"{kind}/{case}/2^{bits}")


@pytest.mark.parametrize("kind", ["btree", "binary_search"])
def test_partitioned_skewed_probes(orc, gj, cuda, kind):
    # Nearly every probe falls into one narrow key range (one partition, a
    # few directory buckets), every 64th into the lowest keys, some are
    # absent: one partition far fuller than the others, across windows.
    import torch

    rng = np.random.default_rng(77)
    col = column(rng, 1 << 18)
    m = 300_000
    hot = col[(1 << 17):(1 << 17) + 512]
    pr = hot[rng.integers(0, len(hot), m)]
    pr[::64] = col[rng.integers(0, 64, len(pr[::64]))]
    pr[::97] = pr[::97] + np.uint64(1)  # some absent keys
    ix = gj.make_index(kind).construct(None, to_dev(torch, col))
    exp = expected(orc, kind, col, pr)
    erows, epos = orc.pairs_from_positions(exp)
    for prepared in (False, True):
        if prepared:
            ix.prepare_partitioned()
        for bits, window in ((8, 0), (11, 0), (8, 65536), (5, 0), (7, 65536)):
            pos, prs, cnt = ix.partitioned_inlj(to_dev(torch, pr), window_size=window, radix_bits=bits,
                                                positions=True, pairs=True)
            np.testing.assert_array_equal(from_dev_u32(pos), exp, err_msg=f"{kind}/2^{bits}/{window}")
            c = int(cnt.item())
            a = prs[: 2 * c].cpu().numpy().view(np.uint32).reshape(-1, 2)
            order = np.argsort(a[:, 0], kind="stable")
            np.testing.assert_array_equal(a[order, 0], erows)
            np.testing.assert_array_equal(a[order, 1], epos)
