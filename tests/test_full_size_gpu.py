"""Parity at the benchmarked index size: a 2^26-key uniform column (the
INLJ configuration's build side) with each index kind's default build -- for
the B+tree that is the 14-bit compressed nodes with 4-key leaves and the
default start table of 2^20 buckets (about 64 keys a bucket), six compressed levels -- probed by 2^24
Zipf(0.5) probes with permuted ranks plus 5 % absent keys.  Every position
and every pair is compared with the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N_LOG2, M_LOG2 = 26, 24


@pytest.fixture(scope="module")
def full_size(gj, orc, cuda):
    keys = gj.generate_sorted_keys(1 << N_LOG2, gj.DIST_UNIFORM, 1 << 63, seed=20261203)
    probes = gj.generate_probes(keys, 1 << M_LOG2, theta=0.5, absent_fraction=0.05, seed=20261204)
    h_keys = keys.cpu().numpy().view(np.uint64)
    h_probes = probes.cpu().numpy().view(np.uint64)
    lb, ex = orc.fast_positions(h_keys, h_probes, orc.hardware_threads())
    return keys, probes, lb, ex


@pytest.mark.parametrize("kind", ["btree", "harmonia", "radix_spline", "binary_search", "learned", "hash"])
def test_full_size_positions_and_pairs(gj, orc, full_size, kind):
    keys, probes, lb, ex = full_size
    want = ex if kind in ("btree", "harmonia", "hash") else lb
    ix = gj.make_index(kind).construct(None, keys)
    got = ix.lookup(probes).cpu().numpy().view(np.uint32)
    bad = np.nonzero(got != want)[0]
    assert len(bad) == 0, f"{kind}: {len(bad)} of {len(want)} positions differ, first rows {bad[:5]}"
    pairs, cnt = ix.inlj_pairs(probes)
    c = int(cnt.item())
    p = pairs[: 2 * c].cpu().numpy().view(np.uint32).reshape(-1, 2)
    rows, pos = orc.pairs_from_positions(want)
    np.testing.assert_array_equal(p[:, 0], rows)
    np.testing.assert_array_equal(p[:, 1], pos)
    ix.free()

