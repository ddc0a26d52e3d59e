"""Parity of the CUDA probe kernels (through the C ABI) against the CPU oracle.

Bit-exact: every position must equal the oracle's restatement of the
reference lookup for the index kind."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LOWER_BOUND_KINDS = ("binary_search", "radix_spline")
EXACT_KINDS = ("btree", "harmonia")


def to_dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def from_dev_u32(t):
    return t.cpu().numpy().view(np.uint32)


def column(rng, n, upper=1 << 63):
    while True:
        k = np.unique(rng.integers(0, upper, size=n + n // 4 + 16, dtype=np.uint64))
        if len(k) >= n:
            return np.sort(rng.choice(k, size=n, replace=False))


def probes_for(rng, col, m):
    n = len(col)
    parts = [col[rng.integers(0, n, size=m)], rng.integers(0, 1 << 63, size=m // 3 + 1, dtype=np.uint64),
             np.array([0, col[0], col[-1], col[-1] + 1, (1 << 64) - 1, 1 << 63], dtype=np.uint64),
             col[:8], col[-8:], col[rng.integers(0, n, size=8)].repeat(4)]
    if col[0] > 0:
        parts.append(np.array([col[0] - 1], dtype=np.uint64))
    return np.concatenate(parts).astype(np.uint64)


def expected(orc, kind, col, pr):
    if kind in LOWER_BOUND_KINDS or kind == "learned":
        return orc.bs_lookup(col, pr)
    if kind == "no_op":
        return np.full(len(pr), 0xFFFFFFFF, dtype=np.uint32)
    return orc.exact_lookup(col, pr)


@pytest.mark.parametrize("kind", ["binary_search", "btree", "harmonia", "radix_spline", "hash"])
@pytest.mark.parametrize("n", [32, 64, 96, 2048, 32 * 1090, 100000 - 100000 % 32, 1 << 20])
def test_lookup_matches_oracle(orc, gj, cuda, kind, n):
    import torch

    rng = np.random.default_rng(n * 7 + len(kind))
    col = column(rng, n)
    pr = probes_for(rng, col, 5000)
    d_col, d_pr = to_dev(torch, col), to_dev(torch, pr)
    ix = gj.make_index(kind).construct(col, d_col)
    got = from_dev_u32(ix.lookup(d_pr))
    exp = expected(orc, kind, col, pr)
    bad = np.nonzero(got != exp)[0]
    assert len(bad) == 0, f"{kind} n={n}: {len(bad)} mismatches, first {bad[:5]} got {got[bad[:5]]} exp {exp[bad[:5]]}"


@pytest.mark.parametrize("kind", ["binary_search", "btree", "radix_spline", "hash"])
@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 63, 65, 4095, 4097])
def test_lookup_small_ragged_sizes(orc, gj, cuda, kind, n):
    import torch

    rng = np.random.default_rng(n + 100)
    col = column(rng, n, upper=1 << 20)
    pr = np.concatenate([np.arange(0, (1 << 20) + 10, 997, dtype=np.uint64), col])
    ix = gj.make_index(kind).construct(None, to_dev(torch, col))
    got = from_dev_u32(ix.lookup(to_dev(torch, pr)))
    np.testing.assert_array_equal(got, expected(orc, kind, col, pr))


@pytest.mark.parametrize("node_keys,leaf_keys", [(4, 4), (4, 16), (4, 64), (8, 8), (8, 16), (16, 16), (32, 16),
                                                  (64, 16), (64, 64), (4, 1), (16, 2), (64, 256), (7, 1), (7, 4),
                                                  (7, 8), (7, 64), (15, 1), (15, 4), (15, 8), (15, 64)])
def test_btree_node_widths(orc, gj, cuda, node_keys, leaf_keys):
    import torch

    rng = np.random.default_rng(node_keys * 100 + leaf_keys)
    for n in sorted({max(1, x) for x in (1, leaf_keys - 1, leaf_keys, leaf_keys + 1, node_keys * leaf_keys + 3, 123457)}):
        col = column(rng, n)
        pr = probes_for(rng, col, 3000)
        ix = gj.btree_index(btree_node_keys=node_keys, btree_leaf_keys=leaf_keys).construct(None, to_dev(torch, col))
        got = from_dev_u32(ix.lookup(to_dev(torch, pr)))
        np.testing.assert_array_equal(got, orc.exact_lookup(col, pr), err_msg=f"W={node_keys} L={leaf_keys} n={n}")


def compressed_key_sets(rng):
    top = (1 << 64) - 1
    dense = np.arange(5, 5 + 70000, dtype=np.uint64)
    runs = np.concatenate([np.arange(1000, 41000, dtype=np.uint64),
                           np.arange(1 << 62, (1 << 62) + 30000, dtype=np.uint64) * np.uint64(3),
                           np.sort(rng.choice(np.arange(1 << 40, (1 << 40) + 200000, dtype=np.uint64), 50000,
                                              replace=False))])
    near_top = np.sort(np.uint64(top) - np.arange(0, 90000, dtype=np.uint64) * np.uint64(7))
    mixed = np.unique(np.concatenate([column(rng, 60000), dense[:20000] * np.uint64(1 << 30)]))
    return {"dense": dense, "runs": np.unique(runs), "near_top": near_top, "mixed": mixed}


@pytest.mark.parametrize("node_keys", [7, 15])
@pytest.mark.parametrize("leaf_keys", [1, 8, 64])
def test_btree_compressed_nodes(orc, gj, cuda, node_keys, leaf_keys):
    # one-sector nodes of 32-bit (width 7) or 15-bit (width 15) deltas: dense
    # keys (shift 0), runs separated by huge gaps (large shifts, separators
    # sharing a bucket -> exact comparisons), keys next to 2^64 - 1, and probes
    # on every key and both neighbours
    import torch

    rng = np.random.default_rng(leaf_keys + 7)
    for name, col in compressed_key_sets(rng).items():
        col = np.ascontiguousarray(col, dtype=np.uint64)
        pr = np.concatenate([col, col - np.uint64(1), col + np.uint64(1),
                             rng.integers(0, 1 << 63, 5000, dtype=np.uint64) * np.uint64(2),
                             np.array([0, 1, (1 << 64) - 1, (1 << 64) - 2, 1 << 63], dtype=np.uint64)])
        ix = gj.btree_index(btree_node_keys=node_keys, btree_leaf_keys=leaf_keys).construct(None, to_dev(torch, col))
        d_pr = to_dev(torch, pr)
        want = orc.exact_lookup(col, pr)
        got = from_dev_u32(ix.lookup(d_pr))
        np.testing.assert_array_equal(got, want, err_msg=f"{name} W={node_keys} L={leaf_keys}")
        # the partitioned kernels search sorted tiles with the default L2 class
        got = np.full(len(pr), 0xFFFFFFFF, dtype=np.uint32)
        _, prs, cnt = ix.partitioned_inlj(d_pr, radix_bits=8, positions=False, pairs=True)
        p = prs[: 2 * int(cnt.item())].cpu().numpy().view(np.uint32).reshape(-1, 2)
        got[p[:, 0]] = p[:, 1]
        np.testing.assert_array_equal(got, want, err_msg=f"partitioned {name} W={node_keys} L={leaf_keys}")


@pytest.mark.parametrize("node_keys", [4, 7, 15, 64])
@pytest.mark.parametrize("start_bits", [1, 6, 24])
def test_btree_start_table(orc, gj, cuda, node_keys, start_bits):
    # scattered lookups start at their key bucket's deepest shared node: from
    # two buckets to more buckets than keys, on dense keys, runs with huge
    # gaps (many empty buckets) and keys next to 2^64 - 1
    import torch

    rng = np.random.default_rng(node_keys * 31 + start_bits)
    for name, col in compressed_key_sets(rng).items():
        col = np.ascontiguousarray(col, dtype=np.uint64)
        pr = np.concatenate([col, col - np.uint64(1), col + np.uint64(1),
                             rng.integers(0, 1 << 63, 5000, dtype=np.uint64) * np.uint64(2),
                             np.array([0, 1, (1 << 64) - 1, (1 << 64) - 2, 1 << 63], dtype=np.uint64)])
        ix = gj.btree_index(btree_node_keys=node_keys, btree_start_bits=start_bits).construct(None,
                                                                                            to_dev(torch, col))
        got = from_dev_u32(ix.lookup(to_dev(torch, pr)))
        np.testing.assert_array_equal(got, orc.exact_lookup(col, pr),
                                      err_msg=f"{name} W={node_keys} start bits {start_bits}")


def test_btree_start_table_size(gj, cuda):
    import torch

    # 16 bytes per bucket; buckets of 2^shift keys cover [min, max]
    col = torch.arange(0, 1 << 16, dtype=torch.int64, device="cuda") * 5
    key_range = 5 * ((1 << 16) - 1)

    def entries(bits):
        shift = max(0, key_range.bit_length() - bits)
        return (key_range >> shift) + 1

    small = gj.btree_index(btree_start_bits=4).construct(None, col).memory_consumption()
    large = gj.btree_index(btree_start_bits=16).construct(None, col).memory_consumption()
    assert large - small == (entries(16) - entries(4)) * 16
    with pytest.raises(gj.GJError):
        gj.btree_index(btree_start_bits=25).construct(None, col)


def test_unaligned_column(orc, gj, cuda):
    # columns that start 8 and 16 bytes into an allocation: 32-byte sector loads must not be used
    import torch

    rng = np.random.default_rng(8)
    col = column(rng, 32 * 3000)
    pr = to_dev(torch, probes_for(rng, col, 5000))
    h_pr = pr.cpu().numpy().view(np.uint64)
    for shift in (1, 2):
        buf = torch.zeros(len(col) + shift, dtype=torch.int64, device="cuda")
        buf[shift:] = to_dev(torch, col)
        d_col = buf[shift:]
        assert d_col.data_ptr() % 32 == 8 * shift
        for kind in ("btree", "harmonia", "binary_search", "radix_spline", "learned"):
            ix = gj.make_index(kind).construct(None, d_col)
            exp = orc.exact_lookup(col, h_pr) if kind in ("btree", "harmonia") else orc.bs_lookup(col, h_pr)
            np.testing.assert_array_equal(from_dev_u32(ix.lookup(pr)), exp, err_msg=f"{kind} shift {shift}")


@pytest.mark.parametrize("cache_keys", [0, 2, 64, 4096])
def test_binary_search_cache_settings(orc, gj, cuda, cache_keys):
    import torch

    rng = np.random.default_rng(cache_keys + 1)
    for n in (100, 5000, 300001):
        col = column(rng, n)
        pr = probes_for(rng, col, 4000)
        ix = gj.binary_search_index(bs_cache_keys=cache_keys).construct(None, to_dev(torch, col))
        np.testing.assert_array_equal(from_dev_u32(ix.lookup(to_dev(torch, pr))), orc.bs_lookup(col, pr))


@pytest.mark.parametrize("bits,err", [(18, 32), (8, 4), (20, 0), (2, 64)])
def test_radix_spline_parameters(orc, gj, cuda, bits, err):
    import torch

    rng = np.random.default_rng(bits * 100 + err)
    col = column(rng, 200000)
    pr = probes_for(rng, col, 20000)
    ix = gj.radix_spline_index(rs_radix_bits=bits, rs_max_error=err).construct(None, to_dev(torch, col))
    np.testing.assert_array_equal(from_dev_u32(ix.lookup(to_dev(torch, pr))), orc.bs_lookup(col, pr))


def test_harmonia_golden_fixture(orc, gj, cuda):
    import os

    import torch

    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "harmonia.npz"))
    sizes = sorted({int(k.split("_")[1]) for k in d.files})
    for n in sizes:
        col, pr = d[f"harmonia_{n}_col"], d[f"harmonia_{n}_probes"]
        ix = gj.harmonia_index().construct(None, to_dev(torch, col))
        np.testing.assert_array_equal(from_dev_u32(ix.lookup(to_dev(torch, pr))), d[f"harmonia_{n}_pos"],
                                      err_msg=f"n={n}")


def test_btree_golden_fixture(orc, gj, cuda):
    import os

    import torch

    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "btree.npz"))
    sizes = sorted({int(k.split("_")[1]) for k in d.files})
    for n in sizes:
        col, pr = d[f"btree_{n}_col"], d[f"btree_{n}_probes"]
        ix = gj.btree_index().construct(None, to_dev(torch, col))
        np.testing.assert_array_equal(from_dev_u32(ix.lookup(to_dev(torch, pr))), d[f"btree_{n}_pos"],
                                      err_msg=f"n={n}")


def test_no_op_index(gj, cuda):
    import torch

    ix = gj.no_op_index().construct(None, torch.zeros(4, dtype=torch.int64, device="cuda"))
    got = from_dev_u32(ix.lookup(torch.arange(100, dtype=torch.int64, device="cuda")))
    assert np.all(got == 0xFFFFFFFF)


def test_empty_probe_column(gj, cuda):
    import torch

    col = torch.arange(0, 64, dtype=torch.int64, device="cuda") * 3
    for kind in ("binary_search", "btree", "harmonia", "radix_spline"):
        ix = gj.make_index(kind).construct(None, col)
        out = ix.lookup(torch.empty(0, dtype=torch.int64, device="cuda"))
        assert out.numel() == 0


def test_build_errors(gj, cuda):
    import torch

    unsorted = torch.tensor([5, 3, 9, 10], dtype=torch.int64, device="cuda")
    with pytest.raises(gj.GJError) as e:
        gj.btree_index().construct(None, unsorted)
    assert e.value.code == 6
    dup = torch.tensor([1, 2, 2, 3], dtype=torch.int64, device="cuda")
    with pytest.raises(gj.GJError):
        gj.binary_search_index().construct(None, dup)
    not32 = torch.arange(0, 33, dtype=torch.int64, device="cuda")
    with pytest.raises(gj.GJError) as e:
        gj.harmonia_index().construct(None, not32)
    assert e.value.code == 1
    with pytest.raises(gj.GJError):
        gj.btree_index(btree_node_keys=48).construct(None, torch.arange(0, 100, dtype=torch.int64, device="cuda"))
    with pytest.raises(gj.GJError):
        gj.btree_index(btree_node_keys=64, btree_leaf_keys=24).construct(
            None, torch.arange(0, 100, dtype=torch.int64, device="cuda"))
    with pytest.raises(gj.GJError):
        gj.btree_index().construct(None, torch.empty(0, dtype=torch.int64, device="cuda"))


def test_memory_consumption(gj, cuda):
    import torch

    col = torch.arange(0, 1 << 16, dtype=torch.int64, device="cuda") * 5
    assert gj.binary_search_index(bs_cache_keys=0).construct(None, col).memory_consumption() == 0
    assert gj.btree_index().construct(None, col).memory_consumption() > 0
    assert gj.harmonia_index().construct(None, col).memory_consumption() > 0
    assert gj.radix_spline_index().construct(None, col).memory_consumption() > 0


def test_lookup_on_side_stream(orc, gj, cuda):
    import torch

    rng = np.random.default_rng(77)
    col = column(rng, 50000)
    pr = probes_for(rng, col, 50000)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        d_col, d_pr = to_dev(torch, col), to_dev(torch, pr)
        ix = gj.btree_index().construct(None, d_col, stream=s)
        out = ix.lookup(d_pr, stream=s)
    s.synchronize()
    np.testing.assert_array_equal(from_dev_u32(out), orc.exact_lookup(col, pr))


def test_hash_index_edge_keys(orc, gj, cuda):
    # keys at both ends of the 64-bit range (UINT64_MAX is storable: empty
    # slots are marked in the position word), dense runs that collide in the
    # table's low bits, and probes on every key and both neighbours
    import torch

    rng = np.random.default_rng(77)
    for name, col in compressed_key_sets(rng).items():
        col = np.ascontiguousarray(col, dtype=np.uint64)
        if name == "near_top":
            assert col[-1] == np.uint64((1 << 64) - 1)
        pr = np.concatenate([col, col - np.uint64(1), col + np.uint64(1),
                             np.array([0, 1, (1 << 64) - 1, 1 << 63], dtype=np.uint64)])
        ix = gj.hash_index().construct(None, to_dev(torch, col))
        assert ix.memory_consumption() >= 16 * 2 * len(col)
        got = from_dev_u32(ix.lookup(to_dev(torch, pr)))
        np.testing.assert_array_equal(got, orc.exact_lookup(col, pr), err_msg=name)


@pytest.mark.parametrize("kind", ["harmonia", "binary_search"])
@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5])
def test_warp_cooperative_lookup(orc, gj, cuda, kind, degree):
    # gj_index_lookup_cooperative: the reference's warp-collective protocol
    # (groups of 2^degree lanes), the per-thread results; ragged probe counts
    # leave the last warp partly inactive
    import torch

    rng = np.random.default_rng(degree)
    for n in (32, 4096, 1 << 18):
        col = column(rng, n)
        pr = probes_for(rng, col, 30001)
        ix = gj.make_index(kind).construct(None, to_dev(torch, col))
        got = from_dev_u32(ix.lookup_cooperative(to_dev(torch, pr), degree))
        np.testing.assert_array_equal(got, expected(orc, kind, col, pr), err_msg=f"n={n}")
        ix.free()


def test_warp_cooperative_lookup_rejects_other_kinds(gj, cuda):
    import torch

    keys = gj.generate_sorted_keys(1 << 10, gj.DIST_UNIFORM, 1 << 63, seed=3)
    ix = gj.make_index("btree").construct(None, keys)
    with pytest.raises(gj.GJError):
        ix.lookup_cooperative(keys[:10], 4)
    ix2 = gj.make_index("harmonia").construct(None, keys)
    with pytest.raises(gj.GJError):
        ix2.lookup_cooperative(keys[:10], 6)
