"""Join materialisation, partitioned INLJ and the star-join aggregate on the
GPU against the CPU oracle."""
import ctypes

import numpy as np
import pytest

from test_lookup_gpu import column, expected, from_dev_u32, probes_for, to_dev

pytestmark = pytest.mark.gpu


def pairs_of(out_pairs, count):
    c = int(count.item())
    a = out_pairs[: 2 * c].cpu().numpy().view(np.uint32).reshape(-1, 2)
    return a[:, 0].copy(), a[:, 1].copy()


@pytest.mark.parametrize("ordered", [True, False])
@pytest.mark.parametrize("kind", ["binary_search", "btree", "harmonia", "radix_spline", "hash"])
@pytest.mark.parametrize("m", [0, 1, 31, 2047, 2048, 2049, 100003])
def test_inlj_pairs_match_oracle(orc, gj, cuda, kind, m, ordered):
    # in probe order, or (gj_inlj_pairs_unordered) the same set
    import torch

    rng = np.random.default_rng(m + 3)
    col = column(rng, 32 * 1000)
    pr = probes_for(rng, col, max(m, 1))[:m]
    ix = gj.make_index(kind).construct(None, to_dev(torch, col))
    out, cnt = ix.inlj_pairs(to_dev(torch, pr) if m else torch.empty(0, dtype=torch.int64, device="cuda"),
                             ordered=ordered)
    rows, pos = pairs_of(out, cnt)
    if not ordered:
        order = np.argsort(rows, kind="stable")
        rows, pos = rows[order], pos[order]
    erows, epos = orc.pairs_from_positions(expected(orc, kind, col, pr))
    np.testing.assert_array_equal(rows, erows)
    np.testing.assert_array_equal(pos, epos)


@pytest.mark.parametrize("kind", ["btree", "learned", "no_op"])
@pytest.mark.parametrize("m", [4095, 4096, 4097, 3 * 1000 * 1000 + 17])
def test_inlj_pairs_compaction_tiles(orc, gj, cuda, kind, m):
    # plain pairs are positions first (parked in the upper half of the pairs
    # buffer), then an ordered compaction over 4096-probe tiles with a
    # look-back over many predecessors; the workspace is reused across calls
    import torch

    rng = np.random.default_rng(m)
    col = column(rng, 32 * 4000)
    pr = probes_for(rng, col, m)[:m]
    ix = gj.make_index(kind).construct(None, to_dev(torch, col))
    d_pr = to_dev(torch, pr)
    ws = None
    for _ in range(2):
        out, cnt = ix.inlj_pairs(d_pr, workspace=ws)
        if ws is None:
            import ctypes

            need = ctypes.c_size_t(0)
            gj.lib().gj_inlj_pairs_workspace_size(m, ctypes.byref(need))
            ws = torch.empty(need.value, dtype=torch.uint8, device="cuda")
            out, cnt = ix.inlj_pairs(d_pr, workspace=ws)
        ix.inlj_pairs_status(ws, m)
        rows, pos = pairs_of(out, cnt)
        erows, epos = orc.pairs_from_positions(expected(orc, kind, col, pr))
        np.testing.assert_array_equal(rows, erows)
        np.testing.assert_array_equal(pos, epos)


def test_inlj_pairs_all_absent(orc, gj, cuda):
    import torch

    col = np.arange(0, 3200, dtype=np.uint64) * 2
    pr = np.arange(1, 6401, 2, dtype=np.uint64)  # odd keys: none present
    ix = gj.btree_index().construct(None, to_dev(torch, col))
    out, cnt = ix.inlj_pairs(to_dev(torch, pr))
    assert int(cnt.item()) == 0


@pytest.mark.parametrize("bits", [1, 4, 8, 12])
def test_range_partition_matches_oracle(orc, gj, cuda, bits):
    import torch

    rng = np.random.default_rng(bits)
    keys = rng.integers(0, 1 << 48, 300001, dtype=np.uint64)
    min_key, shift = 1 << 20, 48 - bits
    rel = gj.range_partition(to_dev(torch, keys), min_key, shift, bits)
    ok, orows, offs = orc.range_partition(keys, min_key, shift, bits)
    np.testing.assert_array_equal(rel.offsets.cpu().numpy().view(np.uint64), offs)
    gk = rel.keys.cpu().numpy().view(np.uint64)
    gr = rel.rows.cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(keys[gr], gk)
    # same tuples per partition (the order inside a partition is not fixed)
    for p in range(1 << bits):
        a, b = int(offs[p]), int(offs[p + 1])
        np.testing.assert_array_equal(np.sort(gr[a:b]), np.sort(orows[a:b]))


@pytest.mark.parametrize("kind", ["binary_search", "btree", "harmonia", "radix_spline"])
@pytest.mark.parametrize("window", [0, 1000, 65536])
def test_partitioned_inlj_equals_plain(orc, gj, cuda, kind, window):
    import torch

    rng = np.random.default_rng(window + 17)
    col = column(rng, 32 * 5000)
    pr = probes_for(rng, col, 120000)
    ix = gj.make_index(kind).construct(None, to_dev(torch, col))
    pos, prs, cnt = ix.partitioned_inlj(to_dev(torch, pr), window_size=window, radix_bits=0, positions=True,
                                        pairs=True)
    exp = expected(orc, kind, col, pr)
    np.testing.assert_array_equal(from_dev_u32(pos), exp)
    rows, bpos = pairs_of(prs, cnt)
    erows, epos = orc.pairs_from_positions(exp)
    order = np.argsort(rows, kind="stable")
    np.testing.assert_array_equal(rows[order], erows)
    np.testing.assert_array_equal(bpos[order], epos)


@pytest.mark.parametrize("bits", [8, 10, 12])
def test_partitioned_inlj_fanouts(orc, gj, cuda, bits):
    import torch

    rng = np.random.default_rng(bits + 50)
    col = column(rng, 1 << 18)
    pr = probes_for(rng, col, 200000)
    ix = gj.btree_index().construct(None, to_dev(torch, col))
    pos, prs, cnt = ix.partitioned_inlj(to_dev(torch, pr), radix_bits=bits, pairs=True)
    exp = orc.exact_lookup(col, pr)
    np.testing.assert_array_equal(from_dev_u32(pos), exp)
    rows, bpos = pairs_of(prs, cnt)
    erows, epos = orc.pairs_from_positions(exp)
    order = np.argsort(rows, kind="stable")
    np.testing.assert_array_equal(rows[order], erows)
    np.testing.assert_array_equal(bpos[order], epos)


@pytest.mark.parametrize("kind", ["btree", "harmonia", "radix_spline", "binary_search", "learned", "hash"])
def test_partitioned_pairs_sorted_tiles(orc, gj, cuda, kind):
    # tiles of equal keys, a tile spanning the whole key range, many windows
    import torch

    rng = np.random.default_rng(99)
    col = column(rng, 32 * 20000)
    pr = np.concatenate([np.full(5000, col[777], dtype=np.uint64), probes_for(rng, col, 300000),
                         np.array([0, (1 << 64) - 1], dtype=np.uint64), np.full(3000, col[-1], dtype=np.uint64)])
    ix = gj.make_index(kind).construct(None, to_dev(torch, col))
    exp = expected(orc, kind, col, pr)
    erows, epos = orc.pairs_from_positions(exp)
    for window, bits in ((len(pr), 8), (70001, 10), (4096, 12)):
        _, prs, cnt = ix.partitioned_inlj(to_dev(torch, pr), window_size=window, radix_bits=bits, positions=False,
                                          pairs=True)
        rows, bpos = pairs_of(prs, cnt)
        order = np.argsort(rows, kind="stable")
        np.testing.assert_array_equal(rows[order], erows, err_msg=f"{kind} window {window}")
        np.testing.assert_array_equal(bpos[order], epos, err_msg=f"{kind} window {window}")


def star_inputs(rng, nfact, ndim):
    dim = np.arange(1, ndim + 1, dtype=np.uint64)
    flag = np.zeros(ndim, dtype=np.uint8)
    flag[rng.choice(ndim, ndim // 6, replace=False)] = 1
    fk = rng.integers(1, ndim + 1, nfact).astype(np.uint32)
    fk[rng.integers(0, nfact, nfact // 50)] = ndim + 7  # dangling foreign keys
    date = rng.integers(0, 2556, nfact).astype(np.uint32)
    price = rng.integers(90000, 10500001, nfact).astype(np.int64)
    disc = rng.integers(0, 11, nfact).astype(np.int64)
    return dim, flag, fk, date, price, disc


@pytest.mark.parametrize("sorted_batches", [False, True])
@pytest.mark.parametrize("kind", ["btree", "harmonia", "binary_search", "radix_spline"])
@pytest.mark.parametrize("nfact", [0, 1, 4095, 4097, 600000])
def test_star_join_matches_oracle(orc, gj, cuda, kind, nfact, sorted_batches):
    import torch

    rng = np.random.default_rng(nfact + 1)
    ndim = 20000
    dim, flag, fk, date, price, disc = star_inputs(rng, max(nfact, 1), ndim)
    fk, date, price, disc = fk[:nfact], date[:nfact], price[:nfact], disc[:nfact]
    lo, hi = 1000, 1030
    ix = gj.make_index(kind).construct(None, to_dev(torch, dim))
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dt).cuda()
    out = gj.star_join_sum(ix, t(fk.view(np.int32), torch.int32), t(date.view(np.int32), torch.int32),
                           t(price, torch.int64), t(disc, torch.int64), t(flag, torch.uint8), lo, hi,
                           sorted_batches=sorted_batches)
    num, den = orc.star_join(fk, date, price, disc, dim, flag, lo, hi)
    got = out.cpu().numpy()
    assert int(got[0]) == num and int(got[1]) == den


def test_star_join_full_window_and_empty_window(orc, gj, cuda):
    import torch

    rng = np.random.default_rng(99)
    dim, flag, fk, date, price, disc = star_inputs(rng, 100000, 5000)
    ix = gj.btree_index().construct(None, to_dev(torch, dim))
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dt).cuda()
    args = (t(fk.view(np.int32), torch.int32), t(date.view(np.int32), torch.int32), t(price, torch.int64),
            t(disc, torch.int64), t(flag, torch.uint8))
    for lo, hi in ((0, 1 << 31), (500, 500), (2555, 2556), (100, 900)):
        num, den = orc.star_join(fk, date, price, disc, dim, flag, lo, hi)
        for sorted_batches in (False, True):  # every row passes / none / a few / a third
            got = gj.star_join_sum(ix, *args, lo, hi, sorted_batches=sorted_batches).cpu().numpy()
            assert (int(got[0]), int(got[1])) == (num, den), (lo, hi, sorted_batches)


@pytest.mark.parametrize("ordered", [True, False])
@pytest.mark.parametrize("kind", ["btree", "radix_spline", "learned"])
@pytest.mark.parametrize("m", [0, 1, 4097, 300001])
def test_inlj_pairs_host_buffers(orc, gj, cuda, kind, m, ordered):
    # probes, pairs and count in pinned host memory, read and written by the
    # kernels; unordered: the same set of pairs, tiles in the order they finish
    import torch

    rng = np.random.default_rng(m + 11)
    col = column(rng, 32 * 3000)
    pr = probes_for(rng, col, max(m, 1))[:m]
    ix = gj.make_index(kind).construct(None, to_dev(torch, col))
    h_pr = torch.from_numpy(pr.view(np.int64).copy()).pin_memory()
    h_pairs = torch.full((2 * max(m, 1),), -1, dtype=torch.int32).pin_memory()
    h_cnt = torch.full((1,), -1, dtype=torch.int64).pin_memory()
    ix.inlj_pairs_host(h_pr, h_pairs, h_cnt, ordered=ordered)
    torch.cuda.synchronize()
    c = int(h_cnt[0])
    got = h_pairs[: 2 * c].numpy().view(np.uint32).reshape(-1, 2)
    erows, epos = orc.pairs_from_positions(expected(orc, kind, col, pr))
    if not ordered:
        got = got[np.argsort(got[:, 0], kind="stable")]
    np.testing.assert_array_equal(got[:, 0], erows)
    np.testing.assert_array_equal(got[:, 1], epos)


@pytest.mark.parametrize("ordered", [True, False])
@pytest.mark.parametrize("m", [(1 << 24) + 54321, 3 * (1 << 24) + 5])
def test_inlj_pairs_host_buffers_large(orc, gj, cuda, m, ordered):
    # tens of millions of probes from host buffers: every pair (in probe
    # order unless unordered), the status reads clean
    import torch

    rng = np.random.default_rng(3)
    col = column(rng, 1 << 16)
    pr = col[rng.integers(0, len(col), m)]
    pr[::7] = pr[::7] + np.uint64(1)  # some absent keys
    ix = gj.btree_index().construct(None, to_dev(torch, col))
    h_pr = torch.from_numpy(pr.view(np.int64).copy()).pin_memory()
    h_pairs = torch.full((2 * m,), -1, dtype=torch.int32).pin_memory()
    h_cnt = torch.full((1,), -1, dtype=torch.int64).pin_memory()
    need = ctypes.c_size_t(0)
    gj.lib().gj_inlj_pairs_host_workspace_size(m, ctypes.byref(need))
    ws = torch.empty(need.value, dtype=torch.uint8, device="cuda")
    ix.inlj_pairs_host(h_pr, h_pairs, h_cnt, ws, ordered=ordered)
    torch.cuda.synchronize()
    ix.inlj_pairs_status(ws, m)
    c = int(h_cnt[0])
    got = h_pairs[: 2 * c].numpy().view(np.uint32).reshape(-1, 2)
    erows, epos = orc.pairs_from_positions(orc.exact_lookup(col, pr))
    if not ordered:
        got = got[np.argsort(got[:, 0], kind="stable")]
    np.testing.assert_array_equal(got[:, 0], erows)
    np.testing.assert_array_equal(got[:, 1], epos)


@pytest.mark.parametrize("m", [(1 << 22) + 12345, 3 * (1 << 22) + 7])
def test_inlj_pairs_large(orc, gj, cuda, m):
    # millions of probes through the two-pass pairs and the allocation-free
    # entry point: pairs in probe order, clean status
    import torch

    rng = np.random.default_rng(m % 1000)
    col = column(rng, 1 << 16)
    pr = col[rng.integers(0, len(col), m)]
    pr[::5] = pr[::5] + np.uint64(1)  # absent keys
    ix = gj.btree_index().construct(None, to_dev(torch, col))
    d_pr = to_dev(torch, pr)
    need = ctypes.c_size_t(0)
    gj.lib().gj_inlj_pairs_workspace_size(m, ctypes.byref(need))
    ws = torch.empty(need.value, dtype=torch.uint8, device="cuda")
    out, cnt = ix.inlj_pairs(d_pr, workspace=ws)
    ix.inlj_pairs_status(ws, m)
    rows, pos = pairs_of(out, cnt)
    erows, epos = orc.pairs_from_positions(orc.exact_lookup(col, pr))
    np.testing.assert_array_equal(rows, erows)
    np.testing.assert_array_equal(pos, epos)
    out2, cnt2 = ix.inlj_pairs_noalloc(d_pr, torch.empty_like(out), torch.zeros_like(cnt))
    rows2, pos2 = pairs_of(out2, cnt2)
    np.testing.assert_array_equal(rows2, erows)
    np.testing.assert_array_equal(pos2, epos)
