"""Batched lookup stream: many batches against several indexes in one
persistent kernel (mode 0) and one launch per batch (mode 1)."""
import numpy as np
import pytest

from test_lookup_gpu import from_dev_u32

pytestmark = pytest.mark.gpu


def test_batch_modes_match_oracle(orc, gj, cuda):
    import torch

    rng = np.random.default_rng(1)
    specs = [("btree", 1 << 16, 0), ("harmonia", 1 << 15, 1), ("radix_spline", 1 << 17, 0),
             ("binary_search", 1 << 14, 2), ("learned", 1 << 16, 1), ("hash", 1 << 16, 2)]
    indexes, cols = [], []
    for i, (kind, n, dist) in enumerate(specs):
        keys = gj.generate_sorted_keys(n, dist, 1 << 63, seed=100 + i)
        kw = {"learned_steps": 50, "learned_leaves": 512} if kind == "learned" else {}
        indexes.append(gj.make_index(kind, **kw).construct(None, keys))
        cols.append(keys)
    nb = 200
    sizes = np.clip(rng.lognormal(7, 1.5, nb).astype(np.int64), 1, 50000)
    sizes[5] = 0  # an empty batch
    which = rng.integers(0, len(specs), nb).astype(np.uint32)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64)
    total = int(sizes.sum())
    probes = torch.empty(total, dtype=torch.int64, device="cuda")
    for b in range(nb):
        if sizes[b]:
            probes[int(offs[b]): int(offs[b]) + int(sizes[b])] = gj.generate_probes(cols[which[b]], int(sizes[b]), theta=0.8,
                                                                     absent_fraction=0.05, seed=b)
    h_probes = probes.cpu().numpy().view(np.uint64)
    exp = np.empty(total, dtype=np.uint32)
    for b in range(nb):
        a, e = int(offs[b]), int(offs[b]) + int(sizes[b])
        col = cols[which[b]].cpu().numpy().view(np.uint64)
        kind = specs[which[b]][0]
        exp[a:e] = (orc.exact_lookup if kind in ("btree", "harmonia", "hash") else orc.bs_lookup)(col, h_probes[a:e])
    for mode in (0, 1):
        out = torch.full((total,), -7, dtype=torch.int32, device="cuda")
        done = torch.zeros(nb + 1, dtype=torch.int64, device="cuda")
        gj.batch_lookup(indexes, which, offs, sizes, probes, out, mode=mode, d_done_ns=done)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(from_dev_u32(out), exp, err_msg=f"mode {mode}")
        d = done.cpu().numpy()
        nonempty = np.concatenate([sizes > 0, [False]])
        assert np.all(d[nonempty] >= d[nb]) and d[nb] > 0, f"mode {mode}: missing or early completion stamps"

    # one plan: graph capture and replays, every tile shape, the autotuner
    plan = gj.batch_plan(indexes, which, offs, sizes, tile_items=2)
    for items in (2, 4, 8, 16):
        if items != 2:
            plan.free()
            plan = gj.batch_plan(indexes, which, offs, sizes, tile_items=items)
        assert plan.tile_items == items
        for rep in range(3):
            out = torch.full((total,), -7, dtype=torch.int32, device="cuda")
            done = torch.zeros(nb + 1, dtype=torch.int64, device="cuda")
            plan.run_graph(probes, out, 0, done)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(from_dev_u32(out), exp, err_msg=f"graph items {items} replay {rep}")
    out = torch.full((total,), -7, dtype=torch.int32, device="cuda")
    best, ms = plan.autotune(probes, out)
    assert best in (2, 4, 8, 16) and ms > 0 and plan.tile_items == best
    out.fill_(-7)
    plan.run_graph(probes, out, 0)
    plan.run_graph(probes, out, 1)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(from_dev_u32(out), exp, err_msg="after autotune")
    plan.free()


def test_batch_plan_arguments(gj, cuda):
    import ctypes

    import torch

    keys = torch.arange(0, 4096, dtype=torch.int64, device="cuda") * 3
    ix = gj.btree_index().construct(None, keys)
    with pytest.raises(gj.GJError):
        gj.batch_plan([ix], [1], [0], [10])  # missing index
    with pytest.raises(gj.GJError):
        gj.batch_plan([ix], [0], [0], [10], tile_items=3)
    empty = gj.batch_plan([ix], [], [], [])
    out = torch.empty(1, dtype=torch.int32, device="cuda")
    empty.run(keys, out)
    empty.run_graph(keys, out)
    torch.cuda.synchronize()
    empty.free()
    assert gj.lib().gj_batch_plan_free(None) == 0
    assert gj.lib().gj_batch_plan_run(None, None, None, 0, None, None) == 1
    del ctypes
