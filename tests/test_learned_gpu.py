"""Learned position model: GPU gradients against the CPU oracle, exact
lookups, and what the trained root buys over the untrained (linear) one."""
import numpy as np
import pytest

from test_lookup_gpu import column, from_dev_u32, probes_for, to_dev

pytestmark = pytest.mark.gpu


def nparams(H):
    return 2 * H + H * H + H + H + 1


@pytest.mark.parametrize("H", [1, 8, 32])
def test_mlp_gradient_matches_oracle(orc, gj, cuda, H):
    import torch

    rng = np.random.default_rng(H)
    P = rng.normal(0, 0.5, nparams(H)).astype(np.float32)
    x = rng.random(3000).astype(np.float32)
    y = np.sort(rng.random(3000)).astype(np.float32)
    g, loss = gj.learned_mlp_grad(torch.from_numpy(P).cuda(), H, torch.from_numpy(x).cuda(),
                                  torch.from_numpy(y).cuda())
    eloss, eg = orc.mlp_loss_grad(P, H, x, y)
    g = g.cpu().numpy().astype(np.float64)
    # float32 accumulation over 3000 samples against the oracle's float64
    scale = np.abs(eg).max()
    np.testing.assert_allclose(g, eg, rtol=2e-3, atol=2e-4 * scale)
    assert abs(loss.item() - eloss) <= 1e-3 * max(1.0, eloss)


@pytest.mark.parametrize("dist", [0, 1, 2])
@pytest.mark.parametrize("root", [0, 1, 3])
def test_learned_lookup_exact(orc, gj, cuda, dist, root):
    import torch

    n = 1 << 18
    keys = gj.generate_sorted_keys(n, dist, 1 << 63, seed=dist + 40)
    probes = gj.generate_probes(keys, 1 << 17, theta=0.0, absent_fraction=0.05, seed=41)
    ix = gj.learned_index(learned_root=root, learned_leaves=4096, learned_steps=200).construct(None, keys)
    got = from_dev_u32(ix.lookup(probes))
    col = keys.cpu().numpy().view(np.uint64)
    pr = probes.cpu().numpy().view(np.uint64)
    np.testing.assert_array_equal(got, orc.bs_lookup(col, pr))
    # also the edge probes
    rng = np.random.default_rng(3)
    edge = probes_for(rng, col, 1000)
    np.testing.assert_array_equal(from_dev_u32(ix.lookup(to_dev(torch, edge))), orc.bs_lookup(col, edge))
    max_err, mean_window = ix.stats()
    assert mean_window >= 1.0 and max_err >= 0


def test_learned_small_and_ragged(orc, gj, cuda):
    import torch

    rng = np.random.default_rng(12)
    for n in (1, 2, 3, 100, 4097):
        col = column(rng, n)
        pr = probes_for(rng, col, 500)
        for root in (0, 1, 3):
            ix = gj.learned_index(learned_root=root, learned_leaves=64, learned_steps=20).construct(None,
                                                                                                  to_dev(torch, col))
            np.testing.assert_array_equal(from_dev_u32(ix.lookup(to_dev(torch, pr))), orc.bs_lookup(col, pr),
                                          err_msg=f"n={n} root={root}")


def test_trained_root_beats_linear_root_on_lognormal(gj, cuda):
    n = 1 << 20
    keys = gj.generate_sorted_keys(n, 1, 1 << 63, seed=77)
    lin = gj.learned_index(learned_root=0, learned_leaves=4096).construct(None, keys)
    mlp = gj.learned_index(learned_root=1, learned_leaves=4096, learned_steps=600).construct(None, keys)
    _, w_lin = lin.stats()
    _, w_mlp = mlp.stats()
    # the trained network routes keys by their learned CDF; the linear root
    # crowds the dense low end of the lognormal keys into few leaves
    assert w_mlp < 0.5 * w_lin, (w_mlp, w_lin)


def test_learned_in_pairs_and_partitioned(orc, gj, cuda):
    n = 1 << 16
    keys = gj.generate_sorted_keys(n, 0, 1 << 63, seed=5)
    probes = gj.generate_probes(keys, 50000, theta=0.5, absent_fraction=0.05, seed=6)
    ix = gj.learned_index(learned_leaves=1024, learned_steps=100).construct(None, keys)
    col = keys.cpu().numpy().view(np.uint64)
    pr = probes.cpu().numpy().view(np.uint64)
    exp = orc.bs_lookup(col, pr)
    pos, _, _ = ix.partitioned_inlj(probes)
    np.testing.assert_array_equal(from_dev_u32(pos), exp)
    out, cnt = ix.inlj_pairs(probes)
    c = int(cnt.item())
    got = out[: 2 * c].cpu().numpy().view(np.uint32).reshape(-1, 2)
    erows, epos = orc.pairs_from_positions(exp)
    np.testing.assert_array_equal(got[:, 0], erows)
    np.testing.assert_array_equal(got[:, 1], epos)


def test_segment_root_beats_linear_root_on_skewed_keys(orc, gj, cuda):
    # the segment table follows the key CDF: far narrower windows than the
    # linear root on lognormal and clustered keys; lookups exact
    for dist in (1, 2):
        keys = gj.generate_sorted_keys(1 << 20, dist, 1 << 63, seed=70 + dist)
        lin = gj.learned_index(learned_root=gj.LEARNED_ROOT_LINEAR, learned_leaves=4096).construct(None, keys)
        seg = gj.learned_index(learned_root=gj.LEARNED_ROOT_SEGMENTS, learned_leaves=4096).construct(None, keys)
        assert seg.root_kind() == gj.LEARNED_ROOT_SEGMENTS
        _, w_lin = lin.stats()
        _, w_seg = seg.stats()
        assert w_seg < 0.5 * w_lin, (dist, w_seg, w_lin)
        probes = gj.generate_probes(keys, 1 << 17, theta=0.0, absent_fraction=0.05, seed=71)
        np.testing.assert_array_equal(from_dev_u32(seg.lookup(probes)),
                                      orc.bs_lookup(keys.cpu().numpy().view(np.uint64),
                                                    probes.cpu().numpy().view(np.uint64)))


def test_segment_root_host_memory(orc, gj, cuda):
    # the segment table read from pinned host memory
    keys = gj.generate_sorted_keys(1 << 18, 1, 1 << 63, seed=81)
    probes = gj.generate_probes(keys, 1 << 16, theta=0.0, absent_fraction=0.05, seed=82)
    h_keys = keys.cpu().pin_memory()
    ix = gj.learned_index(learned_root=gj.LEARNED_ROOT_SEGMENTS, learned_leaves=2048,
                          index_memory=gj.INDEX_MEMORY_HOST).construct(None, h_keys)
    assert ix.host_memory() > 0
    np.testing.assert_array_equal(from_dev_u32(ix.lookup(probes)),
                                  orc.bs_lookup(keys.cpu().numpy().view(np.uint64),
                                                probes.cpu().numpy().view(np.uint64)))


def test_learned_auto_root(orc, gj, cuda):
    # the default root is chosen per column: linear on uniform keys (windows
    # as narrow as any other root's), a root that follows the CDF (segment
    # table or MLP) on lognormal keys; lookups stay exact
    import torch

    from test_lookup_gpu import from_dev_u32

    picks = {}
    for name, dist in (("uniform", gj.DIST_UNIFORM), ("lognormal", gj.DIST_LOGNORMAL)):
        keys = gj.generate_sorted_keys(1 << 20, dist, 1 << 63, seed=17)
        probes = gj.generate_probes(keys, 1 << 18, theta=0.0, absent_fraction=0.05, seed=18)
        ix = gj.learned_index().construct(None, keys)
        assert ix.params.learned_root == gj.LEARNED_ROOT_AUTO
        picks[name] = {gj.LEARNED_ROOT_LINEAR: "linear", gj.LEARNED_ROOT_MLP: "cdf",
                       gj.LEARNED_ROOT_SEGMENTS: "cdf"}[ix.root_kind()]
        h_keys = keys.cpu().numpy().view(np.uint64)
        got = from_dev_u32(ix.lookup(probes))
        np.testing.assert_array_equal(got, orc.bs_lookup(h_keys, probes.cpu().numpy().view(np.uint64)))
    assert picks == {"uniform": "linear", "lognormal": "cdf"}, picks


def test_what_training_adds_over_the_quantile_start(orc, gj, cuda):
    # The MLP root starts as the piecewise-linear CDF through 33 sample
    # quantiles; Adam then trains it on (key, position) samples and the build
    # keeps whichever of the two fits the samples better.  learned_steps = 0
    # keeps the start, so the gain of training is measured directly, at the
    # learned configuration's 2^14 leaves:
    #   uniform keys: none -- the start fits better and is kept;
    #   lognormal, clusters: the sample loss drops, and on the clustered
    #   column (long trained) the mean search window narrows too.
    n, leaves = 1 << 22, 1 << 14
    kw = dict(learned_root=gj.LEARNED_ROOT_MLP, learned_leaves=leaves)
    for dist in (gj.DIST_UNIFORM, gj.DIST_LOGNORMAL, gj.DIST_CLUSTERS):
        keys = gj.generate_sorted_keys(n, dist, 1 << 63, seed=130 + dist)
        start = gj.learned_index(learned_steps=0, **kw).construct(None, keys)
        trained = gj.learned_index(learned_steps=3000, **kw).construct(None, keys)
        l_start, l_start2 = start.losses()
        assert l_start == l_start2, "zero steps keeps the quantile start"
        l_init, l_trained = trained.losses()
        assert abs(l_init - l_start) <= 1e-12 * max(1.0, l_start), "the same start"
        _, w_start = start.stats()
        _, w_trained = trained.stats()
        if dist == gj.DIST_UNIFORM:
            assert l_trained >= l_init and w_trained == w_start, (l_init, l_trained, w_start, w_trained)
        else:
            assert l_trained < 0.8 * l_init, (dist, l_init, l_trained)
        if dist == gj.DIST_CLUSTERS:
            assert w_trained < 0.9 * w_start, (w_start, w_trained)
        # lookups exact either way
        probes = gj.generate_probes(keys, 1 << 16, theta=0.0, absent_fraction=0.05, seed=131)
        want = orc.bs_lookup(keys.cpu().numpy().view(np.uint64), probes.cpu().numpy().view(np.uint64))
        for ix in (start, trained):
            np.testing.assert_array_equal(from_dev_u32(ix.lookup(probes)), want)
