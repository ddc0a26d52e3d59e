"""Oracle-side generators and learned-model math (CPU)."""
import numpy as np


def test_permutation_is_bijective(orc):
    for n in (1, 2, 3, 17, 1000, 4096, 5003):
        seen = np.array([orc.permute(i, n, 1234) for i in range(n)], dtype=np.uint64)
        assert sorted(seen.tolist()) == list(range(n))


def test_zipf_rank_distribution(orc):
    # rejection-inversion (src/zipf.hpp): P(k) ~ k^-q on [1, n]
    n, q, m = 100, 1.0, 40000
    ranks = np.array([orc.zipf_rank(n, q, 7, i) for i in range(m)])
    assert ranks.min() >= 1 and ranks.max() <= n
    p = 1.0 / np.arange(1, n + 1) ** q
    p /= p.sum()
    counts = np.bincount(ranks, minlength=n + 1)[1:]
    expected = p * m
    chi2 = float(((counts - expected) ** 2 / expected).sum())
    assert chi2 < 200, chi2  # 99 dof; a correct sampler gives ~100


def test_zipf_theta_zero_is_uniform(orc):
    n, m = 50, 20000
    ranks = np.array([orc.zipf_rank(n, 0.0, 9, i) for i in range(m)])
    counts = np.bincount(ranks, minlength=n + 1)[1:]
    assert counts.min() > 0.7 * m / n and counts.max() < 1.3 * m / n


def test_mlp_gradient_matches_finite_differences(orc):
    rng = np.random.default_rng(3)
    H = 8
    nparam = 2 * H + H * H + H + H + 1
    P = rng.normal(0, 0.5, nparam).astype(np.float32)
    x = rng.random(64).astype(np.float32)
    y = np.sort(rng.random(64)).astype(np.float32)
    loss, g = orc.mlp_loss_grad(P, H, x, y)
    eps = 1e-3
    for j in rng.choice(nparam, 12, replace=False):
        Pp, Pm = P.copy(), P.copy()
        Pp[j] += eps
        Pm[j] -= eps
        lp, _ = orc.mlp_loss_grad(Pp, H, x, y)
        lm, _ = orc.mlp_loss_grad(Pm, H, x, y)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[j]) <= 2e-2 * max(1.0, abs(fd)), (j, fd, g[j])


def test_mlp_forward_consistent_with_loss(orc):
    rng = np.random.default_rng(4)
    H = 32
    P = rng.normal(0, 0.3, 2 * H + H * H + 2 * H + 1).astype(np.float32)
    x = np.array([0.25], dtype=np.float32)
    f = orc.mlp_forward(P, H, 0.25)
    loss, _ = orc.mlp_loss_grad(P, H, x, np.array([0.0], dtype=np.float32))
    assert abs(loss - f * f) < 1e-3 * max(1, f * f)


def test_range_partition_oracle(orc):
    rng = np.random.default_rng(8)
    keys = rng.integers(0, 1 << 40, 10000, dtype=np.uint64)
    ok, rows, offs = orc.range_partition(keys, 0, 32, 8)
    assert offs[0] == 0 and offs[-1] == len(keys)
    assert np.all(np.diff(offs.astype(np.int64)) >= 0)
    np.testing.assert_array_equal(keys[rows], ok)
    parts = np.minimum(keys >> np.uint64(32), 255)
    for p in range(256):
        seg = rows[offs[p]:offs[p + 1]]
        assert np.all(parts[seg] == p)
        assert np.all(np.diff(seg.astype(np.int64)) > 0)  # stable


def test_star_join_oracle_small(orc):
    dim = np.array([1, 2, 3, 5], dtype=np.uint64)
    flag = np.array([1, 0, 1, 0], dtype=np.uint8)
    fk = np.array([1, 2, 4, 5, 3], dtype=np.uint32)
    date = np.array([10, 10, 10, 9, 12], dtype=np.uint32)
    price = np.array([100, 200, 300, 400, 500], dtype=np.int64)
    disc = np.array([0, 10, 0, 5, 1], dtype=np.int64)
    num, den = orc.star_join(fk, date, price, disc, dim, flag, 10, 12)
    # rows 0, 1 pass (row 2 has no dimension row, 3 and 4 fail the date filter)
    assert den == 100 * 100 + 200 * 90
    assert num == 100 * 100
