"""Device generators: sorted unique build columns and Zipf probe columns."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dist", [0, 1, 2])
@pytest.mark.parametrize("n", [1, 2, 1000, 1 << 20])
def test_sorted_keys_strictly_increasing(gj, cuda, dist, n):
    k = gj.generate_sorted_keys(n, dist, 1 << 63, seed=n + dist).cpu().numpy().view(np.uint64)
    assert len(k) == n
    assert np.all(np.diff(k.astype(np.uint64)) > 0) if n > 1 else True
    assert int(k[-1]) < (1 << 63) + n  # below the bound (lognormal fix-up may add at most n)


def test_sorted_keys_deterministic(gj, cuda):
    a = gj.generate_sorted_keys(100000, 0, 1 << 63, seed=5).cpu().numpy()
    b = gj.generate_sorted_keys(100000, 0, 1 << 63, seed=5).cpu().numpy()
    c = gj.generate_sorted_keys(100000, 0, 1 << 63, seed=6).cpu().numpy()
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def test_uniform_keys_look_uniform(gj, cuda):
    n = 1 << 20
    k = gj.generate_sorted_keys(n, 0, 1 << 63, seed=3).cpu().numpy().view(np.uint64)
    counts = np.bincount((k >> np.uint64(63 - 8)).astype(np.int64), minlength=256)
    assert counts.min() > 0.9 * n / 256 and counts.max() < 1.1 * n / 256


def test_probes_come_from_build_keys(gj, cuda):
    import torch

    keys = gj.generate_sorted_keys(1 << 16, 0, 1 << 63, seed=1)
    for theta in (0.0, 0.5, 1.0):
        pr = gj.generate_probes(keys, 100000, theta=theta, seed=2).cpu().numpy().view(np.uint64)
        kk = keys.cpu().numpy().view(np.uint64)
        assert np.isin(pr, kk).all()


def test_absent_fraction(gj, cuda):
    for dist in (0, 2):
        keys = gj.generate_sorted_keys(1 << 16, dist, 1 << 63, seed=4)
        pr = gj.generate_probes(keys, 200000, theta=0.0, absent_fraction=0.05, seed=9).cpu().numpy().view(np.uint64)
        kk = keys.cpu().numpy().view(np.uint64)
        frac = 1.0 - np.isin(pr, kk).mean()
        assert 0.04 < frac < 0.06, frac


def test_zipf_skew(gj, cuda):
    n, m = 1 << 12, 400000
    keys = gj.generate_sorted_keys(n, 0, 1 << 63, seed=10)
    kk = keys.cpu().numpy().view(np.uint64)
    for theta, lo, hi in ((0.0, 0.0, 0.01), (1.0, 0.08, 0.2)):
        pr = gj.generate_probes(keys, m, theta=theta, seed=11).cpu().numpy().view(np.uint64)
        top = np.sort(np.bincount(np.searchsorted(kk, pr), minlength=n))[::-1]
        share = top[0] / m  # rank-1 share: ~1/H_n for theta = 1
        assert lo <= share <= hi, (theta, share)
