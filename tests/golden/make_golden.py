"""Generate tests/golden/*.npz from the reference's own lookup code.

Runs oracle/_ref/libgjref.so -- the reference's src/search.cuh, src/btree.cuh
and src/harmonia.cuh compiled in place by oracle/Makefile -- on small seeded
inputs and stores inputs and outputs.  Run from the repository root where the
reference tree exists:

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def sorted_unique(rng, n, upper=1 << 63):
    while True:
        k = np.unique(rng.integers(0, upper, size=n + n // 8 + 16, dtype=np.uint64))
        if len(k) >= n:
            sel = np.sort(rng.choice(len(k), size=n, replace=False))
            return k[sel]


def probe_mix(rng, col, m_present=2000, m_absent=1000):
    n = len(col)
    present = col[rng.integers(0, n, size=m_present)]
    absent = rng.integers(0, 1 << 63, size=m_absent, dtype=np.uint64)
    edges = np.array([0, 1, col[0], col[-1], col[-1] + 1, (1 << 64) - 1, (1 << 63)], dtype=np.uint64)
    if col[0] > 0:
        edges = np.append(edges, np.uint64(col[0] - 1))
    return np.concatenate([present, absent, edges, col[:16], col[-16:]]).astype(np.uint64)


def main() -> None:
    if oracle.ref_lib() is None:
        raise SystemExit("oracle/_ref/libgjref.so is not available (reference tree missing?)")
    rng = np.random.default_rng(20261203)

    # binary search / branch-free search (src/search.cuh, src/indexes.cuh:357-361)
    cases = {}
    for n in (2, 3, 31, 32, 33, 1000, 4097):
        col = sorted_unique(rng, n)
        pr = probe_mix(rng, col, 300, 200)
        cases[f"bs_{n}_col"] = col
        cases[f"bs_{n}_probes"] = pr
        cases[f"bs_{n}_lb"] = oracle.ref_bs_lookup(col, pr)
        cases[f"bs_{n}_bf"] = oracle.ref_bs_branch_free_lookup(col, pr)
    np.savez_compressed(os.path.join(OUT, "search.npz"), **cases)

    # clustered B+tree with the reference page geometry (src/btree.cuh)
    cases = {}
    for n in (1, 246, 247, 248, 247 * 247, 247 * 247 + 1):
        col = sorted_unique(rng, n)
        pr = probe_mix(rng, col, 600, 200)
        cases[f"btree_{n}_col"] = col
        cases[f"btree_{n}_probes"] = pr
        cases[f"btree_{n}_pos"] = oracle.ref_btree_lookup(col, pr)
    np.savez_compressed(os.path.join(OUT, "btree.npz"), **cases)

    # Harmonia, 32 keys per node (src/harmonia.cuh); sizes hit 1-4 levels and
    # the under-full rightmost-node case
    cases = {}
    for n in (32, 64, 32 * 33, 32 * 34, 32 * 1089, 32 * 1090):
        col = sorted_unique(rng, n)
        pr = probe_mix(rng, col, 600, 200)
        cases[f"harmonia_{n}_col"] = col
        cases[f"harmonia_{n}_probes"] = pr
        cases[f"harmonia_{n}_pos"] = oracle.ref_harmonia_lookup(col, pr)
        keys, children, depth = oracle.ref_harmonia_arrays(col)
        cases[f"harmonia_{n}_keys"] = keys
        cases[f"harmonia_{n}_children"] = children
        cases[f"harmonia_{n}_depth"] = np.array([depth], dtype=np.uint32)
    np.savez_compressed(os.path.join(OUT, "harmonia.npz"), **cases)

    # the reference's own known-answer settings: iota uint32 keys
    # (test/test_harmonia.cu:18-55,115-130; test/main.cu:144-164)
    # n = 7 and 15 with 8-key nodes make construct() throw in this reference
    # version (Reuse_Input_Memory needs n % node_size == 0,
    # src/harmonia.cuh:350-352); the fixture records that as an empty array
    cases = {}
    for node, n in ((8, 7), (8, 15), (8, 280), (8, 2000), (4, 144)):
        col = np.arange(n, dtype=np.uint32)
        try:
            cases[f"kat_{node}_{n}"] = oracle.ref_harmonia_lookup_u32(col, node, col)
        except RuntimeError:
            cases[f"kat_{node}_{n}"] = np.zeros(0, dtype=np.uint32)
    np.savez_compressed(os.path.join(OUT, "harmonia_kat.npz"), **cases)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
