"""The allocation-free pairs entry point (gj_inlj_pairs_noalloc), for callers
that cannot allocate device memory while probing.  It must emit exactly what
gj_inlj_pairs emits, call after call, although every call reuses the same
library-owned scratch array.  Kept in its own file so that it runs last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pairs(out, cnt):
    c = int(cnt.item())
    return c, out[: 2 * c].cpu().numpy().view(np.uint32).copy()


def test_noalloc_pairs_match_workspace_entry_point(gj, cuda):
    import torch

    keys = gj.generate_sorted_keys(1 << 18, 0, 1 << 63, seed=901)
    ix = gj.btree_index().construct(None, keys)
    for call, (m, seed) in enumerate(((300001, 1), (70000, 2))):  # two calls in a row, different sizes
        probes = gj.generate_probes(keys, m, theta=0.5, absent_fraction=0.1, seed=seed)
        ref_out, ref_cnt = ix.inlj_pairs(probes)
        out = torch.full((2 * m,), -5, dtype=torch.int32, device="cuda")
        cnt = torch.full((1,), -5, dtype=torch.int64, device="cuda")
        ix.inlj_pairs_noalloc(probes, out, cnt)
        torch.cuda.synchronize()
        c_ref, p_ref = _pairs(ref_out, ref_cnt)
        c_got, p_got = _pairs(out, cnt)
        assert c_got == c_ref, f"call {call}: {c_got} pairs, expected {c_ref}"
        np.testing.assert_array_equal(p_got, p_ref, err_msg=f"call {call}")


def test_noalloc_rejects_oversized_batches(gj, cuda):
    L = gj.lib()
    keys = gj.generate_sorted_keys(1 << 10, 0, 1 << 63, seed=902)
    ix = gj.btree_index().construct(None, keys)
    dummy = ctypes.c_void_p(keys.data_ptr())
    rc = L.gj_inlj_pairs_noalloc(ix.handle, dummy, (1 << 28) + 1, dummy, dummy, None)
    assert rc == 8 and b"exceed the limit" in L.gj_last_error_string()
