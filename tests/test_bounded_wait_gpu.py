"""The bounded waits of the ordered pairs compaction, made to run out on
purpose: tile 0 is never claimed, so every later tile's look-back waits for
a count that nothing publishes.  Each wait gives up after a short limit, the
kernel returns with its error word set, and the host reads GJ_ERR_TIMEOUT
through gj_inlj_pairs_status.  Nothing faults or hangs, and the same
context and workspace then serve a normal call."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GJ_ERR_TIMEOUT = 5


@pytest.mark.parametrize("kind", ["btree", "learned"])
def test_lookback_timeout_is_reported(gj, cuda, kind):
    import torch

    L = gj.lib()
    keys = gj.generate_sorted_keys(1 << 16, gj.DIST_UNIFORM, 1 << 63, seed=71)
    ix = gj.make_index(kind).construct(None, keys)
    m = (1 << 20) + 123
    probes = gj.generate_probes(keys, m, theta=0.0, seed=72)
    need = ctypes.c_size_t(0)
    assert L.gj_inlj_pairs_workspace_size(m, ctypes.byref(need)) == 0
    ws = torch.empty(need.value, dtype=torch.uint8, device="cuda")
    pairs = torch.empty(2 * m, dtype=torch.int32, device="cuda")
    cnt = torch.full((1,), -7, dtype=torch.int64, device="cuda")
    rc = L.gj_debug_inlj_pairs_stalled(ix.handle, ctypes.c_void_p(probes.data_ptr()), m,
                                       ctypes.c_void_p(pairs.data_ptr()), ctypes.c_void_p(cnt.data_ptr()),
                                       ctypes.c_void_p(ws.data_ptr()), ws.numel(), 4096, None)
    assert rc == 0, L.gj_last_error_string()
    torch.cuda.synchronize()
    rc = L.gj_inlj_pairs_status(ctypes.c_void_p(ws.data_ptr()), ws.numel(), m, None)
    assert rc == GJ_ERR_TIMEOUT
    assert b"waited too long" in L.gj_last_error_string()
    assert int(cnt.item()) == -7, "the count must not be written when a wait gave up"

    # the context and the workspace stay usable: a normal call on the same
    # workspace succeeds and equals a call on a fresh one
    out, c = ix.inlj_pairs(probes, workspace=ws)
    ix.inlj_pairs_status(ws, m)
    ref_out, ref_c = ix.inlj_pairs(probes)
    assert int(c.item()) == int(ref_c.item())
    k = int(c.item())
    np.testing.assert_array_equal(out[: 2 * k].cpu().numpy(), ref_out[: 2 * k].cpu().numpy())
