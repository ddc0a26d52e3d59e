"""The reference's own device lookups (binary_search_index, btree::lookup,
harmonia_tree::lookup<4>, compiled from its headers into
oracle/_ref/refgpu.cubin) against
the oracle and the library's kernels on the same index data: the three agree
on every probe, so the bench's timing of the reference kernels compares like
with like.  Skipped where the cubin was not built (no reference tree at build
time)."""
import numpy as np
import pytest

from test_lookup_gpu import column, from_dev_u32, probes_for, to_dev

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref(cuda):
    from oracle import ref_gpu

    if not ref_gpu.available():
        pytest.skip("oracle/_ref/refgpu.cubin not built")
    k = ref_gpu.ReferenceKernels()
    yield k
    k.close()


@pytest.mark.parametrize("n", [32, 4096, 1 << 20])
def test_reference_kernels_match_oracle_and_library(orc, gj, ref, n):
    import torch

    from oracle import ref_gpu

    rng = np.random.default_rng(n)
    col = column(rng, n)
    pr = probes_for(rng, col, 200_003)  # not a multiple of the warp: inactive lanes in the last warp
    d_col, d_pr = to_dev(torch, col), to_dev(torch, pr)
    stream = torch.cuda.current_stream()
    out = torch.empty(len(pr), dtype=torch.int32, device="cuda")

    ref.binary_search(d_col, d_pr, out, stream)
    want_lb = orc.bs_lookup(col, pr)
    np.testing.assert_array_equal(from_dev_u32(out), want_lb)
    bs = gj.make_index("binary_search").construct(None, d_col)
    np.testing.assert_array_equal(from_dev_u32(bs.lookup(d_pr)), want_lb)

    want_eq = orc.exact_lookup(col, pr)
    root, pages = ref.btree_pages(d_col, col)
    out.fill_(0)
    ref.btree(root, d_col, d_pr, out, stream)
    np.testing.assert_array_equal(from_dev_u32(out), want_eq)
    bt = gj.make_index("btree").construct(None, d_col)
    np.testing.assert_array_equal(from_dev_u32(bt.lookup(d_pr)), want_eq)
    bt.free()

    hm = gj.make_index("harmonia").construct(None, d_col)
    out.fill_(0)
    view, keep = ref.padded_harmonia(ref_gpu.harmonia_view(gj, hm))
    ref.harmonia(view, d_pr, out, stream)
    np.testing.assert_array_equal(from_dev_u32(out), want_eq)
    np.testing.assert_array_equal(from_dev_u32(hm.lookup(d_pr)), want_eq)
    bs.free()
    hm.free()
