"""The reference's own device lookups on this GPU (BENCHMARK AND TEST
INFRASTRUCTURE ONLY).

``_ref/refgpu.cubin`` is ``ref_gpu.cu`` compiled with the reference's headers
(``src/search.cuh``, ``src/btree.cuh``, ``src/harmonia.cuh``) for sm_103a by ``make refgpu``,
only where the reference tree is present; a cubin is device code, so one
built there runs on any GB300 host.  ``ReferenceKernels`` loads it through
the CUDA driver API into the current (PyTorch) context and launches its
kernels the way the reference launches ``lookup_kernel``
(src/index_lookup_new.cu:191-196: one thread per probe, 128-thread blocks).
It times and checks the reference's GPU code beside the library's; the
library itself never loads it.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "refgpu.cubin")
BLOCK = 128  # the reference's default block size (src/index_lookup_config.hpp:27)


class HarmoniaView(ctypes.Structure):
    """gj::harmonia_view (include/gpujoin/device.cuh) as gj_index_device_view writes it."""
    _fields_ = [(f, ctypes.c_uint64) for f in ("keys", "children", "col", "n", "inner_size")] + \
               [(f, ctypes.c_uint32) for f in ("depth", "cached_nodes", "cached_levels", "col_aligned")] + \
               [(f, ctypes.c_uint64) for f in ("min_key", "start")] + \
               [(f, ctypes.c_uint32) for f in ("start_shift", "start_entries")]


def available() -> bool:
    return os.path.exists(CUBIN)


class ReferenceKernels:
    """ref_bs_lookup (binary_search_index's lookup), ref_btree_lookup
    (btree::lookup over pages in the reference's layout) and
    ref_harmonia_lookup (harmonia_tree::lookup<4>) from the cubin; each
    writes u32 positions, 0xFFFFFFFF where the reference returns its invalid
    tid."""

    def __init__(self):
        import torch

        if not available():
            raise FileNotFoundError("oracle/_ref/refgpu.cubin not built (needs the reference tree at build time)")
        torch.cuda.current_stream().synchronize()  # the primary context exists and is current
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        for name in ("ref_bs_lookup", "ref_btree_lookup", "ref_harmonia_lookup"):
            f = ctypes.c_void_p()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), name)
            self.fn[name] = f

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")

    def _launch(self, name, args, m, stream):
        vals = [a if isinstance(a, ctypes._SimpleCData) else ctypes.c_uint64(a) for a in args]
        params = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.byref(v), ctypes.c_void_p) for v in vals])
        grid = max(1, (m + BLOCK - 1) // BLOCK)
        self._check(self.cu.cuLaunchKernel(self.fn[name], ctypes.c_uint(grid), ctypes.c_uint(1), ctypes.c_uint(1),
                                           ctypes.c_uint(BLOCK), ctypes.c_uint(1), ctypes.c_uint(1), ctypes.c_uint(0),
                                           ctypes.c_void_p(stream.cuda_stream), params, None), name)

    def binary_search(self, col, probes, out, stream):
        """Lower bound of each probe in the sorted uint64 column (device tensors)."""
        assert col.dtype.itemsize == 8 and probes.dtype.itemsize == 8 and out.dtype.itemsize == 4
        assert out.numel() >= probes.numel()
        self._launch("ref_bs_lookup", [col.data_ptr(), col.numel(), probes.data_ptr(), probes.numel(),
                                       out.data_ptr()], probes.numel(), stream)

    def btree_layout(self):
        """The page layout this cubin was compiled with (ref_btree_layout):
        page size, header size, separator offset, child pointer offset,
        separators per inner node, keys per leaf."""
        import numpy as np

        ptr, size = ctypes.c_uint64(), ctypes.c_size_t()
        self._check(self.cu.cuModuleGetGlobal_v2(ctypes.byref(ptr), ctypes.byref(size), self.mod,
                                                 b"ref_btree_layout"), "cuModuleGetGlobal")
        out = np.zeros(6, dtype=np.uint64)
        assert size.value == out.nbytes
        self._check(self.cu.cuMemcpyDtoH_v2(out.ctypes.data_as(ctypes.c_void_p), ptr, ctypes.c_size_t(out.nbytes)),
                    "cuMemcpyDtoH")
        return [int(v) for v in out]

    def btree_pages(self, col, h_col):
        """The reference's clustered B+tree over the device column `col`
        (host copy `h_col`, uint64), built by the oracle's restatement of
        btree::construct (load factor 1.0, as btree_index::construct,
        src/indexes.cuh:126-127) and written in this cubin's page layout to
        device memory.  Returns (root pointer, pages tensor to keep alive)."""
        import numpy as np
        import torch

        import oracle

        page, _, keys_off, children_off, inner_keys, leaf_keys = self.btree_layout()
        tree = oracle.BTree(np.ascontiguousarray(h_col).view(np.uint64), leaf_keys, inner_keys)
        nodes = oracle.lib().orc_btree_nodes(tree._h)
        pages = torch.empty(nodes * page, dtype=torch.uint8, device=col.device)
        image, root = tree.pages(page, keys_off, children_off, pages.data_ptr(), col.data_ptr())
        pages.copy_(torch.from_numpy(image))
        torch.cuda.synchronize()
        return pages.data_ptr() + root * page, pages

    def btree(self, root, col, probes, out, stream):
        """Exact match of each probe through the pages of btree_pages."""
        assert col.dtype.itemsize == 8 and probes.dtype.itemsize == 8 and out.dtype.itemsize == 4
        assert out.numel() >= probes.numel()
        self._launch("ref_btree_lookup", [col.data_ptr(), col.data_ptr() + 8 * col.numel(), root,
                                          probes.data_ptr(), probes.numel(), out.data_ptr()], probes.numel(), stream)

    def padded_harmonia(self, view: HarmoniaView):
        """A copy of a Harmonia view whose inner keys and column are followed
        by one 32-key node of UINT64_MAX.  For a probe above a node's last
        separator harmonia_tree::lookup reads node_start[32]
        (src/harmonia.cuh:754-756), one element past the node; for the last
        node of the inner keys or of the column that is one past the array.
        The padding keeps those reads inside the buffers.  Returns (view,
        buffers to keep alive)."""
        import torch

        pad = 32
        keys = torch.full((view.inner_size + pad,), -1, dtype=torch.int64, device="cuda")
        col = torch.full((view.n + pad,), -1, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        if view.inner_size:
            self._check(self.cu.cuMemcpyDtoD_v2(ctypes.c_uint64(keys.data_ptr()), ctypes.c_uint64(view.keys),
                                                ctypes.c_size_t(8 * view.inner_size)), "cuMemcpyDtoD")
        self._check(self.cu.cuMemcpyDtoD_v2(ctypes.c_uint64(col.data_ptr()), ctypes.c_uint64(view.col),
                                            ctypes.c_size_t(8 * view.n)), "cuMemcpyDtoD")
        v = HarmoniaView()
        ctypes.memmove(ctypes.byref(v), ctypes.byref(view), ctypes.sizeof(v))
        v.keys, v.col = keys.data_ptr(), col.data_ptr()
        return v, (keys, col)

    def harmonia(self, view: HarmoniaView, probes, out, stream):
        """Exact match of each probe through a Harmonia tree given by its
        device view (padded: padded_harmonia)."""
        assert probes.dtype.itemsize == 8 and out.dtype.itemsize == 4 and out.numel() >= probes.numel()
        self._launch("ref_harmonia_lookup", [view.keys, view.col, view.children, view.n, view.inner_size,
                                             ctypes.c_uint32(view.depth), probes.data_ptr(), probes.numel(),
                                             out.data_ptr()], probes.numel(), stream)

    def close(self):
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = None


def harmonia_view(gj, ix) -> HarmoniaView:
    """The device view of a constructed gpujoin_gb300 Harmonia index."""
    v = HarmoniaView()
    gj._check(gj.lib().gj_index_device_view(ix.handle, ctypes.byref(v), ctypes.sizeof(v)))
    return v
