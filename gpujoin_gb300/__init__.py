"""gpujoin_gb300 -- GB300-native index-nested-loop-join probe engine.

Python host mirror of the reference's index/operator API (josefschmeisser/
gpujoin ``src/indexes.cuh``, ``src/indexes.hpp``, ``src/index_lookup_config.hpp``,
``src/partitioned_relation.hpp``) over the C ABI of ``libgpujoin.so``
(declared in ``include/gpujoin.h``).  All compute runs in the hand-written
sm_103a kernels of that library; there is no CPU fallback: if the library
cannot be loaded, every entry point raises.

Device buffers are torch CUDA tensors.  uint64 columns are carried in int64
tensors (same bits) and uint32 positions in int32 tensors;
``INVALID_POS`` (0xFFFFFFFF) therefore reads as -1 in an int32 tensor.
"""
from __future__ import annotations

import ctypes
import dataclasses
import enum
import os
from typing import Optional, Tuple

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.environ.get("GJ_LIB_PATH", os.path.join(HERE, "libgpujoin.so"))

INVALID_POS = 0xFFFFFFFF

GJ_OK = 0
_ERRORS = {
    1: "invalid argument",
    2: "CUDA error",
    3: "unsupported",
    4: "out of memory",
    5: "timeout",
    6: "unsorted build keys",
    7: "workspace too small",
    8: "size exceeds limit",
}

DIST_UNIFORM = 0
DIST_LOGNORMAL = 1
DIST_CLUSTERS = 2

LEARNED_ROOT_LINEAR = 0
LEARNED_ROOT_MLP = 1
LEARNED_ROOT_AUTO = 2  # all roots built, the cheapest kept unless its windows are much wider
LEARNED_ROOT_SEGMENTS = 3  # piecewise-linear CDF over 4096 equal-width key segments


class GJError(RuntimeError):
    """A non-zero status from the C ABI (code, message from gj_last_error_string)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{_ERRORS.get(code, 'error')} ({code}): {message}")
        self.code = code


class index_type_enum(enum.IntEnum):
    """src/indexes.hpp:5, plus the learned index."""

    btree = 0
    harmonia = 1
    binary_search = 2
    radix_spline = 3
    no_op = 4
    learned = 5
    hash = 6


class gj_index_params(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("btree_node_keys", ctypes.c_uint32),
        ("btree_leaf_keys", ctypes.c_uint32),
        ("rs_radix_bits", ctypes.c_uint32),
        ("rs_max_error", ctypes.c_uint32),
        ("bs_cache_keys", ctypes.c_uint32),
        ("smem_cache_bytes", ctypes.c_uint32),
        ("learned_leaves", ctypes.c_uint32),
        ("learned_root", ctypes.c_uint32),
        ("learned_hidden", ctypes.c_uint32),
        ("learned_steps", ctypes.c_uint32),
        ("learned_batch", ctypes.c_uint32),
        ("learned_lr", ctypes.c_float),
        ("index_memory", ctypes.c_uint32),
        ("btree_start_bits", ctypes.c_uint32),
        ("seed", ctypes.c_uint64),
    ]


# probe orders (gj_autotune_ordering)
ORDER_PROBE = 0
ORDER_SORTED_TILES = 1
ORDER_PARTITIONED = 2

# gj_index_params.index_memory
INDEX_MEMORY_DEVICE = 0
INDEX_MEMORY_HOST = 1


class gj_q14_tables(ctypes.Structure):
    _fields_ = [
        ("n_lineitem", ctypes.c_uint64),
        ("n_part", ctypes.c_uint64),
        ("l_partkey", ctypes.POINTER(ctypes.c_uint32)),
        ("l_shipdate", ctypes.POINTER(ctypes.c_uint32)),
        ("l_extendedprice", ctypes.POINTER(ctypes.c_int64)),
        ("l_discount", ctypes.POINTER(ctypes.c_int64)),
        ("p_partkey", ctypes.POINTER(ctypes.c_uint64)),
        ("p_promo", ctypes.POINTER(ctypes.c_uint8)),
    ]


_LIB: Optional[ctypes.CDLL] = None
_vp = ctypes.c_void_p
_u64 = ctypes.c_uint64
_u32 = ctypes.c_uint32
_i32 = ctypes.c_int
_sz = ctypes.c_size_t

_SIGNATURES = {
    "gj_abi_version": (_u32, []),
    "gj_last_error_string": (ctypes.c_char_p, []),
    "gj_index_params_default": (None, [ctypes.POINTER(gj_index_params)]),
    "gj_parse_index_type": (_i32, [ctypes.c_char_p, ctypes.POINTER(_i32)]),
    "gj_index_type_name": (ctypes.c_char_p, [_i32]),
    "gj_index_build": (_i32, [_i32, _vp, _vp, _u64, ctypes.POINTER(gj_index_params), _vp, ctypes.POINTER(_vp)]),
    "gj_index_free": (_i32, [_vp]),
    "gj_index_memory_consumption": (_u64, [_vp]),
    "gj_index_host_memory": (_u64, [_vp]),
    "gj_index_get_type": (_i32, [_vp, ctypes.POINTER(_i32)]),
    "gj_index_size": (_u64, [_vp]),
    "gj_index_learned_stats": (_i32, [_vp, ctypes.POINTER(_u64), ctypes.POINTER(ctypes.c_double)]),
    "gj_index_learned_root": (_i32, [_vp, ctypes.POINTER(_u32)]),
    "gj_index_learned_losses": (_i32, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    "gj_index_device_view": (_i32, [_vp, _vp, _sz]),
    "gj_index_lookup": (_i32, [_vp, _vp, _u64, _vp, _vp]),
    "gj_inlj_pairs_workspace_size": (_i32, [_u64, ctypes.POINTER(_sz)]),
    "gj_inlj_pairs": (_i32, [_vp, _vp, _u64, _vp, _vp, _vp, _sz, _vp]),
    "gj_inlj_pairs_unordered": (_i32, [_vp, _vp, _u64, _vp, _vp, _vp, _sz, _vp]),
    "gj_inlj_pairs_status": (_i32, [_vp, _sz, _u64, _vp]),
    "gj_debug_inlj_pairs_stalled": (_i32, [_vp, _vp, _u64, _vp, _vp, _vp, _sz, _u32, _vp]),
    "gj_inlj_pairs_host_workspace_size": (_i32, [_u64, ctypes.POINTER(_sz)]),
    "gj_inlj_pairs_host": (_i32, [_vp, _vp, _u64, _vp, _vp, _vp, _sz, _vp]),
    "gj_inlj_pairs_host_unordered": (_i32, [_vp, _vp, _u64, _vp, _vp, _vp, _sz, _vp]),
    "gj_inlj_pairs_noalloc": (_i32, [_vp, _vp, _u64, _vp, _vp, _vp]),
    "gj_partition_workspace_size": (_i32, [_u64, _u32, ctypes.POINTER(_sz)]),
    "gj_index_key_range": (_i32, [_vp, ctypes.POINTER(_u64), ctypes.POINTER(_u64)]),
    "gj_index_lookup_cooperative": (_i32, [_vp, _vp, _u64, _vp, _u32, _vp]),
    "gj_partition_shift": (_i32, [_u64, _u64, _u32, ctypes.POINTER(_u32)]),
    "gj_range_partition": (_i32, [_vp, _u64, _u64, _u32, _u32, _vp, _vp, _vp, _vp, _sz, _vp]),
    "gj_partitioned_lookup": (_i32, [_vp, _vp, _vp, _u64, _vp, _vp]),
    "gj_partitioned_inlj_workspace_size": (_i32, [_vp, _u64, _u32, ctypes.POINTER(_sz)]),
    "gj_index_prepare_partitioned": (_i32, [_vp, _vp]),
    "gj_partitioned_inlj": (_i32, [_vp, _vp, _u64, _u64, _u32, _vp, _vp, _vp, _vp, _sz, _vp]),
    "gj_tpch_load_q14": (_i32, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(gj_q14_tables)]),
    "gj_tpch_free_q14": (None, [ctypes.POINTER(gj_q14_tables)]),
    "gj_tpch_day": (_i32, [_i32, _i32, _i32, ctypes.POINTER(_u32)]),
    "gj_tpch_q14": (_i32, [ctypes.POINTER(gj_q14_tables), _vp, ctypes.POINTER(ctypes.c_int64),
                           ctypes.POINTER(ctypes.c_double)]),
    "gj_star_join_sum": (_i32, [_vp, _vp, _vp, _vp, _vp, _u64, _vp, _u32, _u32, _vp, _vp]),
    "gj_star_join_sum_sorted": (_i32, [_vp, _vp, _vp, _vp, _vp, _u64, _vp, _u32, _u32, _vp, _vp]),
    "gj_learned_mlp_grad": (_i32, [_vp, _u32, _vp, _vp, _u64, _vp, _vp, _vp]),
    "gj_autotune_partitioned": (_i32, [_vp, _vp, _u64, _vp, ctypes.POINTER(_u32), ctypes.POINTER(_u64),
                                       ctypes.POINTER(ctypes.c_float)]),
    "gj_index_lookup_sorted": (_i32, [_vp, _vp, _u64, _vp, _vp]),
    "gj_inlj_pairs_sorted": (_i32, [_vp, _vp, _u64, _vp, _vp, _vp, _sz, _vp]),
    "gj_autotune_ordering": (_i32, [_vp, _vp, _u64, _vp, ctypes.POINTER(_u32), ctypes.POINTER(ctypes.c_float)]),
    "gj_autotune_btree": (_i32, [_vp, _u64, _vp, _u64, _vp, ctypes.POINTER(_u32), ctypes.POINTER(_u32),
                                 ctypes.POINTER(ctypes.c_float)]),
    "gj_autotune_partitioned_btree": (_i32, [_vp, _u64, _vp, _u64, _vp, ctypes.POINTER(_u32), ctypes.POINTER(_u32),
                                             ctypes.POINTER(_u32), ctypes.POINTER(_u64),
                                             ctypes.POINTER(ctypes.c_float)]),
    "gj_batch_plan_create": (_i32, [ctypes.POINTER(_vp), _u32, _vp, _vp, _vp, _u32, _u32, _vp, ctypes.POINTER(_vp)]),
    "gj_batch_plan_free": (_i32, [_vp]),
    "gj_batch_plan_tile_items": (_i32, [_vp, ctypes.POINTER(_u32)]),
    "gj_batch_plan_run": (_i32, [_vp, _vp, _vp, _u32, _vp, _vp]),
    "gj_batch_plan_run_graph": (_i32, [_vp, _vp, _vp, _u32, _vp, _vp]),
    "gj_batch_plan_autotune": (_i32, [_vp, _vp, _vp, _vp, ctypes.POINTER(_u32), ctypes.POINTER(ctypes.c_float)]),
    "gj_calibrate_sink_words": (_i32, [ctypes.POINTER(_u64)]),
    "gj_calibrate_random_sectors": (_i32, [_vp, _u64, _u64, _u64, _u32, _vp, _vp]),
    "gj_generate_workspace_size": (_i32, [_u64, ctypes.POINTER(_sz)]),
    "gj_generate_sorted_keys": (_i32, [_vp, _u64, _u32, _u64, _u64, _vp, _sz, _vp]),
    "gj_generate_probes": (_i32, [_vp, _u64, _vp, _u64, ctypes.c_double, ctypes.c_double, _u64, _vp]),
}


def exported_symbols():
    """Names of every C entry point this module binds (all declared in include/gpujoin.h)."""
    return list(_SIGNATURES)


def lib() -> ctypes.CDLL:
    """Load libgpujoin.so (building it first if it is missing).  Raises if unavailable."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _build

            _build.build()
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIB = L
    return _LIB


def _check(rc: int) -> None:
    if rc != GJ_OK:
        msg = lib().gj_last_error_string()
        raise GJError(rc, msg.decode() if msg else "")


def _torch():
    import torch

    return torch


def _stream(stream=None) -> int:
    torch = _torch()
    if stream is None:
        stream = torch.cuda.current_stream()
    return stream.cuda_stream


def _hptr(t) -> int:
    """Address of a contiguous host tensor (pinned memory for the zero-copy entry points)."""
    if t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous host tensor")
    return t.data_ptr()


def _ptr(t) -> Optional[int]:
    if t is None:
        return None
    if isinstance(t, int):
        return t
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return t.data_ptr()


def _empty(n: int, dtype, device):
    torch = _torch()
    return torch.empty(n, dtype=dtype, device=device)


def _workspace(nbytes: int, device):
    torch = _torch()
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


def parse_index_type(name: str) -> index_type_enum:
    """parse_index_type (src/indexes.cpp:5-19); raises RuntimeError("unknown index type")."""
    out = _i32(0)
    rc = lib().gj_parse_index_type(name.encode(), ctypes.byref(out))
    if rc != GJ_OK:
        raise RuntimeError("unknown index type")
    return index_type_enum(out.value)


def default_params(**overrides) -> gj_index_params:
    p = gj_index_params()
    lib().gj_index_params_default(ctypes.byref(p))
    for k, v in overrides.items():
        if not hasattr(p, k):
            raise AttributeError(f"unknown index parameter {k}")
        setattr(p, k, v)
    return p


# --------------------------------------------------------------------------
# indexes (src/indexes.cuh)
# --------------------------------------------------------------------------
class abstract_index:
    """abstract_index<Key> (src/indexes.cuh:30-39) over a device column of uint64 keys."""

    index_type: index_type_enum = index_type_enum.no_op

    def __init__(self, **params):
        self.params = default_params(**params)
        self._handle = _vp(None)
        self.d_column = None

    # construct(h_column, d_column) -- src/indexes.cuh:36
    def construct(self, h_column, d_column, stream=None) -> "abstract_index":
        """d_column: the sorted keys as a CUDA tensor or as a pinned host tensor
        (Grace memory, read by the kernels over NVLink-C2C).  Where the index's
        own arrays live is the index_memory parameter (HBM by default)."""
        torch = _torch()
        if d_column is None or not (d_column.is_cuda or d_column.is_pinned()):
            raise ValueError("d_column must be a CUDA tensor or a pinned host tensor")
        if not d_column.is_contiguous():
            raise ValueError("d_column must be contiguous")
        if d_column.dtype not in (torch.int64, getattr(torch, "uint64", torch.int64)):
            raise ValueError("d_column must hold 64-bit keys")
        self.free()
        h_ptr = None
        if h_column is not None:
            import numpy as np

            self._h_column = np.ascontiguousarray(h_column, dtype=np.uint64)
            h_ptr = self._h_column.ctypes.data
        with torch.cuda.device(d_column.device if d_column.is_cuda else torch.cuda.current_device()):
            _check(lib().gj_index_build(int(self.index_type), d_column.data_ptr(), h_ptr, d_column.numel(),
                                        ctypes.byref(self.params), _stream(stream), ctypes.byref(self._handle)))
        self.d_column = d_column
        self._h_column = None
        return self

    def memory_consumption(self) -> int:
        """src/indexes.cuh:38"""
        return int(lib().gj_index_memory_consumption(self._handle))

    def host_memory(self) -> int:
        """Bytes of the index's own arrays in pinned host memory (index_memory=INDEX_MEMORY_HOST)."""
        return int(lib().gj_index_host_memory(self._handle))

    @property
    def handle(self) -> int:
        if not self._handle.value:
            raise RuntimeError("index not constructed")
        return self._handle.value

    @property
    def size(self) -> int:
        return int(lib().gj_index_size(self._handle)) if self._handle.value else 0

    def type_name(self) -> str:
        return lib().gj_index_type_name(int(self.index_type)).decode()

    # ---- probe operators ------------------------------------------------
    def lookup(self, d_probes, out=None, stream=None):
        """Plain INLJ probe (lookup_kernel, src/index_lookup_common.cuh:217-245) -> int32 positions."""
        torch = _torch()
        m = d_probes.numel()
        if out is None:
            out = _empty(m, torch.int32, d_probes.device)
        _check(lib().gj_index_lookup(self.handle, _ptr(d_probes), m, _ptr(out), _stream(stream)))
        return out

    def inlj_pairs(self, d_probes, out_pairs=None, out_count=None, workspace=None, stream=None,
                   ordered: bool = True):
        """(probe row, build pos) pairs of the matches, in probe order (ij_lookup_kernel);
        ordered=False: the same pairs in the order their tiles finish (gj_inlj_pairs_unordered)."""
        torch = _torch()
        m = d_probes.numel()
        dev = d_probes.device
        if out_pairs is None:
            out_pairs = _empty(2 * max(m, 1), torch.int32, dev)
        if out_count is None:
            out_count = torch.zeros(1, dtype=torch.int64, device=dev)
        if workspace is None:
            need = _sz(0)
            _check(lib().gj_inlj_pairs_workspace_size(m, ctypes.byref(need)))
            workspace = _workspace(need.value, dev)
        fn = lib().gj_inlj_pairs if ordered else lib().gj_inlj_pairs_unordered
        _check(fn(self.handle, _ptr(d_probes), m, _ptr(out_pairs), _ptr(out_count), _ptr(workspace),
                  workspace.numel(), _stream(stream)))
        return out_pairs, out_count

    def lookup_cooperative(self, d_probes, degree=4, out=None, stream=None):
        """lookup() through the warp-collective search (groups of 2**degree lanes;
        cooperative_binary_search / harmonia_tree::lookup<Degree>): binary search and Harmonia."""
        torch = _torch()
        m = d_probes.numel()
        if out is None:
            out = _empty(m, torch.int32, d_probes.device)
        _check(lib().gj_index_lookup_cooperative(self.handle, _ptr(d_probes), m, _ptr(out), int(degree),
                                                 _stream(stream)))
        return out

    def lookup_sorted(self, d_probes, out=None, stream=None):
        """Block-wise sorted lookup (bws_lookup, src/index_lookup_common.cuh:398-549): the positions of lookup()."""
        torch = _torch()
        m = d_probes.numel()
        if out is None:
            out = _empty(m, torch.int32, d_probes.device)
        _check(lib().gj_index_lookup_sorted(self.handle, _ptr(d_probes), m, _ptr(out), _stream(stream)))
        return out

    def inlj_pairs_sorted(self, d_probes, out_pairs=None, out_count=None, workspace=None, stream=None):
        """The pairs of inlj_pairs() from block-wise sorted tiles (key order inside a tile)."""
        torch = _torch()
        m = d_probes.numel()
        dev = d_probes.device
        if out_pairs is None:
            out_pairs = _empty(2 * max(m, 1), torch.int32, dev)
        if out_count is None:
            out_count = torch.zeros(1, dtype=torch.int64, device=dev)
        if workspace is None:
            need = _sz(0)
            _check(lib().gj_inlj_pairs_workspace_size(m, ctypes.byref(need)))
            workspace = _workspace(need.value, dev)
        _check(lib().gj_inlj_pairs_sorted(self.handle, _ptr(d_probes), m, _ptr(out_pairs), _ptr(out_count),
                                          _ptr(workspace), workspace.numel(), _stream(stream)))
        return out_pairs, out_count

    def autotune_ordering(self, d_probes, stream=None):
        """(ORDER_PROBE, ORDER_SORTED_TILES or ORDER_PARTITIONED, best ms) for
        pairs of these probes."""
        o, ms = _u32(0), ctypes.c_float(0)
        _check(lib().gj_autotune_ordering(self.handle, _ptr(d_probes), d_probes.numel(), _stream(stream),
                                          ctypes.byref(o), ctypes.byref(ms)))
        return o.value, ms.value

    def inlj_pairs_host(self, h_probes, h_pairs, h_count, workspace=None, stream=None, ordered: bool = True):
        """inlj_pairs on pinned HOST tensors (probes int64, pairs int32 of 2m, count int64 of 1): the
        kernels read and write host memory directly; the result is valid after the stream syncs.
        ordered=False: the same pairs in the order their tiles finish (gj_inlj_pairs_host_unordered)."""
        m = h_probes.numel()
        if workspace is None:
            need = _sz(0)
            _check(lib().gj_inlj_pairs_host_workspace_size(m, ctypes.byref(need)))
            workspace = _workspace(need.value, _torch().device("cuda", _torch().cuda.current_device()))
        fn = lib().gj_inlj_pairs_host if ordered else lib().gj_inlj_pairs_host_unordered
        _check(fn(self.handle, _hptr(h_probes), m, _hptr(h_pairs), _hptr(h_count), _ptr(workspace), workspace.numel(),
                  _stream(stream)))
        return h_pairs, h_count

    @staticmethod
    def inlj_pairs_status(workspace, m: int, stream=None) -> None:
        """Raise GJError (GJ_ERR_TIMEOUT) if the last inlj_pairs on this
        workspace gave up a bounded wait; synchronises the stream."""
        _check(lib().gj_inlj_pairs_status(_ptr(workspace), workspace.numel(), m, _stream(stream)))

    def inlj_pairs_noalloc(self, d_probes, out_pairs, out_count, stream=None):
        """inlj_pairs without a workspace: the scratch is a fixed array inside the
        library, for callers that cannot allocate while probing (at most
        2^28 probes per call; overlapping calls must be serialised).  The
        caller's buffers are written in place: out_pairs must hold 2m int32 and
        out_count one int64, on the probes' device."""
        torch = _torch()
        m = d_probes.numel()
        if out_pairs.dtype != torch.int32 or out_pairs.numel() < 2 * m:
            raise ValueError(f"inlj_pairs_noalloc: out_pairs must be int32 with at least {2 * m} elements")
        if out_count.dtype != torch.int64 or out_count.numel() < 1:
            raise ValueError("inlj_pairs_noalloc: out_count must be int64 with at least one element")
        if out_pairs.device != d_probes.device or out_count.device != d_probes.device:
            raise ValueError("inlj_pairs_noalloc: probes, pairs and count must be on the same device")
        if not (out_pairs.is_contiguous() and out_count.is_contiguous()):
            raise ValueError("inlj_pairs_noalloc: out_pairs and out_count must be contiguous")
        _check(lib().gj_inlj_pairs_noalloc(self.handle, _ptr(d_probes), d_probes.numel(), _ptr(out_pairs),
                                           _ptr(out_count), _stream(stream)))
        return out_pairs, out_count

    def prepare_partitioned(self, stream=None):
        """Build and keep the partition directory partitioned_inlj probes
        through (otherwise it is built per call in the workspace)."""
        _check(lib().gj_index_prepare_partitioned(self.handle, _stream(stream)))
        return self

    def partitioned_inlj(self, d_probes, window_size: int = 0, radix_bits: int = 0, positions: bool = True,
                         pairs: bool = False, workspace=None, stream=None):
        """Windowed partitioned INLJ (src/index_lookup_partitioning.cu:436-507)."""
        torch = _torch()
        m = d_probes.numel()
        dev = d_probes.device
        window = window_size if window_size else max(m, 1)
        pos = _empty(m, torch.int32, dev) if positions else None
        prs = _empty(2 * max(m, 1), torch.int32, dev) if pairs else None
        cnt = torch.zeros(1, dtype=torch.int64, device=dev) if pairs else None
        if workspace is None:
            need = _sz(0)
            _check(lib().gj_partitioned_inlj_workspace_size(self.handle, window, radix_bits, ctypes.byref(need)))
            workspace = _workspace(need.value, dev)
        _check(lib().gj_partitioned_inlj(self.handle, _ptr(d_probes), m, window, radix_bits, _ptr(pos), _ptr(prs),
                                         _ptr(cnt), _ptr(workspace), workspace.numel(), _stream(stream)))
        return pos, prs, cnt

    def partitioned_lookup(self, d_part_keys, d_part_rows, out, stream=None):
        """partitioned_lookup_kernel (src/index_lookup_partitioning.cu:218-248): out[row] = lookup(key)."""
        _check(lib().gj_partitioned_lookup(self.handle, _ptr(d_part_keys), _ptr(d_part_rows), d_part_keys.numel(),
                                           _ptr(out), _stream(stream)))
        return out

    def free(self) -> None:
        if getattr(self, "_handle", None) is not None and self._handle.value:
            _check(lib().gj_index_free(self._handle))
            self._handle = _vp(None)

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class btree_index(abstract_index):
    """btree_index (src/indexes.cuh:93-147): clustered B+tree (node and leaf widths are build parameters)."""

    index_type = index_type_enum.btree


class harmonia_index(abstract_index):
    """harmonia_index (src/indexes.cuh:257-307): column size must be a multiple of 32."""

    index_type = index_type_enum.harmonia


class binary_search_index(abstract_index):
    """binary_search_index (src/indexes.cuh:336-375): lower bound, INVALID_POS at n."""

    index_type = index_type_enum.binary_search


class radix_spline_index(abstract_index):
    """radix_spline_index (src/indexes.cuh:176-248): 18 radix bits, spline error 32 by default."""

    index_type = index_type_enum.radix_spline


class no_op_index(abstract_index):
    """no_op_index (src/indexes.cuh:384-406): every probe returns INVALID_POS."""

    index_type = index_type_enum.no_op

    def construct(self, h_column, d_column, stream=None):
        torch = _torch()
        if d_column is None:
            d_column = torch.empty(0, dtype=torch.int64, device="cuda")
        return super().construct(h_column, d_column, stream)


class learned_index(abstract_index):
    """Trained position model (root + linear leaves) with an exact bounded search."""

    index_type = index_type_enum.learned

    def root_kind(self) -> int:
        """LEARNED_ROOT_LINEAR, LEARNED_ROOT_MLP or LEARNED_ROOT_SEGMENTS: the
        root the build kept."""
        r = _u32(0)
        _check(lib().gj_index_learned_root(self.handle, ctypes.byref(r)))
        return r.value

    def losses(self) -> Tuple[float, float]:
        """MLP root: sample loss at the quantile start and after training."""
        a, b = ctypes.c_double(0), ctypes.c_double(0)
        _check(lib().gj_index_learned_losses(self.handle, ctypes.byref(a), ctypes.byref(b)))
        return float(a.value), float(b.value)

    def stats(self) -> Tuple[int, float]:
        me = _u64(0)
        mw = ctypes.c_double(0)
        _check(lib().gj_index_learned_stats(self.handle, ctypes.byref(me), ctypes.byref(mw)))
        return int(me.value), float(mw.value)


class hash_index(abstract_index):
    """The reference's hash-join table (src/linear_probing_hashtable.cuh) as an index: linear probing,
    load factor <= 0.5; position of the equal key, else GJ_INVALID_POS."""

    index_type = index_type_enum.hash


_INDEX_CLASSES = {
    index_type_enum.btree: btree_index,
    index_type_enum.harmonia: harmonia_index,
    index_type_enum.binary_search: binary_search_index,
    index_type_enum.radix_spline: radix_spline_index,
    index_type_enum.no_op: no_op_index,
    index_type_enum.learned: learned_index,
    index_type_enum.hash: hash_index,
}


def make_index(kind, **params) -> abstract_index:
    """Index object for an index_type_enum value or a reference index name."""
    if isinstance(kind, str):
        kind = parse_index_type(kind)
    return _INDEX_CLASSES[index_type_enum(kind)](**params)


# --------------------------------------------------------------------------
# partitioning (src/partitioned_relation.hpp, src/index_lookup_partitioning.cu)
# --------------------------------------------------------------------------
@dataclasses.dataclass
class partitioned_relation:
    """partitioned_relation<T> (src/partitioned_relation.hpp:27-50) in SoA form:
    keys / rows of the partitioned tuples and the start offset of each partition."""

    keys: object
    rows: object
    offsets: object
    radix_bits: int

    @property
    def fanout(self) -> int:
        return 1 << self.radix_bits


def range_partition(d_keys, min_key: int, shift: int, radix_bits: int, workspace=None,
                    stream=None) -> partitioned_relation:
    torch = _torch()
    m = d_keys.numel()
    dev = d_keys.device
    out_k = _empty(max(m, 1), torch.int64, dev)
    out_r = _empty(max(m, 1), torch.int32, dev)
    offs = _empty((1 << radix_bits) + 1, torch.int64, dev)
    if workspace is None:
        need = _sz(0)
        _check(lib().gj_partition_workspace_size(m, radix_bits, ctypes.byref(need)))
        workspace = _workspace(need.value, dev)
    _check(lib().gj_range_partition(_ptr(d_keys), m, min_key, shift, radix_bits, _ptr(out_k), _ptr(out_r), _ptr(offs),
                                    _ptr(workspace), workspace.numel(), _stream(stream)))
    return partitioned_relation(out_k[:m], out_r[:m], offs, radix_bits)


# --------------------------------------------------------------------------
# star join (src/tpch/tpch_14_ij.cu, src/tpch/cpu_only.cpp:230-275)
# --------------------------------------------------------------------------
# --------------------------------------------------------------------------
# TPC-H Q14 from dbgen .tbl files (src/tpch/common.cpp, src/tpch/cpu_only.cpp)
# --------------------------------------------------------------------------
def tpch_day(year: int, month: int, day: int) -> int:
    """The loader's day number of a date (days since 1970-01-01)."""
    out = _u32(0)
    _check(lib().gj_tpch_day(year, month, day, ctypes.byref(out)))
    return out.value


def tpch_load_q14(lineitem_tbl: str, part_tbl: str) -> dict:
    """Q14's columns of two .tbl files as numpy arrays (copied out of the library's buffers)."""
    import numpy as np

    t = gj_q14_tables()
    _check(lib().gj_tpch_load_q14(lineitem_tbl.encode(), part_tbl.encode(), ctypes.byref(t)))
    try:
        nl, npart = int(t.n_lineitem), int(t.n_part)

        def arr(ptr, n, dtype):
            return np.ctypeslib.as_array(ptr, shape=(max(n, 1),))[:n].astype(dtype, copy=True)

        return {"l_partkey": arr(t.l_partkey, nl, np.uint32), "l_shipdate": arr(t.l_shipdate, nl, np.uint32),
                "l_extendedprice": arr(t.l_extendedprice, nl, np.int64),
                "l_discount": arr(t.l_discount, nl, np.int64), "p_partkey": arr(t.p_partkey, npart, np.uint64),
                "p_promo": arr(t.p_promo, npart, np.uint8)}
    finally:
        lib().gj_tpch_free_q14(ctypes.byref(t))


def tpch_q14(lineitem_tbl: str, part_tbl: str, stream=None):
    """Q14 on the GPU from two .tbl files: ((promo sum, total sum), promo_revenue percent)."""
    t = gj_q14_tables()
    _check(lib().gj_tpch_load_q14(lineitem_tbl.encode(), part_tbl.encode(), ctypes.byref(t)))
    try:
        sums = (ctypes.c_int64 * 2)()
        rev = ctypes.c_double(0)
        _check(lib().gj_tpch_q14(ctypes.byref(t), _stream(stream), sums, ctypes.byref(rev)))
        return (int(sums[0]), int(sums[1])), rev.value
    finally:
        lib().gj_tpch_free_q14(ctypes.byref(t))


def star_join_sum(dim_index: abstract_index, d_fk, d_date, d_price, d_discount, d_dim_flag, lo: int, hi: int,
                  out=None, stream=None, sorted_batches: bool = False):
    """Returns a 2-element int64 tensor [sum over flagged rows, sum over all rows].
    sorted_batches: the reference's pipelined ij_pbws order (gj_star_join_sum_sorted)."""
    torch = _torch()
    if out is None:
        out = torch.zeros(2, dtype=torch.int64, device=d_fk.device)
    fn = lib().gj_star_join_sum_sorted if sorted_batches else lib().gj_star_join_sum
    _check(fn(dim_index.handle, _ptr(d_fk), _ptr(d_date), _ptr(d_price), _ptr(d_discount), d_fk.numel(),
              _ptr(d_dim_flag), lo, hi, _ptr(out), _stream(stream)))
    return out


def learned_mlp_grad(d_params, hidden: int, d_x, d_y, stream=None):
    """GPU backward pass of the learned root MLP: (gradient of the summed
    squared error, that sum) over the samples (x, y)."""
    torch = _torch()
    grad = torch.empty_like(d_params)
    loss = torch.zeros(1, dtype=torch.float64, device=d_params.device)
    _check(lib().gj_learned_mlp_grad(_ptr(d_params), hidden, _ptr(d_x), _ptr(d_y), d_x.numel(), _ptr(grad),
                                     _ptr(loss), _stream(stream)))
    return grad, loss


# --------------------------------------------------------------------------
# batched lookup stream
# --------------------------------------------------------------------------
def autotune_partitioned(index, d_probes, stream=None):
    """Fastest (radix_bits, window_size, ms) of the partitioned INLJ on these probes."""
    bits, window, ms = _u32(0), _u64(0), ctypes.c_float(0)
    _check(lib().gj_autotune_partitioned(index.handle, _ptr(d_probes), d_probes.numel(), _stream(stream),
                                         ctypes.byref(bits), ctypes.byref(window), ctypes.byref(ms)))
    return bits.value, window.value, ms.value


def autotune_partitioned_btree(d_keys, d_probes, stream=None):
    """Fastest (node_keys, leaf_keys, radix_bits, window_size, ms) of a partitioned INLJ over a B+tree."""
    w, l, bits, window, ms = _u32(0), _u32(0), _u32(0), _u64(0), ctypes.c_float(0)
    _check(lib().gj_autotune_partitioned_btree(_ptr(d_keys), d_keys.numel(), _ptr(d_probes), d_probes.numel(),
                                               _stream(stream), ctypes.byref(w), ctypes.byref(l), ctypes.byref(bits),
                                               ctypes.byref(window), ctypes.byref(ms)))
    return w.value, l.value, bits.value, window.value, ms.value


def autotune_btree(d_keys, d_probes, stream=None):
    """Fastest (node_keys, leaf_keys, ms) of B+tree lookups of these probes into these keys."""
    w, l, ms = _u32(0), _u32(0), ctypes.c_float(0)
    _check(lib().gj_autotune_btree(_ptr(d_keys), d_keys.numel(), _ptr(d_probes), d_probes.numel(), _stream(stream),
                                   ctypes.byref(w), ctypes.byref(l), ctypes.byref(ms)))
    return w.value, l.value, ms.value


class batch_plan:
    """Plan of a batched lookup stream: many probe batches against several
    indexes, descriptors uploaded once.  run() enqueues one persistent kernel
    (mode 0) or one launch per batch (mode 1); run_graph() replays the run
    through a CUDA graph the plan captures; autotune() picks the tile shape."""

    def __init__(self, indexes, batch_index, probe_offset, batch_size, tile_items: int = 0, stream=None):
        import numpy as np

        self.indexes = list(indexes)  # the plan refers to them: keep them alive
        arr_t = _vp * len(self.indexes)
        handles = arr_t(*[ix.handle for ix in self.indexes])
        self._bi = np.ascontiguousarray(batch_index, dtype=np.uint32)
        self._po = np.ascontiguousarray(probe_offset, dtype=np.uint64)
        self._bs = np.ascontiguousarray(batch_size, dtype=np.uint64)
        self.num_batches = len(self._bi)
        out = _vp()
        _check(lib().gj_batch_plan_create(handles, len(self.indexes), self._bi.ctypes.data, self._po.ctypes.data,
                                          self._bs.ctypes.data, self.num_batches, tile_items, _stream(stream),
                                          ctypes.byref(out)))
        self._plan = out

    @property
    def tile_items(self) -> int:
        v = _u32(0)
        _check(lib().gj_batch_plan_tile_items(self._plan, ctypes.byref(v)))
        return v.value

    def run(self, d_probes, d_positions, mode: int = 0, d_done_ns=None, stream=None):
        _check(lib().gj_batch_plan_run(self._plan, _ptr(d_probes), _ptr(d_positions), mode, _ptr(d_done_ns),
                                       _stream(stream)))
        return d_positions

    def run_graph(self, d_probes, d_positions, mode: int = 0, d_done_ns=None, stream=None):
        _check(lib().gj_batch_plan_run_graph(self._plan, _ptr(d_probes), _ptr(d_positions), mode, _ptr(d_done_ns),
                                             _stream(stream)))
        return d_positions

    def autotune(self, d_probes, d_positions, stream=None):
        items, ms = _u32(0), ctypes.c_float(0)
        _check(lib().gj_batch_plan_autotune(self._plan, _ptr(d_probes), _ptr(d_positions), _stream(stream),
                                            ctypes.byref(items), ctypes.byref(ms)))
        return items.value, ms.value

    def free(self) -> None:
        if getattr(self, "_plan", None) is not None and self._plan.value:
            _check(lib().gj_batch_plan_free(self._plan))
            self._plan = _vp(None)

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def batch_lookup(indexes, batch_index, probe_offset, batch_size, d_probes, d_positions, mode: int = 0,
                 d_done_ns=None, graph: bool = False, stream=None):
    """One-shot batched lookup (plan, run, free); mode 0 = persistent kernel, 1 = one launch per batch."""
    plan = batch_plan(indexes, batch_index, probe_offset, batch_size, stream=stream)
    (plan.run_graph if graph else plan.run)(d_probes, d_positions, mode, d_done_ns, stream)
    _torch().cuda.synchronize(d_probes.device)
    plan.free()
    return d_positions


# --------------------------------------------------------------------------
# synthetic inputs (src/index_lookup_common.cuh:44-206)
# --------------------------------------------------------------------------
def generate_sorted_keys(n: int, distribution: int = DIST_UNIFORM, upper: int = 1 << 63, seed: int = 1,
                         device="cuda", stream=None):
    torch = _torch()
    out = _empty(max(n, 1), torch.int64, device)
    need = _sz(0)
    _check(lib().gj_generate_workspace_size(n, ctypes.byref(need)))
    ws = _workspace(need.value, out.device)
    _check(lib().gj_generate_sorted_keys(_ptr(out), n, distribution, upper, seed, _ptr(ws), ws.numel(),
                                         _stream(stream)))
    return out[:n]


def generate_probes(d_keys, m: int, theta: float = 0.0, absent_fraction: float = 0.0, seed: int = 2, stream=None):
    torch = _torch()
    out = _empty(max(m, 1), torch.int64, d_keys.device)
    _check(lib().gj_generate_probes(_ptr(d_keys), d_keys.numel(), _ptr(out), m, float(theta), float(absent_fraction),
                                    seed, _stream(stream)))
    return out[:m]


# --------------------------------------------------------------------------
# experiment configuration (src/index_lookup_config.hpp:18-37)
# --------------------------------------------------------------------------
@dataclasses.dataclass
class experiment_config:
    approach: str = "plain"
    index_type: str = "btree"
    scenario: str = "single"
    output_file: str = ""
    num_lookups: int = int(1e8)
    num_elements: int = int(1e6)
    max_bits: int = 0
    zipf_factor: float = 1.25
    block_size: int = 128
    dataset: str = "sparse"
    lookup_pattern: str = "uniform"
    sorted_lookups: bool = False
    partitioning_approach_ignore_bits: int = 4
    partitioning_approach_dynamic_bit_range: bool = True
    partitioning_approach_window_size: int = 10000


radix_bits = 11  # src/index_lookup_config.hpp:37 (the reference's fixed fanout)
