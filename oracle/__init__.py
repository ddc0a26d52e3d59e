"""CPU oracle for the gpujoin INLJ probe path (TEST INFRASTRUCTURE ONLY).

This package is the checker.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline / reference legs of ``bench.py`` may import it; the CUDA
product in ``gpujoin_gb300`` never does, and has no CPU fallback.

``liboracle.so`` is the C restatement in ``oracle.c`` (each routine cites the
reference file:line it follows).  ``_ref/libgjref.so`` -- built only where the
reference tree is present -- runs the reference's own ``search.cuh``,
``btree.cuh`` and ``harmonia.cuh`` lookups on the host and pins the
restatement (see ``ref_harness.cpp``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
INV = 0xFFFFFFFF

_u64p = ctypes.POINTER(ctypes.c_uint64)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_i64p = ctypes.POINTER(ctypes.c_int64)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, if asked and possible, _ref/libgjref.so)."""
    targets = ["oracle"]
    if ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


_LIB: Optional[ctypes.CDLL] = None
_REF: Optional[ctypes.CDLL] = None


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc_lower_bound.restype = ctypes.c_uint64
        L.orc_lower_bound.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_branch_free_lower_bound.restype = ctypes.c_uint64
        L.orc_branch_free_lower_bound.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_branchy_binary_search.restype = ctypes.c_uint64
        L.orc_branchy_binary_search.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint64]
        for name in ("orc_bs_lookup", "orc_bs_branch_free_lookup", "orc_exact_lookup"):
            f = getattr(L, name)
            f.restype = None
            f.argtypes = [_u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64, _u32p, ctypes.c_int]
        L.orc_btree_build.restype = _vp
        L.orc_btree_build.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
        L.orc_btree_lookup.restype = None
        L.orc_btree_lookup.argtypes = [_vp, _u64p, ctypes.c_uint64, _u32p, ctypes.c_int]
        L.orc_btree_lower_bound.restype = None
        L.orc_btree_lower_bound.argtypes = [_vp, _u64p, ctypes.c_uint64, _u32p, ctypes.c_int]
        L.orc_btree_depth.restype = ctypes.c_uint32
        L.orc_btree_depth.argtypes = [_vp]
        L.orc_btree_free.argtypes = [_vp]
        L.orc_btree_nodes.restype = ctypes.c_uint64
        L.orc_btree_nodes.argtypes = [_vp]
        L.orc_btree_write_pages.restype = ctypes.c_int64
        L.orc_btree_write_pages.argtypes = [_vp, _u8p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64,
                                            ctypes.c_uint64, ctypes.c_uint64]
        L.orc_harmonia_build.restype = _vp
        L.orc_harmonia_build.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint32, ctypes.POINTER(ctypes.c_int)]
        L.orc_harmonia_lookup.restype = None
        L.orc_harmonia_lookup.argtypes = [_vp, _u64p, ctypes.c_uint64, _u32p, ctypes.c_int]
        L.orc_harmonia_arrays.restype = None
        L.orc_harmonia_arrays.argtypes = [_vp, ctypes.POINTER(_u64p), _u64p, ctypes.POINTER(_u64p), _u64p,
                                          ctypes.POINTER(ctypes.c_uint32)]
        L.orc_harmonia_free.argtypes = [_vp]
        L.orc_rs_build.restype = _vp
        L.orc_rs_build.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
        L.orc_rs_lookup.restype = None
        L.orc_rs_lookup.argtypes = [_vp, _u64p, _u64p, ctypes.c_uint64, _u32p, ctypes.c_int]
        L.orc_rs_estimate.restype = ctypes.c_double
        L.orc_rs_estimate.argtypes = [_vp, ctypes.c_uint64]
        L.orc_rs_arrays.restype = None
        L.orc_rs_arrays.argtypes = [_vp, ctypes.POINTER(_u32p), _u64p, ctypes.POINTER(_u64p),
                                    ctypes.POINTER(_f64p), _u64p, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_rs_free.argtypes = [_vp]
        L.orc_range_partition.restype = None
        L.orc_range_partition.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32,
                                          ctypes.c_uint32, _u64p, _u32p, _u64p]
        L.orc_pairs_from_positions.restype = ctypes.c_uint64
        L.orc_pairs_from_positions.argtypes = [_u32p, ctypes.c_uint64, _u32p, _u32p]
        L.orc_star_join.restype = None
        L.orc_star_join.argtypes = [_u32p, _u32p, _i64p, _i64p, ctypes.c_uint64, _u64p, _u8p,
                                    ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, _i64p]
        L.orc_mix64.restype = ctypes.c_uint64
        L.orc_mix64.argtypes = [ctypes.c_uint64]
        L.orc_zipf_rank.restype = ctypes.c_uint64
        L.orc_zipf_rank.argtypes = [ctypes.c_uint64, ctypes.c_double, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_permute.restype = ctypes.c_uint64
        L.orc_permute.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.orc_zipf_probes.restype = None
        L.orc_zipf_probes.argtypes = [_u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64, ctypes.c_double,
                                      ctypes.c_uint64, ctypes.c_int]
        L.orc_mlp_loss_grad.restype = ctypes.c_double
        L.orc_mlp_loss_grad.argtypes = [_f32p, ctypes.c_int, _f32p, _f32p, ctypes.c_uint64, _f64p]
        L.orc_mlp_forward.restype = ctypes.c_float
        L.orc_mlp_forward.argtypes = [_f32p, ctypes.c_int, ctypes.c_float]
        L.orc_hardware_threads.restype = ctypes.c_int
        _LIB = L
    return _LIB


def ref_lib() -> Optional[ctypes.CDLL]:
    """The reference-built checker, or None where it cannot exist."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libgjref.so")
        if not os.path.exists(path):
            try:
                build(ref=True)
            except Exception:
                return None
        if not os.path.exists(path):
            return None
        R = ctypes.CDLL(path)
        R.ref_bs_lookup.restype = None
        R.ref_bs_lookup.argtypes = [_u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64, _u32p]
        R.ref_bs_branch_free_lookup.restype = None
        R.ref_bs_branch_free_lookup.argtypes = [_u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64, _u32p]
        R.ref_branchy_binary_search.restype = ctypes.c_uint64
        R.ref_branchy_binary_search.argtypes = [_u64p, ctypes.c_uint64, ctypes.c_uint64]
        R.ref_btree_lookup.restype = ctypes.c_int
        R.ref_btree_lookup.argtypes = [_u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64, _u32p,
                                       ctypes.POINTER(ctypes.c_uint32)]
        R.ref_btree_layout.restype = None
        R.ref_btree_layout.argtypes = [_u64p]
        R.ref_btree_canonical.restype = ctypes.c_uint64
        R.ref_btree_canonical.argtypes = [_u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64]
        R.ref_harmonia_lookup_u64.restype = ctypes.c_int
        R.ref_harmonia_lookup_u64.argtypes = [_u64p, ctypes.c_uint64, _u64p, ctypes.c_uint64, _u32p]
        R.ref_harmonia_arrays_u64.restype = ctypes.c_int
        R.ref_harmonia_arrays_u64.argtypes = [_u64p, ctypes.c_uint64, _u64p, _u64p, _u64p, _u64p,
                                              ctypes.POINTER(ctypes.c_uint32)]
        R.ref_harmonia_lookup_u32.restype = ctypes.c_int
        R.ref_harmonia_lookup_u32.argtypes = [_u32p, ctypes.c_uint64, ctypes.c_uint32, _u32p,
                                              ctypes.c_uint64, _u32p]
        _REF = R
    return _REF


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint64)


# --------------------------------------------------------------------------
# lookups
# --------------------------------------------------------------------------
def bs_lookup(col, probes, threads: int = 0, branch_free: bool = False) -> np.ndarray:
    col, probes = _u64(col), _u64(probes)
    out = np.empty(len(probes), dtype=np.uint32)
    f = lib().orc_bs_branch_free_lookup if branch_free else lib().orc_bs_lookup
    f(_ptr(col, _u64p), len(col), _ptr(probes, _u64p), len(probes), _ptr(out, _u32p), threads)
    return out


def exact_lookup(col, probes, threads: int = 0) -> np.ndarray:
    col, probes = _u64(col), _u64(probes)
    out = np.empty(len(probes), dtype=np.uint32)
    lib().orc_exact_lookup(_ptr(col, _u64p), len(col), _ptr(probes, _u64p), len(probes), _ptr(out, _u32p), threads)
    return out


class BTree:
    """Clustered B+tree restatement (src/btree.cuh); 247/246 = reference page geometry."""

    def __init__(self, col, leaf_keys: int = 247, inner_keys: int = 246):
        self.col = _u64(col)
        self._h = lib().orc_btree_build(_ptr(self.col, _u64p), len(self.col), leaf_keys, inner_keys)
        if not self._h:
            raise RuntimeError("btree: empty column")

    @property
    def depth(self) -> int:
        return lib().orc_btree_depth(self._h)

    def lookup(self, probes, threads: int = 0) -> np.ndarray:
        probes = _u64(probes)
        out = np.empty(len(probes), dtype=np.uint32)
        lib().orc_btree_lookup(self._h, _ptr(probes, _u64p), len(probes), _ptr(out, _u32p), threads)
        return out

    def lower_bound(self, probes, threads: int = 0) -> np.ndarray:
        """bs_lookup's results (first key >= probe, INV at n) through the tree."""
        probes = _u64(probes)
        out = np.empty(len(probes), dtype=np.uint32)
        lib().orc_btree_lower_bound(self._h, _ptr(probes, _u64p), len(probes), _ptr(out, _u32p), threads)
        return out

    def pages(self, page_bytes: int, keys_off: int, children_off: int, pages_base: int, col_base: int):
        """The tree in the reference's device page layout (orc_btree_write_pages):
        (uint8 page image, root node number).  Pointers are formed from
        pages_base (where the image will be copied) and col_base (the device
        column)."""
        nodes = lib().orc_btree_nodes(self._h)
        out = np.empty(nodes * page_bytes, dtype=np.uint8)
        root = lib().orc_btree_write_pages(self._h, _ptr(out, _u8p), page_bytes, keys_off, children_off,
                                           pages_base, col_base)
        if root < 0:
            raise ValueError("btree pages: offsets do not fit the page")
        return out, int(root)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_btree_free(self._h)
            self._h = None


class Harmonia:
    """Harmonia restatement (src/harmonia.cuh:133-404, :640-668)."""

    def __init__(self, col, max_keys: int = 32):
        self.col = _u64(col)
        err = ctypes.c_int(0)
        self._h = lib().orc_harmonia_build(_ptr(self.col, _u64p), len(self.col), max_keys, ctypes.byref(err))
        if not self._h:
            raise RuntimeError(f"harmonia: build failed (code {err.value})")

    def lookup(self, probes, threads: int = 0) -> np.ndarray:
        probes = _u64(probes)
        out = np.empty(len(probes), dtype=np.uint32)
        lib().orc_harmonia_lookup(self._h, _ptr(probes, _u64p), len(probes), _ptr(out, _u32p), threads)
        return out

    def arrays(self) -> Tuple[np.ndarray, np.ndarray, int]:
        kp, cp = _u64p(), _u64p()
        nk, nc, d = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint32()
        lib().orc_harmonia_arrays(self._h, ctypes.byref(kp), ctypes.byref(nk), ctypes.byref(cp),
                                  ctypes.byref(nc), ctypes.byref(d))
        keys = np.ctypeslib.as_array(kp, shape=(max(nk.value, 1),))[: nk.value].copy()
        children = np.ctypeslib.as_array(cp, shape=(nc.value,)).copy()
        return keys, children, d.value

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_harmonia_free(self._h)
            self._h = None


class RadixSpline:
    """RadixSpline restatement (builder: published GreedySplineCorridor; lookup src/rs.cuh:118-154)."""

    def __init__(self, col, radix_bits: int = 18, max_error: int = 32):
        self.col = _u64(col)
        self._h = lib().orc_rs_build(_ptr(self.col, _u64p), len(self.col), radix_bits, max_error)
        if not self._h:
            raise RuntimeError("radix spline: invalid parameters")

    def lookup(self, probes, threads: int = 0) -> np.ndarray:
        probes = _u64(probes)
        out = np.empty(len(probes), dtype=np.uint32)
        lib().orc_rs_lookup(self._h, _ptr(self.col, _u64p), _ptr(probes, _u64p), len(probes), _ptr(out, _u32p),
                            threads)
        return out

    def estimate(self, key: int) -> float:
        return lib().orc_rs_estimate(self._h, int(key))

    def arrays(self):
        tp, xp, yp = _u32p(), _u64p(), _f64p()
        tl, npt, sb = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint32()
        lib().orc_rs_arrays(self._h, ctypes.byref(tp), ctypes.byref(tl), ctypes.byref(xp), ctypes.byref(yp),
                            ctypes.byref(npt), ctypes.byref(sb))
        table = np.ctypeslib.as_array(tp, shape=(tl.value,)).copy()
        sx = np.ctypeslib.as_array(xp, shape=(npt.value,)).copy()
        sy = np.ctypeslib.as_array(yp, shape=(npt.value,)).copy()
        return table, sx, sy, sb.value

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_rs_free(self._h)
            self._h = None


# --------------------------------------------------------------------------
# partition, pairs, star join
# --------------------------------------------------------------------------
def range_partition(keys, min_key: int, shift: int, radix_bits: int):
    keys = _u64(keys)
    m = len(keys)
    ok = np.empty(m, dtype=np.uint64)
    orows = np.empty(m, dtype=np.uint32)
    offsets = np.empty((1 << radix_bits) + 1, dtype=np.uint64)
    lib().orc_range_partition(_ptr(keys, _u64p), m, int(min_key), shift, radix_bits, _ptr(ok, _u64p),
                              _ptr(orows, _u32p), _ptr(offsets, _u64p))
    return ok, orows, offsets


def fast_positions(col, probes, threads: int = 0) -> Tuple[np.ndarray, np.ndarray]:
    """(lower bound, exact) positions of every probe for large checks: the
    lower bound (bs_lookup's semantics) through the oracle B+tree, and the
    exact-match form (B+tree / Harmonia / hash semantics) derived from it."""
    col, probes = _u64(col), _u64(probes)
    lb = BTree(col, 247, 246).lower_bound(probes, threads)
    ok = lb != INV
    hit = np.zeros(len(probes), dtype=bool)
    hit[ok] = col[lb[ok]] == probes[ok]
    return lb, np.where(hit, lb, np.uint32(INV)).astype(np.uint32)


def pairs_from_positions(pos) -> Tuple[np.ndarray, np.ndarray]:
    pos = np.ascontiguousarray(pos, dtype=np.uint32)
    rows = np.empty(len(pos), dtype=np.uint32)
    bpos = np.empty(len(pos), dtype=np.uint32)
    c = lib().orc_pairs_from_positions(_ptr(pos, _u32p), len(pos), _ptr(rows, _u32p), _ptr(bpos, _u32p))
    return rows[:c].copy(), bpos[:c].copy()


def star_join(fk, date, price, disc, dim_keys, dim_flag, lo: int, hi: int) -> Tuple[int, int]:
    fk = np.ascontiguousarray(fk, dtype=np.uint32)
    date = np.ascontiguousarray(date, dtype=np.uint32)
    price = np.ascontiguousarray(price, dtype=np.int64)
    disc = np.ascontiguousarray(disc, dtype=np.int64)
    dim_keys = _u64(dim_keys)
    dim_flag = np.ascontiguousarray(dim_flag, dtype=np.uint8)
    out = np.zeros(2, dtype=np.int64)
    lib().orc_star_join(_ptr(fk, _u32p), _ptr(date, _u32p), _ptr(price, _i64p), _ptr(disc, _i64p), len(fk),
                        _ptr(dim_keys, _u64p), _ptr(dim_flag, _u8p), len(dim_keys), lo, hi, _ptr(out, _i64p))
    return int(out[0]), int(out[1])


# --------------------------------------------------------------------------
# generators and learned-model math
# --------------------------------------------------------------------------
def mix64(x: int) -> int:
    return lib().orc_mix64(x & 0xFFFFFFFFFFFFFFFF)


def zipf_rank(n: int, q: float, seed: int, index: int) -> int:
    return lib().orc_zipf_rank(n, q, seed, index)


def permute(x: int, n: int, seed: int) -> int:
    return lib().orc_permute(x, n, seed)


def zipf_probes(col, m: int, q: float, seed: int, threads: int = 0) -> np.ndarray:
    col = _u64(col)
    out = np.empty(m, dtype=np.uint64)
    lib().orc_zipf_probes(_ptr(col, _u64p), len(col), _ptr(out, _u64p), m, float(q), seed, threads)
    return out


def mlp_loss_grad(params, hidden: int, x, y):
    params = np.ascontiguousarray(params, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    g = np.zeros(len(params), dtype=np.float64)
    loss = lib().orc_mlp_loss_grad(_ptr(params, _f32p), hidden, _ptr(x, _f32p), _ptr(y, _f32p), len(x),
                                   _ptr(g, _f64p))
    return loss, g


def mlp_forward(params, hidden: int, x: float) -> float:
    params = np.ascontiguousarray(params, dtype=np.float32)
    return lib().orc_mlp_forward(_ptr(params, _f32p), hidden, float(x))


def hardware_threads() -> int:
    return lib().orc_hardware_threads()


# --------------------------------------------------------------------------
# reference-built checker
# --------------------------------------------------------------------------
def ref_bs_lookup(col, probes) -> Optional[np.ndarray]:
    R = ref_lib()
    if R is None:
        return None
    col, probes = _u64(col), _u64(probes)
    out = np.empty(len(probes), dtype=np.uint32)
    R.ref_bs_lookup(_ptr(col, _u64p), len(col), _ptr(probes, _u64p), len(probes), _ptr(out, _u32p))
    return out


def ref_bs_branch_free_lookup(col, probes) -> Optional[np.ndarray]:
    R = ref_lib()
    if R is None:
        return None
    col, probes = _u64(col), _u64(probes)
    out = np.empty(len(probes), dtype=np.uint32)
    R.ref_bs_branch_free_lookup(_ptr(col, _u64p), len(col), _ptr(probes, _u64p), len(probes), _ptr(out, _u32p))
    return out


def ref_btree_lookup(col, probes):
    R = ref_lib()
    if R is None:
        return None
    col, probes = _u64(col), _u64(probes)
    out = np.empty(len(probes), dtype=np.uint32)
    depth = ctypes.c_uint32(0)
    rc = R.ref_btree_lookup(_ptr(col, _u64p), len(col), _ptr(probes, _u64p), len(probes), _ptr(out, _u32p),
                            ctypes.byref(depth))
    if rc != 0:
        raise RuntimeError("reference btree build failed")
    return out


def ref_btree_layout():
    """(page size, header size, separator offset, child pointer offset,
    separators per inner node, keys per leaf) of the reference's uint64
    B+tree pages, or None without the reference-built checker."""
    R = ref_lib()
    if R is None:
        return None
    out = np.zeros(6, dtype=np.uint64)
    R.ref_btree_layout(_ptr(out, _u64p))
    return [int(v) for v in out]


def ref_btree_canonical(col):
    """The reference's host-built B+tree as ref_btree_canonical's word stream."""
    R = ref_lib()
    if R is None:
        return None
    col = _u64(col)
    need = R.ref_btree_canonical(_ptr(col, _u64p), len(col), None, 0)
    out = np.empty(max(need, 1), dtype=np.uint64)
    R.ref_btree_canonical(_ptr(col, _u64p), len(col), _ptr(out, _u64p), need)
    return out[:need]


def btree_canonical_from_pages(pages, page_bytes, keys_off, children_off, root, pages_base, col_base):
    """The same word stream read back from a page image (BTree.pages)."""
    words = []
    level = [root]
    while level:
        nxt = []
        for node in level:
            pg = pages[node * page_bytes:(node + 1) * page_bytes]
            count = int(pg[:2].view(np.uint16)[0])
            final = int(pg[3])
            words += [count, final]
            words += [int(k) for k in pg[keys_off:keys_off + 8 * count].view(np.uint64)]
            ptrs = pg[children_off:children_off + 8 * (count + 1)].view(np.uint64)
            for p in ptrs:
                if final:
                    words.append((int(p) - col_base) // 8)
                else:
                    nxt.append((int(p) - pages_base) // page_bytes)
        level = nxt
    return np.array(words, dtype=np.uint64)


def ref_harmonia_lookup(col, probes):
    R = ref_lib()
    if R is None:
        return None
    col, probes = _u64(col), _u64(probes)
    out = np.empty(len(probes), dtype=np.uint32)
    rc = R.ref_harmonia_lookup_u64(_ptr(col, _u64p), len(col), _ptr(probes, _u64p), len(probes), _ptr(out, _u32p))
    if rc != 0:
        raise RuntimeError("reference harmonia construct threw")
    return out


def ref_harmonia_arrays(col):
    R = ref_lib()
    if R is None:
        return None
    col = _u64(col)
    nk, nc, d = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint32()
    rc = R.ref_harmonia_arrays_u64(_ptr(col, _u64p), len(col), None, ctypes.byref(nk), None, ctypes.byref(nc),
                                   ctypes.byref(d))
    if rc != 0:
        raise RuntimeError("reference harmonia construct threw")
    keys = np.empty(max(nk.value, 1), dtype=np.uint64)
    children = np.empty(nc.value, dtype=np.uint64)
    R.ref_harmonia_arrays_u64(_ptr(col, _u64p), len(col), _ptr(keys, _u64p), ctypes.byref(nk),
                              _ptr(children, _u64p), ctypes.byref(nc), ctypes.byref(d))
    return keys[: nk.value], children, d.value


def ref_harmonia_lookup_u32(col, node_size: int, probes):
    R = ref_lib()
    if R is None:
        return None
    col = np.ascontiguousarray(col, dtype=np.uint32)
    probes = np.ascontiguousarray(probes, dtype=np.uint32)
    out = np.empty(len(probes), dtype=np.uint32)
    rc = R.ref_harmonia_lookup_u32(_ptr(col, _u32p), len(col), node_size, _ptr(probes, _u32p), len(probes),
                                   _ptr(out, _u32p))
    if rc != 0:
        raise RuntimeError(f"reference harmonia construct failed (code {rc})")
    return out
