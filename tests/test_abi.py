"""The C ABI surface of libgpujoin.so, checked without a GPU: the library
loads, exports every function include/gpujoin.h declares, and rejects bad
arguments before touching the device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gpujoin.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gj_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_functions():
    names = declared_functions()
    assert "gj_index_build" in names and "gj_index_lookup" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(gj):
    L = gj.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, f"symbols declared in gpujoin.h but not exported: {missing}"


def test_bindings_cover_header(gj):
    assert sorted(gj.exported_symbols()) == declared_functions()


_C_TYPES = {"uint8_t": ctypes.c_uint8, "uint32_t": ctypes.c_uint32, "uint64_t": ctypes.c_uint64,
            "int64_t": ctypes.c_int64, "float": ctypes.c_float}


def declared_structs():
    """{name: [(field, C type, is_pointer)]} of every struct defined in the header."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for name, body in re.findall(r"typedef struct (\w+) \{(.*?)\} \1;", text, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            ctype, names = decl.split(None, 1)
            for f in names.split(","):
                f = f.strip()
                fields.append((f.lstrip("*"), ctype, f.startswith("*") or ctype.endswith("*")))
        out[name] = fields
    return out


def test_struct_mirrors_match_header(gj):
    # every struct of the ABI: the ctypes mirror has the header's fields, in
    # order, with the same types (a renamed or reordered field would pass
    # wrong values silently)
    structs = declared_structs()
    assert set(structs) == {"gj_index_params", "gj_q14_tables"}
    for name, fields in structs.items():
        mirror = getattr(gj, name)._fields_
        assert [f for f, _ in mirror] == [f for f, _, _ in fields], name
        for (f, ct), (_, c_type, ptr) in zip(mirror, fields):
            want = _C_TYPES[c_type.rstrip("*")]
            assert ct == (ctypes.POINTER(want) if ptr else want), (name, f)


def test_abi_version_and_names(gj):
    L = gj.lib()
    assert L.gj_abi_version() == 1
    for t in gj.index_type_enum:
        assert L.gj_index_type_name(int(t)).decode() == t.name
    assert L.gj_index_type_name(99) is None


def test_parse_index_type(gj):
    # src/indexes.cpp:5-19
    for name in ("btree", "harmonia", "binary_search", "radix_spline", "no_op", "learned", "hash"):
        assert gj.parse_index_type(name).name == name
    with pytest.raises(RuntimeError, match="unknown index type"):
        gj.parse_index_type("hash_table")


def test_params_defaults(gj):
    p = gj.default_params()
    assert p.struct_size == ctypes.sizeof(gj.gj_index_params)
    assert p.btree_node_keys == 15 and p.btree_leaf_keys == 4
    assert p.rs_radix_bits == 18 and p.rs_max_error == 32
    assert p.learned_leaves == 0 and p.learned_hidden == 32
    assert p.learned_root == gj.LEARNED_ROOT_AUTO and p.btree_start_bits == 0


def test_argument_errors_without_device(gj):
    L = gj.lib()
    out = ctypes.c_void_p()
    assert L.gj_index_build(0, None, None, 10, None, None, None) == 1
    assert L.gj_index_build(42, None, None, 10, None, None, ctypes.byref(out)) == 1
    assert b"unknown index type" in L.gj_last_error_string()
    assert L.gj_index_lookup(None, None, 0, None, None) == 1
    assert L.gj_index_free(None) == 0
    sz = ctypes.c_size_t()
    assert L.gj_inlj_pairs_workspace_size(1 << 20, ctypes.byref(sz)) == 0 and sz.value > 0
    assert L.gj_partition_workspace_size(100, 0, ctypes.byref(sz)) == 1
    assert L.gj_partition_workspace_size(100, 13, ctypes.byref(sz)) == 1
    assert L.gj_generate_workspace_size(1000, ctypes.byref(sz)) == 0


def test_oversized_column_rejected(gj):
    L = gj.lib()
    out = ctypes.c_void_p()
    # 2^32 - 1 keys cannot be addressed by 32-bit positions ('value_t' does not suffice)
    assert L.gj_index_build(2, ctypes.c_void_p(16), None, (1 << 32) - 1, None, None, ctypes.byref(out)) == 8


def test_experiment_config_defaults(gj):
    # src/index_lookup_config.hpp:18-37
    c = gj.experiment_config()
    assert c.approach == "plain" and c.index_type == "btree" and c.block_size == 128
    assert c.partitioning_approach_window_size == 10000 and gj.radix_bits == 11
