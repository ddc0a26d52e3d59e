// ref_harness.cpp -- CPU checker built FROM THE REFERENCE'S OWN HEADERS.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file against the
// reference sources where they lie (src/search.cuh, src/btree.cuh,
// src/harmonia.cuh) into oracle/_ref/libgjref.so.  It is used to pin the C
// restatement in oracle/oracle.c and to generate tests/golden/ fixtures.
// Nothing here is product code and nothing of the reference is copied: the
// reference headers are #included from their original location.
//
// The device lookups are executed on the host through oracle/shim/devstubs.h
// (host stand-ins for the warp intrinsics); __device__ is a no-op attribute
// for a host compiler.

#include <cstdint>
#include <cstring>
#include <iostream>
#include <limits>
#include <memory>
#include <numeric>
#include <sstream>
#include <vector>

#include <cuda_runtime.h>  // CUDA attribute macros (__device__ etc.) for a host compiler

#include "search.cuh"
#include "btree.cuh"
#include "harmonia.cuh"

namespace {
template <class T>
using host_alloc = std::allocator<T>;

constexpr uint32_t kInv32 = 0xFFFFFFFFu;

// The reference's builders print progress to std::cout; keep the checker quiet.
struct quiet_cout {
    std::streambuf* old;
    std::ostringstream sink;
    quiet_cout() : old(std::cout.rdbuf(sink.rdbuf())) {}
    ~quiet_cout() { std::cout.rdbuf(old); }
};
}  // namespace

extern "C" {

// binary_search_index::cooperative_lookup (src/indexes.cuh:357-361) over the
// reference's lower_bound (src/search.cuh:26-41).
void ref_bs_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes, uint64_t m, uint32_t* out) {
    for (uint64_t i = 0; i < m; ++i) {
        const device_size_t pos = lower_bound(probes[i], col, n);
        out[i] = pos < n ? static_cast<uint32_t>(pos) : kInv32;
    }
}

// branch_free_lower_bound_search (src/search.cuh:143-158), defined for n >= 2.
void ref_bs_branch_free_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes, uint64_t m,
                               uint32_t* out) {
    for (uint64_t i = 0; i < m; ++i) {
        const device_size_t pos = branch_free_lower_bound_search(probes[i], col, n);
        out[i] = pos < n ? static_cast<uint32_t>(pos) : kInv32;
    }
}

// branchy_binary_search (src/search.cuh:86-101) on one array.
uint64_t ref_branchy_binary_search(const uint64_t* arr, uint64_t n, uint64_t key) {
    return branchy_binary_search(key, arr, n);
}

// Clustered B+tree (src/btree.cuh) built with load factor 1.0 as in
// btree_index::construct (src/indexes.cuh:126-127); lookup :504-531.
int ref_btree_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes, uint64_t m, uint32_t* out,
                     uint32_t* depth_out) {
    using tree_t = index_structures::btree<uint64_t, uint64_t, host_alloc, ~0ull>;
    if (n == 0) return 1;
    std::vector<uint64_t> keys(col, col + n);
    quiet_cout q;
    tree_t tree;
    tree.construct(keys, 1.0f);
    tree_t::device_handle_t h{};
    h.column_begin = keys.data();
    h.column_end = keys.data() + keys.size();
    h.root = tree.root;
    uint32_t depth = 0;
    {
        const tree_t::NodeBase* node = tree.root;
        for (;;) {
            ++depth;
            auto inner = static_cast<const tree_t::InnerNode*>(node);
            if (inner->header.isFinalInner) break;
            node = static_cast<const tree_t::NodeBase*>(inner->children[0]);
        }
    }
    for (uint64_t i = 0; i < m; ++i) {
        const uint64_t r = tree_t::lookup(h, probes[i]);
        out[i] = r == ~0ull ? kInv32 : static_cast<uint32_t>(r);
    }
    if (depth_out) *depth_out = depth;
    return 0;
}

// The reference's B+tree page layout (src/btree.cuh:30-64) for uint64 keys
// and values: page size, header size, offsets of the separators and of the
// child pointers within an inner page, separators per inner node, keys per
// leaf.
void ref_btree_layout(uint64_t out[6]) {
    using tree_t = index_structures::btree<uint64_t, uint64_t, host_alloc, ~0ull>;
    out[0] = tree_t::page_size;
    out[1] = sizeof(tree_t::NodeBase);
    out[2] = __builtin_offsetof(tree_t::InnerNode, keys);
    out[3] = __builtin_offsetof(tree_t::InnerNode, children);
    out[4] = tree_t::InnerNode::maxEntries;
    out[5] = tree_t::LeafNode::maxEntries;
}

// The reference's host-built B+tree (load factor 1.0) as a canonical word
// stream, breadth first from the root: per inner node its count, its
// isFinalInner flag and its count separators, and for a final inner node
// its count + 1 children as column positions.  Writes at most cap words;
// returns the stream's length.
uint64_t ref_btree_canonical(const uint64_t* col, uint64_t n, uint64_t* out, uint64_t cap) {
    using tree_t = index_structures::btree<uint64_t, uint64_t, host_alloc, ~0ull>;
    if (n == 0) return 0;
    std::vector<uint64_t> keys(col, col + n);
    quiet_cout q;
    tree_t tree;
    tree.construct(keys, 1.0f);
    uint64_t len = 0;
    auto put = [&](uint64_t w) {
        if (len < cap) out[len] = w;
        ++len;
    };
    std::vector<const tree_t::InnerNode*> level{static_cast<const tree_t::InnerNode*>(tree.root)};
    while (!level.empty()) {
        std::vector<const tree_t::InnerNode*> next;
        for (const tree_t::InnerNode* nd : level) {
            put(nd->header.count);
            put(nd->header.isFinalInner ? 1 : 0);
            for (unsigned i = 0; i < nd->header.count; ++i) put(nd->keys[i]);
            for (unsigned i = 0; i <= nd->header.count; ++i) {
                if (nd->header.isFinalInner)
                    put(static_cast<uint64_t>(static_cast<const uint64_t*>(nd->children[i]) - keys.data()));
                else
                    next.push_back(static_cast<const tree_t::InnerNode*>(nd->children[i]));
            }
        }
        level.swap(next);
    }
    return len;
}

// Harmonia with 32 keys per node (fanout 33, src/indexes.cuh:264), host
// lookup src/harmonia.cuh:640-668.  Returns 1 if construct() throws.
int ref_harmonia_lookup_u64(const uint64_t* col, uint64_t n, const uint64_t* probes, uint64_t m,
                            uint32_t* out) {
    using tree_t = harmonia::harmonia_tree<uint64_t, uint64_t, host_alloc, 32 + 1, ~0ull>;
    // The host lookup reads node_start[lb] one past a leaf node for probes
    // above the largest key; spare capacity keeps that read inside the buffer.
    std::vector<uint64_t> keys;
    keys.reserve(n + 64);
    keys.assign(col, col + n);
    quiet_cout q;
    tree_t tree;
    try {
        tree.construct(keys);
    } catch (const std::exception&) {
        return 1;
    }
    for (uint64_t i = 0; i < m; ++i) {
        const uint64_t r = tree.lookup(probes[i]);
        out[i] = r == ~0ull ? kInv32 : static_cast<uint32_t>(r);
    }
    return 0;
}

// The built Harmonia arrays (inner key array, children prefix array) for
// fanout 33 over u64 keys, so the product's builder can be compared array
// by array.  Pass null buffers to query the sizes.
int ref_harmonia_arrays_u64(const uint64_t* col, uint64_t n, uint64_t* keys_out, uint64_t* nkeys,
                            uint64_t* children_out, uint64_t* nchildren, uint32_t* depth) {
    using tree_t = harmonia::harmonia_tree<uint64_t, uint64_t, host_alloc, 32 + 1, ~0ull>;
    std::vector<uint64_t> keys(col, col + n);
    quiet_cout q;
    tree_t tree;
    try {
        tree.construct(keys);
    } catch (const std::exception&) {
        return 1;
    }
    *nkeys = tree.inner_nodes_key_array_size;
    *nchildren = tree.children.size();
    *depth = tree.depth;
    if (keys_out) std::memcpy(keys_out, tree.keys.data(), sizeof(uint64_t) * tree.inner_nodes_key_array_size);
    if (children_out) std::memcpy(children_out, tree.children.data(), sizeof(uint64_t) * tree.children.size());
    return 0;
}

// The reference's known-answer setting (test/test_harmonia.cu:37-55,
// test/main.cu:144-164): uint32 keys with a configurable node size.
int ref_harmonia_lookup_u32(const uint32_t* col, uint64_t n, uint32_t node_size, const uint32_t* probes,
                            uint64_t m, uint32_t* out) {
    std::vector<uint32_t> keys;
    keys.reserve(n + 64);
    keys.assign(col, col + n);
    quiet_cout q;
    auto run = [&](auto& tree) -> int {
        try {
            tree.construct(keys);
        } catch (const std::exception&) {
            return 1;
        }
        for (uint64_t i = 0; i < m; ++i) out[i] = tree.lookup(probes[i]);
        return 0;
    };
    switch (node_size) {
        case 4: { harmonia::harmonia_tree<uint32_t, uint32_t, host_alloc, 4 + 1, kInv32> t; return run(t); }
        case 8: { harmonia::harmonia_tree<uint32_t, uint32_t, host_alloc, 8 + 1, kInv32> t; return run(t); }
        case 32: { harmonia::harmonia_tree<uint32_t, uint32_t, host_alloc, 32 + 1, kInv32> t; return run(t); }
        default: return 2;
    }
}

}  // extern "C"
