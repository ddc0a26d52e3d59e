// ref_gpu.cu -- the reference's OWN device lookups, for timing beside the
// library's kernels.
//
// TEST AND BENCHMARK INFRASTRUCTURE ONLY.  oracle/Makefile compiles this
// file with the reference's headers where they lie (src/search.cuh,
// src/harmonia.cuh) into a cubin for sm_103a (oracle/_ref/refgpu.cubin);
// bench.py loads it through the CUDA driver API on the GPU host.  Nothing of
// the reference is copied: its headers are #included from their location.
//
// The kernels follow lookup_kernel (src/index_lookup_common.cuh:217-245),
// launched as the reference launches it (src/index_lookup_new.cu:191-196:
// one thread per probe, 128-thread blocks): a grid-stride loop over the
// probes rounded up to whole warps, so that every lane reaches the
// warp-cooperative lookup, with active = (i < m).  Inactive lanes search key
// 0 instead of reading probes[m] (the reference reads one element past the
// probe column there).
//   ref_bs_lookup:        binary_search_index's device lookup with its
//                         configured search functor,
//                         branchy_lower_bound_search_algorithm
//                         (src/indexes.cuh:328-361, src/search.cuh:26-53),
//                         invalid at n;
//   ref_btree_lookup:     btree_index's device lookup, btree::lookup
//                         (src/btree.cuh:504-531, clustered) from a device
//                         handle {column_begin, column_end, root} over pages
//                         in the reference's layout (ref_btree_layout below
//                         states it; the host writes the pages);
//   ref_harmonia_lookup:  harmonia_tree::lookup<4> (src/harmonia.cuh:740-786)
//                         on a device handle over the caller's Harmonia
//                         arrays (level-order keys, children prefix array,
//                         the column as the leaf level), as harmonia_index
//                         builds it (src/indexes.cuh:257-307).
#include <cstdint>
#include <memory>

#include "search.cuh"
#include "btree.cuh"
#include "harmonia.cuh"

namespace {
constexpr uint64_t kInvalid64 = ~0ull;
using harmonia_t = harmonia::harmonia_tree<uint64_t, uint64_t, std::allocator, 32 + 1, kInvalid64>;
using btree_t = index_structures::btree<uint64_t, uint64_t, std::allocator, kInvalid64>;
}  // namespace

// page size, header size, offset of the separators, offset of the child
// pointers, separators per inner node, keys per leaf -- read by the host
// that writes the pages, so that they follow this compilation's layout
extern "C" __device__ const uint64_t ref_btree_layout[6] = {
    btree_t::page_size,
    sizeof(btree_t::NodeBase),
    __builtin_offsetof(btree_t::InnerNode, keys),
    __builtin_offsetof(btree_t::InnerNode, children),
    btree_t::InnerNode::maxEntries,
    btree_t::LeafNode::maxEntries,
};

extern "C" __global__ void ref_btree_lookup(const uint64_t* column_begin, const uint64_t* column_end,
                                            const void* root, const uint64_t* probes, uint64_t m, uint32_t* out) {
    btree_t::device_handle_t h;
    h.column_begin = column_begin;
    h.column_end = column_end;
    h.root = static_cast<btree_t::NodeBase*>(const_cast<void*>(root));
    h.depth = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m; i += stride) {
        const uint64_t v = btree_t::lookup(h, probes[i]);
        out[i] = v == kInvalid64 ? 0xFFFFFFFFu : (uint32_t)v;
    }
}

extern "C" __global__ void ref_bs_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes, uint64_t m,
                                         uint32_t* out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t limit = (m + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < limit; i += stride) {
        if (i >= m) continue;
        const device_size_t pos = branchy_lower_bound_search_algorithm{}(probes[i], col, (device_size_t)n);
        out[i] = pos < n ? (uint32_t)pos : 0xFFFFFFFFu;
    }
}

extern "C" __global__ void ref_harmonia_lookup(const uint64_t* keys, const uint64_t* leaf_keys,
                                               const uint64_t* children, uint64_t size, uint64_t inner_size,
                                               uint32_t depth, const uint64_t* probes, uint64_t m, uint32_t* out) {
    harmonia_t::device_handle_t h;
    h.keys = keys;
    h.leaf_keys = leaf_keys;
    h.children = children;
    h.values = nullptr;
    h.size = size;
    h.inner_nodes_key_array_size = inner_size;
    h.depth = depth;
    h.caching_depth = 0;
    for (unsigned l = 0; l < harmonia_t::max_depth; ++l) h.ntg_degree[l] = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t limit = (m + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < limit; i += stride) {
        const bool active = i < m;
        const uint64_t key = active ? probes[i] : 0;
        const uint64_t v = harmonia_t::lookup<4>(active, h, key);
        if (active) out[i] = v == kInvalid64 ? 0xFFFFFFFFu : (uint32_t)v;
    }
}
