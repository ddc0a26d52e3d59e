// gj_index.cu -- C ABI: library state, index construction and the probe
// entry points.
//
// Index construction replaces abstract_index::construct and its overrides
// (src/indexes.cuh:36,126,218,285,364); every index borrows the caller's
// device column as the reference's binary_search_index / radix_spline_index
// do, and the B+tree and Harmonia use it as their leaf level.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "gj_internal.h"

namespace gj {

// ---------------------------------------------------------------------------
// errors and device properties
// ---------------------------------------------------------------------------
namespace {
thread_local std::string g_last_error;
}

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

const char* last_error() { return g_last_error.c_str(); }

int current_device_info(device_info* out) {
    static device_info cache[64];
    int dev = 0;
    GJ_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("device ordinal %d out of range", dev);
        return GJ_ERR_UNSUPPORTED;
    }
    if (cache[dev].device != dev) {
        device_info di;
        di.device = dev;
        GJ_CUDA_TRY(cudaDeviceGetAttribute(&di.sm_count, cudaDevAttrMultiProcessorCount, dev));
        int v = 0;
        GJ_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        di.smem_optin = (size_t)v;
        GJ_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, dev));
        di.l2_bytes = (size_t)v;
        cache[dev] = di;
    }
    *out = cache[dev];
    return GJ_OK;
}

namespace {

// ---------------------------------------------------------------------------
// build kernels
// ---------------------------------------------------------------------------
__global__ void k_count_unsorted(const uint64_t* __restrict__ col, uint64_t n, unsigned long long* bad) {
    unsigned long long local = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i + 1 < n; i += (uint64_t)gridDim.x * blockDim.x)
        local += (col[i] >= col[i + 1]);
    if (local) atomicAdd(bad, local);
}

// fence[j] = col[j << shift] for j < used, UINT64_MAX up to slots
__global__ void k_gather_fence(const uint64_t* __restrict__ col, uint64_t n, uint32_t shift, uint32_t slots,
                               uint64_t* __restrict__ fence) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < slots; j += gridDim.x * blockDim.x) {
        const uint64_t p = (uint64_t)j << shift;
        fence[j] = p < n ? col[p] : UINT64_MAX;
    }
}

// start table of a B+tree: entry b = the deepest node shared by the exact
// descents of every key of bucket b, [min + b * 2^shift, min + (b + 1) * 2^shift)
// clamped to max (v reads every level from global memory: no shared cache)
template <int W>
__global__ void k_btree_start(btree_view v, uint64_t entries, uint64_t* __restrict__ out) {
    for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; b < entries;
         b += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t lo = v.min_key + (b << v.start_shift);
        const uint64_t hi = b + 1 == entries ? v.max_key : lo + ((1ull << v.start_shift) - 1);
        const btree_cursor c = btree_common_node<W, false>(v, nullptr, lo, hi);
        out[2 * b] = c.base;
        out[2 * b + 1] = (uint64_t)c.node | ((uint64_t)(uint32_t)c.level << 32);
    }
}

// start table of a Harmonia tree: entry b = the deepest node shared by the
// descents of every key of bucket b (the bucket's first and last key)
__global__ void k_harmonia_start(harmonia_view v, uint64_t max_key, uint64_t entries, uint64_t* __restrict__ out) {
    for (uint64_t b = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; b < entries;
         b += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t lo = v.min_key + (b << v.start_shift);
        const uint64_t hi = b + 1 == entries ? max_key : lo + ((1ull << v.start_shift) - 1);
        out[b] = harmonia_common_node(v, lo, hi);
    }
}

// B+tree level l, W separators per node, fanout F = W + 1: slot k = (node j,
// separator c) is the max key of child j*F + c one level down, which covers
// the column range [child * span, (child + 1) * span); UINT64_MAX past the end
__global__ void k_gather_btree_level(const uint64_t* __restrict__ col, uint64_t n, uint64_t span, uint32_t W,
                                     uint64_t slots, uint64_t* __restrict__ level) {
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < slots; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t child = (k / W) * (W + 1) + (k % W);
        const uint64_t first = child * span;
        if (first < n) {
            uint64_t last = first + span;
            if (last > n) last = n;
            level[k] = col[last - 1];
        } else {
            level[k] = UINT64_MAX;
        }
    }
}

// Compressed level l (W = 7): node j's base from its parent's encoding (the
// rule the lookup applies), its shift from its subtree's largest key, and 7
// separator deltas (the last key of each child's subtree; 0xFFFFFFFF for a
// missing child).  span = column keys under one child of a level-l node.
__global__ void k_encode_btree_c7(const uint64_t* __restrict__ col, uint64_t n, uint64_t span, uint64_t nodes,
                                  const uint32_t* __restrict__ parent, const uint64_t* __restrict__ parent_base,
                                  uint64_t min_key, uint64_t* __restrict__ base_out, uint32_t* __restrict__ out) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < nodes; j += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t B = min_key;
        if (parent) {
            const uint64_t p = j >> 3, c = j & 7;
            B = parent_base[p];
            if (c) B += (uint64_t)parent[p * 8 + c] << (parent[p * 8] & 63u);
        }
        base_out[j] = B;
        const uint64_t end = (j + 1) * 8 * span < n ? (j + 1) * 8 * span : n;
        const uint64_t range = col[end - 1] - B;
        const unsigned bits = range ? 64u - (unsigned)__clzll(range) : 0u;
        const uint32_t sh = bits > 31 ? bits - 31 : 0;
        uint32_t* w = out + j * 8;
        w[0] = sh;
        for (uint32_t i = 0; i < 7; ++i) {
            const uint64_t first = (j * 8 + i) * span;
            if (first < n) {
                const uint64_t last = first + span < n ? first + span : n;
                w[i + 1] = (uint32_t)((col[last - 1] - B) >> sh);
            } else {
                w[i + 1] = kBtreeAbsent;
            }
        }
    }
}

// nodes of 16 lanes of 16 bits (node width 15): lane 0 = header | shift,
// lanes 1..15 = bias | separator (rounded down) relative to the node's base,
// the delta at most kBtreeMaxDelta16; kBtreeAbsent16 past the column's end
__global__ void k_encode_btree_c15(const uint64_t* __restrict__ col, uint64_t n, uint64_t span, uint64_t nodes,
                                   const uint16_t* __restrict__ parent, const uint64_t* __restrict__ parent_base,
                                   uint64_t min_key, uint64_t* __restrict__ base_out, uint16_t* __restrict__ out) {
    for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < nodes; j += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t B = min_key;
        if (parent) {
            const uint64_t p = j >> 4, c = j & 15;
            B = parent_base[p];
            if (c) B += (uint64_t)(parent[p * 16 + c] & 0x7FFFu) << (parent[p * 16] & 63u);
        }
        base_out[j] = B;
        const uint64_t end = (j + 1) * 16 * span < n ? (j + 1) * 16 * span : n;
        const uint64_t range = col[end - 1] - B;
        const unsigned bits = range ? 64u - (unsigned)__clzll(range) : 0u;
        uint32_t sh = bits > 14 ? bits - 14 : 0;
        if ((range >> sh) > kBtreeMaxDelta16) sh += 1;
        uint16_t* w = out + j * 16;
        w[0] = (uint16_t)(kBtreeHeader16 | sh);
        for (uint32_t i = 0; i < 15; ++i) {
            const uint64_t first = (j * 16 + i) * span;
            if (first < n) {
                const uint64_t last = first + span < n ? first + span : n;
                w[i + 1] = (uint16_t)(kBtreeLaneBias16 | ((col[last - 1] - B) >> sh));
            } else {
                w[i + 1] = (uint16_t)kBtreeAbsent16;
            }
        }
    }
}

// storage of the index's own arrays: HBM, or pinned host memory that the
// kernels read through its device mapping (the same address under unified
// addressing)
__global__ void k_hash_clear(hash_slot* slots, uint64_t capacity) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < capacity;
         i += (uint64_t)gridDim.x * blockDim.x)
        slots[i] = hash_slot{~0ull, kHashEmpty, 0u};
}

// insert (src/linear_probing_hashtable.cuh:36-46): claim the first free slot
// from the key's home bucket on; the keys are unique, so no slot is matched
__global__ void k_hash_insert(const uint64_t* __restrict__ col, uint64_t n, hash_slot* slots, uint64_t mask,
                              unsigned int* full) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t key = col[i];
        uint64_t b = murmur3_fmix64(key) & mask;
        bool placed = false;
        for (uint64_t step = 0; step <= mask && !placed; ++step) {
            for (uint64_t s = 2 * b; s < 2 * b + 2; ++s) {
                if (atomicCAS(&slots[s].pos, kHashEmpty, (uint32_t)i) == kHashEmpty) {
                    slots[s].key = key;
                    placed = true;
                    break;
                }
            }
            b = (b + 1) & mask;
        }
        if (!placed) atomicExch(full, 1u);
    }
}

int device_alloc(gj_index* idx, size_t bytes, void** out) {
    void* p = nullptr;
    if (idx->params.index_memory == GJ_INDEX_MEMORY_HOST) {
        const cudaError_t e = cudaHostAlloc(&p, bytes ? bytes : 16, cudaHostAllocMapped);
        if (e != cudaSuccess) {
            set_error("cudaHostAlloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? GJ_ERR_OUT_OF_MEMORY : GJ_ERR_CUDA;
        }
        idx->host_allocations.push_back(p);
        idx->host_bytes += bytes;
        *out = p;
        return GJ_OK;
    }
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        set_error("cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? GJ_ERR_OUT_OF_MEMORY : GJ_ERR_CUDA;
    }
    idx->allocations.push_back(p);
    *out = p;
    return GJ_OK;
}

uint32_t aligned32(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 31u) == 0 ? 1u : 0u; }

int host_copy_of_column(const uint64_t* d_keys, const uint64_t* h_keys, uint64_t n, std::vector<uint64_t>* store,
                        const uint64_t** out) {
    if (h_keys) {
        *out = h_keys;
        return GJ_OK;
    }
    store->resize(n);
    GJ_CUDA_TRY(cudaMemcpy(store->data(), d_keys, n * sizeof(uint64_t), cudaMemcpyDefault));
    *out = store->data();
    return GJ_OK;
}

int build_binary_search(gj_index* idx, cudaStream_t s) {
    idx->bs.col = idx->d_col;
    idx->bs.n = idx->n;
    idx->bs.col_aligned = aligned32(idx->d_col);
    const uint32_t want = idx->params.bs_cache_keys;
    if (want == 0 || idx->n < 64) return GJ_OK;
    // slots: a power of two <= want; stride 2^shift with slots * 2^shift >= n
    uint32_t slots = 1;
    while ((slots << 1) <= want && (slots << 1) != 0) slots <<= 1;
    uint32_t shift = 0;
    while (((uint64_t)slots << shift) < idx->n) ++shift;
    // do not sample finer than needed
    while (slots > 2 && ((uint64_t)(slots >> 1) << shift) >= idx->n) slots >>= 1;
    uint32_t steps = 0;
    while ((1u << steps) < slots) ++steps;
    void* p = nullptr;
    GJ_TRY(device_alloc(idx, (size_t)slots * sizeof(uint64_t), &p));
    k_gather_fence<<<(slots + 255) / 256, 256, 0, s>>>(idx->d_col, idx->n, shift, slots, static_cast<uint64_t*>(p));
    GJ_CUDA_TRY(cudaGetLastError());
    idx->bs.fence = static_cast<uint64_t*>(p);
    idx->bs.fence_slots = slots;
    idx->bs.fence_shift = shift;
    idx->bs.fence_steps = steps;
    idx->bytes = (uint64_t)slots * sizeof(uint64_t);
    return GJ_OK;
}

int build_btree(gj_index* idx, cudaStream_t s) {
    const uint32_t W = idx->params.btree_node_keys;
    const uint32_t L = idx->params.btree_leaf_keys ? idx->params.btree_leaf_keys : 4;
    if (!(W == 4 || W == kBtreeCompressed || W == 8 || W == kBtreeCompressed16 || W == 16 || W == 32 || W == 64) ||
        L == 0 || L > 4096 || (L & (L - 1)) != 0) {
        set_error("btree: node width %u / leaf width %u not supported (nodes of 4, 7 (compressed), 8, 15 "
                  "(compressed), 16, 32 or 64 separators, leaves of a power of two up to 4096 keys)", W, L);
        return GJ_ERR_INVALID_ARGUMENT;
    }
    const uint64_t n = idx->n;
    const bool compressed = W == kBtreeCompressed || W == kBtreeCompressed16;
    const uint32_t fan_log = W == kBtreeCompressed ? 3u : 4u;  // compressed nodes: log2 of the fanout
    const uint32_t words = compressed ? 4u : W;  // 64-bit words per node
    const uint64_t F = (uint64_t)W + 1;
    // level sizes: level l has ceil(nodes[l-1] / F) nodes; nodes[0] = leaves
    std::vector<uint64_t> nodes(1, (n + L - 1) / L);
    for (int l = 1;; ++l) {
        if (l >= kBtreeMaxLevels) {
            set_error("btree: more than %d levels", kBtreeMaxLevels - 1);
            return GJ_ERR_UNSUPPORTED;
        }
        const uint64_t cnt = (nodes[l - 1] + F - 1) / F;
        nodes.push_back(cnt);
        if (cnt == 1) break;
    }
    const uint32_t height = (uint32_t)nodes.size() - 1;
    // storage: top level first so that the shared-memory cache is a prefix
    std::vector<uint64_t> offset(height + 1, 0);
    uint64_t total = 0;
    for (uint32_t l = height; l >= 1; --l) {
        offset[l] = total;
        total += nodes[l] * words;
    }
    void* p = nullptr;
    GJ_TRY(device_alloc(idx, total * sizeof(uint64_t), &p));
    uint64_t* base = static_cast<uint64_t*>(p);
    uint64_t min_key = 0;
    GJ_CUDA_TRY(cudaMemcpyAsync(&min_key, idx->d_col, sizeof(uint64_t), cudaMemcpyDefault, s));
    if (compressed) {
        // top down: a node's base comes from its parent's encoding
        uint64_t* bases[2] = {nullptr, nullptr};
        cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&bases[0]), nodes[1] * sizeof(uint64_t));
        if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&bases[1]), nodes[1] * sizeof(uint64_t));
        if (e != cudaSuccess) {
            cudaFree(bases[0]);
            set_error("btree: scratch allocation failed: %s", cudaGetErrorString(e));
            return GJ_ERR_OUT_OF_MEMORY;
        }
        GJ_CUDA_TRY(cudaStreamSynchronize(s));  // min_key
        int rc = GJ_OK;
        for (uint32_t l = height; l >= 1 && rc == GJ_OK; --l) {
            const uint64_t span = (uint64_t)L << (fan_log * (l - 1));
            const int grid = (int)std::min<uint64_t>((nodes[l] + 255) / 256, 65535);
            const uint64_t* parent = l == height ? nullptr : base + offset[l + 1];
            if (W == kBtreeCompressed)
                k_encode_btree_c7<<<grid, 256, 0, s>>>(idx->d_col, n, span, nodes[l],
                                                       reinterpret_cast<const uint32_t*>(parent), bases[(l + 1) & 1],
                                                       min_key, bases[l & 1],
                                                       reinterpret_cast<uint32_t*>(base + offset[l]));
            else
                k_encode_btree_c15<<<grid, 256, 0, s>>>(idx->d_col, n, span, nodes[l],
                                                        reinterpret_cast<const uint16_t*>(parent), bases[(l + 1) & 1],
                                                        min_key, bases[l & 1],
                                                        reinterpret_cast<uint16_t*>(base + offset[l]));
            if (cudaGetLastError() != cudaSuccess) {
                set_error("btree: encoding kernel failed to launch");
                rc = GJ_ERR_CUDA;
            }
            idx->bt.level[l] = base + offset[l];
        }
        const cudaError_t se = cudaStreamSynchronize(s);
        cudaFree(bases[0]);
        cudaFree(bases[1]);
        GJ_TRY(rc);
        if (se != cudaSuccess) {
            set_error("btree: encoding failed: %s", cudaGetErrorString(se));
            return GJ_ERR_CUDA;
        }
    } else {
        uint64_t span = L;  // column keys below one child of a level-1 node
        for (uint32_t l = 1; l <= height; ++l) {
            const uint64_t slots = nodes[l] * W;
            const int grid = (int)std::min<uint64_t>((slots + 255) / 256, 65535);
            k_gather_btree_level<<<grid, 256, 0, s>>>(idx->d_col, n, span, W, slots, base + offset[l]);
            GJ_CUDA_TRY(cudaGetLastError());
            idx->bt.level[l] = base + offset[l];
            span *= F;
        }
    }
    // shared-memory cache: as many top levels as fit the budget
    uint32_t cached = 0;
    uint64_t cache_keys = 0;
    for (uint32_t l = height; l >= 1; --l) {
        const uint64_t add = nodes[l] * words;
        if ((cache_keys + add) * sizeof(uint64_t) > idx->params.smem_cache_bytes) break;
        cache_keys += add;
        cached += 1;
        idx->bt.smem_offset[l] = (uint32_t)offset[l];
    }
    idx->bt.col = idx->d_col;
    idx->bt.n = n;
    idx->bt.height = height;
    idx->bt.cached_levels = cached;
    idx->bt.cache_keys = (uint32_t)cache_keys;
    idx->bt.node_keys = W;
    idx->bt.leaf_keys = L;
    idx->bt.col_aligned = aligned32(idx->d_col);
    uint64_t maxk = 0;
    GJ_CUDA_TRY(cudaMemcpyAsync(&maxk, idx->d_col + n - 1, sizeof(uint64_t), cudaMemcpyDefault, s));
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    idx->bt.max_key = maxk;
    idx->bt.min_key = min_key;
    idx->bytes = total * sizeof(uint64_t);

    // start table: by default about one bucket per 64 keys (2^1 .. 2^20
    // buckets, at most 16 MB), so that most buckets lie inside one node two
    // levels above the leaves; finer tables (measured at 2^21 - 2^23 buckets
    // for 2^26 keys) fall out of L2 and make every start a DRAM access
    uint32_t R = idx->params.btree_start_bits;
    if (R > 24) {
        set_error("btree: start table bits must be at most 24");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    if (R == 0) {
        R = 1;
        while (R < 20 && (n >> (R + 7)) != 0) ++R;
    }
    const uint64_t range = maxk - min_key;
    const uint32_t used = range ? 64u - (uint32_t)__builtin_clzll(range) : 0u;
    const uint32_t shift = used > R ? used - R : 0u;
    const uint64_t entries = (range >> shift) + 1;
    void* tp = nullptr;
    GJ_TRY(device_alloc(idx, entries * 16, &tp));
    btree_view tv = idx->bt;
    tv.cached_levels = 0;
    tv.start_shift = shift;
    const int grid = (int)std::min<uint64_t>((entries + 255) / 256, 4096);
    uint64_t* table = static_cast<uint64_t*>(tp);
    switch (W) {
        case 4: k_btree_start<4><<<grid, 256, 0, s>>>(tv, entries, table); break;
        case kBtreeCompressed: k_btree_start<kBtreeCompressed><<<grid, 256, 0, s>>>(tv, entries, table); break;
        case 8: k_btree_start<8><<<grid, 256, 0, s>>>(tv, entries, table); break;
        case kBtreeCompressed16: k_btree_start<kBtreeCompressed16><<<grid, 256, 0, s>>>(tv, entries, table); break;
        case 16: k_btree_start<16><<<grid, 256, 0, s>>>(tv, entries, table); break;
        case 32: k_btree_start<32><<<grid, 256, 0, s>>>(tv, entries, table); break;
        default: k_btree_start<64><<<grid, 256, 0, s>>>(tv, entries, table); break;
    }
    GJ_CUDA_TRY(cudaGetLastError());
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    idx->bt.start = table;
    idx->bt.start_shift = shift;
    idx->bt.start_entries = (uint32_t)entries;
    idx->bytes += entries * 16;
    return GJ_OK;
}

int build_harmonia(gj_index* idx, const uint64_t* h_keys, cudaStream_t s) {
    if (idx->n % kHarmoniaKeys != 0) {
        set_error("harmonia: when Reuse_Input_Memory is set the dataset set must be a multiple of the node size "
                  "(n = %llu, node size %d)", (unsigned long long)idx->n, kHarmoniaKeys);
        return GJ_ERR_INVALID_ARGUMENT;
    }
    std::vector<uint64_t> store;
    const uint64_t* col = nullptr;
    GJ_TRY(host_copy_of_column(idx->d_col, h_keys, idx->n, &store, &col));
    harmonia_arrays ha;
    GJ_TRY(build_harmonia_arrays(col, idx->n, &ha));
    void *pk = nullptr, *pc = nullptr;
    GJ_TRY(device_alloc(idx, ha.keys.size() * sizeof(uint64_t), &pk));
    GJ_TRY(device_alloc(idx, ha.children.size() * sizeof(uint64_t), &pc));
    if (!ha.keys.empty())
        GJ_CUDA_TRY(cudaMemcpyAsync(pk, ha.keys.data(), ha.keys.size() * sizeof(uint64_t), cudaMemcpyDefault, s));
    GJ_CUDA_TRY(cudaMemcpyAsync(pc, ha.children.data(), ha.children.size() * sizeof(uint64_t), cudaMemcpyDefault, s));
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    idx->hm.keys = static_cast<uint64_t*>(pk);
    idx->hm.children = static_cast<uint64_t*>(pc);
    idx->hm.col = idx->d_col;
    idx->hm.n = idx->n;
    idx->hm.inner_size = ha.keys.size();
    idx->hm.depth = ha.depth;
    // shared-memory cache: whole top levels (keys + children) within the budget
    const uint64_t per_node = (kHarmoniaKeys + 1) * sizeof(uint64_t);
    uint64_t cached = 0;
    uint32_t cached_levels = 0;
    for (uint32_t l = 0; l + 1 < ha.depth; ++l) {
        if ((cached + ha.level_nodes[l]) * per_node > idx->params.smem_cache_bytes) break;
        cached += ha.level_nodes[l];
        cached_levels += 1;
    }
    idx->hm.cached_nodes = (uint32_t)cached;
    idx->hm.cached_levels = cached_levels;
    idx->hm.col_aligned = aligned32(idx->d_col);
    idx->bytes = (ha.keys.size() + ha.children.size()) * sizeof(uint64_t);

    // start table, as for the B+tree (one bucket per about 64 keys, 2^1 ..
    // 2^20 buckets, btree_start_bits to override): most buckets then lie
    // inside one node above the leaves, or one leaf node, and a lookup
    // starts there instead of at the root
    const uint64_t n = idx->n;
    uint32_t R = idx->params.btree_start_bits;
    if (R > 24) {
        set_error("harmonia: start table bits must be at most 24");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    if (R == 0) {
        R = 1;
        while (R < 20 && (n >> (R + 7)) != 0) ++R;
    }
    const uint64_t min_key = col[0], max_key = col[n - 1];
    const uint64_t range = max_key - min_key;
    const uint32_t used = range ? 64u - (uint32_t)__builtin_clzll(range) : 0u;
    const uint32_t shift = used > R ? used - R : 0u;
    const uint64_t entries = (range >> shift) + 1;
    void* tp = nullptr;
    GJ_TRY(device_alloc(idx, entries * sizeof(uint64_t), &tp));
    harmonia_view tv = idx->hm;
    tv.cached_nodes = 0;
    tv.cached_levels = 0;
    tv.min_key = min_key;
    tv.start = nullptr;
    tv.start_shift = shift;
    const int grid = (int)std::min<uint64_t>((entries + 255) / 256, 4096);
    k_harmonia_start<<<grid, 256, 0, s>>>(tv, max_key, entries, static_cast<uint64_t*>(tp));
    GJ_CUDA_TRY(cudaGetLastError());
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    idx->hm.min_key = min_key;
    idx->hm.start = static_cast<const uint64_t*>(tp);
    idx->hm.start_shift = shift;
    idx->hm.start_entries = (uint32_t)entries;
    idx->bytes += entries * sizeof(uint64_t);
    return GJ_OK;
}

int build_radix_spline_index(gj_index* idx, const uint64_t* h_keys, cudaStream_t s) {
    std::vector<uint64_t> store;
    const uint64_t* col = nullptr;
    GJ_TRY(host_copy_of_column(idx->d_col, h_keys, idx->n, &store, &col));
    radix_spline_arrays rs;
    GJ_TRY(build_radix_spline(col, idx->n, idx->params.rs_radix_bits, idx->params.rs_max_error, &rs));
    // points with the slope of their segment (the estimate's division, done once)
    std::vector<rs_point> pts(rs.sx.size());
    for (size_t i = 0; i < pts.size(); ++i) {
        pts[i].x = rs.sx[i];
        pts[i].y = rs.sy[i];
        pts[i].slope = i + 1 < pts.size() ? (rs.sy[i + 1] - rs.sy[i]) / (double)(rs.sx[i + 1] - rs.sx[i]) : 0.0;
        pts[i].pad = 0;
    }
    void *pt = nullptr, *pp = nullptr;
    GJ_TRY(device_alloc(idx, rs.table.size() * sizeof(uint32_t), &pt));
    GJ_TRY(device_alloc(idx, pts.size() * sizeof(rs_point), &pp));
    GJ_CUDA_TRY(cudaMemcpyAsync(pt, rs.table.data(), rs.table.size() * sizeof(uint32_t), cudaMemcpyDefault, s));
    GJ_CUDA_TRY(cudaMemcpyAsync(pp, pts.data(), pts.size() * sizeof(rs_point), cudaMemcpyDefault, s));
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    idx->rs.col = idx->d_col;
    idx->rs.n = idx->n;
    idx->rs.table = static_cast<uint32_t*>(pt);
    idx->rs.pts = static_cast<const rs_point*>(pp);
    idx->rs.min_key = rs.min_key;
    idx->rs.max_key = rs.max_key;
    idx->rs.shift = rs.shift;
    idx->rs.max_error = idx->params.rs_max_error;
    idx->rs.col_aligned = aligned32(idx->d_col);
    idx->bytes = rs.table.size() * sizeof(uint32_t) + pts.size() * sizeof(rs_point);
    return GJ_OK;
}

// hash table over the column; built in HBM and copied when the index lives in
// host memory (atomics stay on the device)
int build_hash(gj_index* idx, cudaStream_t s) {
    const uint64_t n = idx->n;
    uint64_t capacity = 2;
    while (capacity < 2 * n) capacity <<= 1;
    const size_t bytes = capacity * sizeof(hash_slot);
    void* p = nullptr;
    GJ_TRY(device_alloc(idx, bytes, &p));
    const bool host = idx->params.index_memory == GJ_INDEX_MEMORY_HOST;
    hash_slot* table = static_cast<hash_slot*>(p);
    unsigned int* full = nullptr;
    if (host) {
        const cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&table), bytes);
        if (e != cudaSuccess) {
            set_error("hash: scratch table of %zu bytes: %s", bytes, cudaGetErrorString(e));
            return GJ_ERR_OUT_OF_MEMORY;
        }
    }
    int rc = GJ_OK;
    if (cudaMalloc(reinterpret_cast<void**>(&full), sizeof(unsigned int)) != cudaSuccess) {
        set_error("hash: flag allocation failed");
        rc = GJ_ERR_OUT_OF_MEMORY;
    }
    unsigned int h_full = 0;
    if (rc == GJ_OK) {
        cudaMemsetAsync(full, 0, sizeof(unsigned int), s);
        k_hash_clear<<<(int)std::min<uint64_t>((capacity + 255) / 256, 65535), 256, 0, s>>>(table, capacity);
        k_hash_insert<<<(int)std::min<uint64_t>((n + 255) / 256, 65535), 256, 0, s>>>(idx->d_col, n, table,
                                                                                      capacity / 2 - 1, full);
        if (host) cudaMemcpyAsync(p, table, bytes, cudaMemcpyDefault, s);
        cudaMemcpyAsync(&h_full, full, sizeof(h_full), cudaMemcpyDeviceToHost, s);
        const cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("hash: build failed: %s", cudaGetErrorString(e));
            rc = GJ_ERR_CUDA;
        } else if (h_full) {
            set_error("hash: table full");
            rc = GJ_ERR_CUDA;
        }
    }
    cudaFree(full);
    if (host) cudaFree(table);
    GJ_TRY(rc);
    idx->hs.slots = static_cast<const hash_slot*>(p);
    idx->hs.mask = capacity / 2 - 1;
    idx->hs.n = n;
    idx->bytes = bytes;
    return GJ_OK;
}

}  // namespace

int build_learned(gj_index* idx, cudaStream_t s);  // gj_learned.cu

// owned allocation of an index (released by gj_index_free)
int device_alloc_for(gj_index* idx, size_t bytes, void** out) { return device_alloc(idx, bytes, out); }
uint32_t column_aligned32(const void* p) { return aligned32(p); }

}  // namespace gj

using namespace gj;

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

uint32_t gj_abi_version(void) { return GJ_ABI_VERSION; }

const char* gj_last_error_string(void) { return gj::last_error(); }

void gj_index_params_default(gj_index_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->struct_size = sizeof(gj_index_params);
    p->btree_node_keys = kBtreeCompressed16;
    p->btree_leaf_keys = 4;
    p->rs_radix_bits = 18;
    p->rs_max_error = 32;
    p->bs_cache_keys = 4096;
    p->smem_cache_bytes = 16384;
    p->learned_leaves = 0;  // about 128 keys per leaf, 2^10 .. 2^20
    p->learned_root = GJ_LEARNED_ROOT_AUTO;
    p->learned_hidden = 32;
    p->learned_steps = 600;
    p->learned_batch = 8192;
    p->learned_lr = 1e-3f;
    p->seed = 0x5eedULL;
}

int gj_parse_index_type(const char* name, int* out_type) {
    GJ_CHECK_ARG(name && out_type, "gj_parse_index_type: null argument");
    static const struct {
        const char* name;
        int type;
    } table[] = {{"btree", GJ_INDEX_BTREE},
                 {"harmonia", GJ_INDEX_HARMONIA},
                 {"binary_search", GJ_INDEX_BINARY_SEARCH},
                 {"radix_spline", GJ_INDEX_RADIX_SPLINE},
                 {"no_op", GJ_INDEX_NO_OP},
                 {"learned", GJ_INDEX_LEARNED},
                 {"hash", GJ_INDEX_HASH}};
    for (const auto& e : table) {
        if (std::strcmp(name, e.name) == 0) {
            *out_type = e.type;
            return GJ_OK;
        }
    }
    set_error("unknown index type");
    return GJ_ERR_INVALID_ARGUMENT;
}

const char* gj_index_type_name(int type) {
    switch (type) {
        case GJ_INDEX_BTREE: return "btree";
        case GJ_INDEX_HARMONIA: return "harmonia";
        case GJ_INDEX_BINARY_SEARCH: return "binary_search";
        case GJ_INDEX_RADIX_SPLINE: return "radix_spline";
        case GJ_INDEX_NO_OP: return "no_op";
        case GJ_INDEX_LEARNED: return "learned";
        case GJ_INDEX_HASH: return "hash";
        default: return nullptr;
    }
}

int gj_index_build(int type, const uint64_t* d_keys, const uint64_t* h_keys, uint64_t n,
                   const gj_index_params* params, void* stream, gj_index** out_index) {
    GJ_CHECK_ARG(out_index, "gj_index_build: out_index is null");
    *out_index = nullptr;
    GJ_CHECK_ARG(gj_index_type_name(type) != nullptr, "gj_index_build: unknown index type");
    GJ_CHECK_ARG(d_keys || type == GJ_INDEX_NO_OP, "gj_index_build: d_keys is null");
    if (type != GJ_INDEX_NO_OP && n == 0) {
        set_error("gj_index_build: empty column");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    if (n >= (uint64_t)GJ_INVALID_POS) {
        set_error("'value_t' does not suffice: %llu keys do not fit 32-bit positions", (unsigned long long)n);
        return GJ_ERR_TOO_LARGE;
    }
    gj_index_params p;
    gj_index_params_default(&p);
    if (params) {
        GJ_CHECK_ARG(params->struct_size == sizeof(gj_index_params), "gj_index_build: params.struct_size mismatch");
        p = *params;
    }
    GJ_CHECK_ARG(p.index_memory == GJ_INDEX_MEMORY_DEVICE || p.index_memory == GJ_INDEX_MEMORY_HOST,
                 "gj_index_build: index_memory must be GJ_INDEX_MEMORY_DEVICE or GJ_INDEX_MEMORY_HOST");
    cudaStream_t s = as_stream(stream);
    if (type == GJ_INDEX_LEARNED && p.learned_root == GJ_LEARNED_ROOT_AUTO) {
        // the roots in order of lookup cost -- linear, the segment table (one
        // L1 load more), a 16-wide MLP, a 32-wide MLP -- on the same column;
        // the cheapest whose mean search window is at most twice the
        // narrowest + 16 keys is kept (a window of w keys costs about
        // log2(w / 4) sector loads, a 32-wide root about a thousand
        // instructions, a 16-wide one a quarter of that)
        constexpr int kCand = 4;
        const uint32_t roots[kCand] = {GJ_LEARNED_ROOT_LINEAR, GJ_LEARNED_ROOT_SEGMENTS, GJ_LEARNED_ROOT_MLP,
                                       GJ_LEARNED_ROOT_MLP};
        const uint32_t widths[kCand] = {0, 0, 16, 32};
        gj_index* cand[kCand] = {nullptr, nullptr, nullptr, nullptr};
        for (int i = 0; i < kCand; ++i) {
            gj_index_params pc = p;
            pc.learned_root = roots[i];
            if (widths[i]) pc.learned_hidden = widths[i];
            const int rc = gj_index_build(type, d_keys, h_keys, n, &pc, stream, &cand[i]);
            if (rc != GJ_OK) {
                for (gj_index* c : cand) gj_index_free(c);
                return rc;
            }
        }
        double best = cand[0]->learned_mean_window;
        for (gj_index* c : cand) best = c->learned_mean_window < best ? c->learned_mean_window : best;
        int keep = kCand - 1;
        for (int i = 0; i < kCand; ++i) {
            if (cand[i]->learned_mean_window <= 2.0 * best + 16.0) {
                keep = i;
                break;
            }
        }
        for (int i = 0; i < kCand; ++i)
            if (i != keep) gj_index_free(cand[i]);
        *out_index = cand[keep];
        return GJ_OK;
    }
    std::unique_ptr<gj_index> idx(new gj_index());
    idx->type = type;
    idx->n = n;
    idx->d_col = d_keys;
    idx->params = p;
    GJ_CUDA_TRY(cudaGetDevice(&idx->device));

    if (type != GJ_INDEX_NO_OP && n > 1) {
        unsigned long long* d_bad = nullptr;
        GJ_CUDA_TRY(cudaMallocAsync(&d_bad, sizeof(unsigned long long), s));
        cudaMemsetAsync(d_bad, 0, sizeof(unsigned long long), s);
        const int grid = (int)std::min<uint64_t>((n + 255) / 256, 4096);
        k_count_unsorted<<<grid, 256, 0, s>>>(d_keys, n, d_bad);
        unsigned long long bad = 0;
        cudaMemcpyAsync(&bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(d_bad, s);
        GJ_CUDA_TRY(cudaStreamSynchronize(s));
        if (bad) {
            set_error("build keys are not strictly increasing (%llu violations)", bad);
            return GJ_ERR_UNSORTED;
        }
    }
    if (n > 0 && d_keys) {
        // key range, kept on the host (partition functions need it per call)
        GJ_CUDA_TRY(cudaMemcpyAsync(&idx->min_key, d_keys, sizeof(uint64_t), cudaMemcpyDefault, s));
        GJ_CUDA_TRY(cudaMemcpyAsync(&idx->max_key, d_keys + n - 1, sizeof(uint64_t), cudaMemcpyDefault, s));
        GJ_CUDA_TRY(cudaStreamSynchronize(s));
    }

    int rc = GJ_OK;
    switch (type) {
        case GJ_INDEX_BINARY_SEARCH: rc = build_binary_search(idx.get(), s); break;
        case GJ_INDEX_BTREE: rc = build_btree(idx.get(), s); break;
        case GJ_INDEX_HARMONIA: rc = build_harmonia(idx.get(), h_keys, s); break;
        case GJ_INDEX_RADIX_SPLINE: rc = build_radix_spline_index(idx.get(), h_keys, s); break;
        case GJ_INDEX_LEARNED: rc = build_learned(idx.get(), s); break;
        case GJ_INDEX_HASH: rc = build_hash(idx.get(), s); break;
        case GJ_INDEX_NO_OP: break;
    }
    if (rc == GJ_OK) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) {
            set_error("index build: %s", cudaGetErrorString(e));
            rc = GJ_ERR_CUDA;
        }
    }
    if (rc != GJ_OK) {
        for (void* a : idx->allocations) cudaFree(a);
        for (void* a : idx->host_allocations) cudaFreeHost(a);
        return rc;
    }
    *out_index = idx.release();
    return GJ_OK;
}

int gj_index_free(gj_index* index) {
    if (!index) return GJ_OK;
    int prev = -1;
    cudaGetDevice(&prev);
    if (prev != index->device) cudaSetDevice(index->device);
    int rc = GJ_OK;
    for (void* a : index->allocations) {
        cudaError_t e = cudaFree(a);
        if (e != cudaSuccess && rc == GJ_OK) {
            set_error("cudaFree: %s", cudaGetErrorString(e));
            rc = GJ_ERR_CUDA;
        }
    }
    for (void* a : index->host_allocations) {
        cudaError_t e = cudaFreeHost(a);
        if (e != cudaSuccess && rc == GJ_OK) {
            set_error("cudaFreeHost: %s", cudaGetErrorString(e));
            rc = GJ_ERR_CUDA;
        }
    }
    if (prev != index->device && prev >= 0) cudaSetDevice(prev);
    delete index;
    return rc;
}

uint64_t gj_index_memory_consumption(const gj_index* index) { return index ? index->bytes : 0; }

uint64_t gj_index_host_memory(const gj_index* index) { return index ? index->host_bytes : 0; }

int gj_index_get_type(const gj_index* index, int* out_type) {
    GJ_CHECK_ARG(index && out_type, "gj_index_get_type: null argument");
    *out_type = index->type;
    return GJ_OK;
}

uint64_t gj_index_size(const gj_index* index) { return index ? index->n : 0; }

int gj_index_learned_stats(const gj_index* index, uint64_t* max_error, double* mean_window) {
    GJ_CHECK_ARG(index, "gj_index_learned_stats: null index");
    if (index->type != GJ_INDEX_LEARNED) {
        set_error("gj_index_learned_stats: not a learned index");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    if (max_error) *max_error = index->learned_max_error;
    if (mean_window) *mean_window = index->learned_mean_window;
    return GJ_OK;
}

int gj_index_learned_root(const gj_index* index, uint32_t* root) {
    GJ_CHECK_ARG(index && root, "gj_index_learned_root: null argument");
    if (index->type != GJ_INDEX_LEARNED) {
        set_error("gj_index_learned_root: not a learned index");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    *root = index->params.learned_root;
    return GJ_OK;
}

int gj_index_learned_losses(const gj_index* index, double* init_loss, double* trained_loss) {
    GJ_CHECK_ARG(index && init_loss && trained_loss, "gj_index_learned_losses: null argument");
    if (index->type != GJ_INDEX_LEARNED || index->params.learned_root != GJ_LEARNED_ROOT_MLP) {
        set_error("gj_index_learned_losses: not a learned index with an MLP root");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    *init_loss = index->learned_init_loss;
    *trained_loss = index->learned_trained_loss;
    return GJ_OK;
}

int gj_index_device_view(const gj_index* index, void* view, size_t view_bytes) {
    GJ_CHECK_ARG(index, "gj_index_device_view: null index");
    auto copy = [&](const void* src, size_t bytes) -> int {
        if (view_bytes != bytes || (bytes && !view)) {
            set_error("gj_index_device_view: view_bytes %zu does not match the %zu-byte view of this index kind",
                      view_bytes, bytes);
            return GJ_ERR_INVALID_ARGUMENT;
        }
        if (bytes) std::memcpy(view, src, bytes);
        return GJ_OK;
    };
    switch (index->type) {
        case GJ_INDEX_BINARY_SEARCH: return copy(&index->bs, sizeof(index->bs));  // its fence lives in global memory
        case GJ_INDEX_BTREE: {
            gj::btree_view v = index->bt;
            v.cached_levels = 0;
            return copy(&v, sizeof(v));
        }
        case GJ_INDEX_HARMONIA: {
            gj::harmonia_view v = index->hm;
            v.cached_nodes = 0;
            v.cached_levels = 0;
            return copy(&v, sizeof(v));
        }
        case GJ_INDEX_RADIX_SPLINE: return copy(&index->rs, sizeof(index->rs));
        case GJ_INDEX_LEARNED: return copy(&index->ln, sizeof(index->ln));
        case GJ_INDEX_HASH: return copy(&index->hs, sizeof(index->hs));
        default: return copy(nullptr, 0);
    }
}

int gj_index_lookup(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_positions,
                    void* stream) {
    GJ_CHECK_ARG(index, "gj_index_lookup: null index");
    GJ_CHECK_ARG(m == 0 || (d_probes && d_positions), "gj_index_lookup: null buffer");
    return launch_lookup(index, d_probes, m, d_positions, as_stream(stream));
}

int gj_inlj_pairs_workspace_size(uint64_t m, size_t* bytes) {
    GJ_CHECK_ARG(bytes, "gj_inlj_pairs_workspace_size: null argument");
    *bytes = pairs_workspace_bytes(m);
    return GJ_OK;
}

int gj_inlj_pairs(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs, uint64_t* d_count,
                  void* d_workspace, size_t workspace_bytes, void* stream) {
    GJ_CHECK_ARG(index && d_count, "gj_inlj_pairs: null argument");
    GJ_CHECK_ARG(m == 0 || (d_probes && d_pairs), "gj_inlj_pairs: null buffer");
    if (m > (uint64_t)UINT32_MAX) {
        set_error("gj_inlj_pairs: probe rows must fit 32 bits");
        return GJ_ERR_TOO_LARGE;
    }
    // positions are parked in the upper half of the pairs buffer (2m u32)
    return launch_pairs(index, d_probes, m, nullptr, d_pairs, nullptr, d_count, d_workspace, workspace_bytes,
                        d_pairs ? d_pairs + m : nullptr, as_stream(stream));
}

int gj_inlj_pairs_unordered(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                            uint64_t* d_count, void* d_workspace, size_t workspace_bytes, void* stream) {
    GJ_CHECK_ARG(index && d_count, "gj_inlj_pairs_unordered: null argument");
    GJ_CHECK_ARG(m == 0 || (d_probes && d_pairs), "gj_inlj_pairs_unordered: null buffer");
    if (m > (uint64_t)UINT32_MAX) {
        set_error("gj_inlj_pairs_unordered: probe rows must fit 32 bits");
        return GJ_ERR_TOO_LARGE;
    }
    return launch_pairs_unordered(index, d_probes, m, d_pairs, d_count, d_workspace, workspace_bytes,
                                  as_stream(stream));
}

int gj_debug_inlj_pairs_stalled(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                                uint64_t* d_count, void* d_workspace, size_t workspace_bytes, uint32_t spin_limit,
                                void* stream) {
    GJ_CHECK_ARG(index && d_count && d_probes && d_pairs, "gj_debug_inlj_pairs_stalled: null argument");
    GJ_CHECK_ARG(m > 0 && m <= (uint64_t)UINT32_MAX, "gj_debug_inlj_pairs_stalled: m not in [1, 2^32)");
    GJ_CHECK_ARG(spin_limit > 0, "gj_debug_inlj_pairs_stalled: spin_limit must be > 0");
    return launch_pairs_stalled(index, d_probes, m, d_pairs, d_count, d_workspace, workspace_bytes, spin_limit,
                                as_stream(stream));
}

int gj_index_lookup_sorted(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_positions,
                           void* stream) {
    GJ_CHECK_ARG(index, "gj_index_lookup_sorted: null index");
    GJ_CHECK_ARG(m == 0 || (d_probes && d_positions), "gj_index_lookup_sorted: null buffer");
    return launch_sorted_lookup(index, d_probes, m, d_positions, as_stream(stream));
}

int gj_inlj_pairs_sorted(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                         uint64_t* d_count, void* d_workspace, size_t workspace_bytes, void* stream) {
    GJ_CHECK_ARG(index && d_count, "gj_inlj_pairs_sorted: null argument");
    GJ_CHECK_ARG(m == 0 || (d_probes && d_pairs), "gj_inlj_pairs_sorted: null buffer");
    if (m > (uint64_t)UINT32_MAX) {
        set_error("gj_inlj_pairs_sorted: probe rows must fit 32 bits");
        return GJ_ERR_TOO_LARGE;
    }
    return launch_partitioned_pairs(index, d_probes, nullptr, m, d_pairs, nullptr, d_count, d_workspace,
                                    workspace_bytes, as_stream(stream));
}

// device address of a caller buffer the GPU may touch: pinned or registered
// host memory (through NVLink-C2C / PCIe), managed or device memory, or
// pageable host memory on systems where the GPU reads the CPU's page tables
static int device_address(const void* p, const char* what, void** out) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        set_error("%s: not a pointer the CUDA runtime knows", what);
        return GJ_ERR_INVALID_ARGUMENT;
    }
    if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) {
        if (!a.devicePointer) {
            set_error("%s: host allocation is not mapped into the device address space", what);
            return GJ_ERR_INVALID_ARGUMENT;
        }
        *out = a.devicePointer;
        return GJ_OK;
    }
    int dev = 0, pageable = 0;
    GJ_CUDA_TRY(cudaGetDevice(&dev));
    GJ_CUDA_TRY(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev));
    if (!pageable) {
        set_error("%s: pageable host memory; pin it (cudaHostAlloc / cudaHostRegister)", what);
        return GJ_ERR_INVALID_ARGUMENT;
    }
    *out = const_cast<void*>(p);
    return GJ_OK;
}

int gj_inlj_pairs_host_workspace_size(uint64_t m, size_t* bytes) {
    GJ_CHECK_ARG(bytes, "gj_inlj_pairs_host_workspace_size: null argument");
    *bytes = pairs_workspace_bytes(m);
    return GJ_OK;
}

// gj_inlj_pairs_host and gj_inlj_pairs_host_unordered (name: the entry
// point, for the error messages)
static int host_pairs(const char* name, bool ordered, const gj_index* index, const uint64_t* h_probes, uint64_t m,
                      uint32_t* h_pairs, uint64_t* h_count, void* d_workspace, size_t workspace_bytes, void* stream) {
    if (!index || !h_count) {
        set_error("%s: null argument", name);
        return GJ_ERR_INVALID_ARGUMENT;
    }
    if (m != 0 && (!h_probes || !h_pairs)) {
        set_error("%s: null buffer", name);
        return GJ_ERR_INVALID_ARGUMENT;
    }
    if (m > (uint64_t)UINT32_MAX) {
        set_error("%s: probe rows must fit 32 bits", name);
        return GJ_ERR_TOO_LARGE;
    }
    const std::string what = name;
    void *probes = nullptr, *pairs = nullptr, *count = nullptr;
    GJ_TRY(device_address(h_count, (what + ": count").c_str(), &count));
    if (m == 0) {
        // nothing to launch: the count is written once earlier work on the stream is done
        GJ_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
        *h_count = 0;
        return GJ_OK;
    }
    GJ_TRY(device_address(h_probes, (what + ": probes").c_str(), &probes));
    GJ_TRY(device_address(h_pairs, (what + ": pairs").c_str(), &pairs));
    // One pass: each tile reads its probes from host memory, searches them
    // and writes its pairs back, so host-link reads, searches and writes of
    // different tiles overlap (a separate compaction pass would serialise
    // the writes behind the searches).
    if (!ordered)
        return launch_pairs_unordered(index, static_cast<const uint64_t*>(probes), m, static_cast<uint32_t*>(pairs),
                                      static_cast<uint64_t*>(count), d_workspace, workspace_bytes, as_stream(stream));
    return launch_pairs(index, static_cast<const uint64_t*>(probes), m, nullptr, static_cast<uint32_t*>(pairs),
                        nullptr, static_cast<uint64_t*>(count), d_workspace, workspace_bytes, nullptr,
                        as_stream(stream));
}

int gj_inlj_pairs_host(const gj_index* index, const uint64_t* h_probes, uint64_t m, uint32_t* h_pairs,
                       uint64_t* h_count, void* d_workspace, size_t workspace_bytes, void* stream) {
    return host_pairs("gj_inlj_pairs_host", true, index, h_probes, m, h_pairs, h_count, d_workspace, workspace_bytes,
                      stream);
}

int gj_inlj_pairs_host_unordered(const gj_index* index, const uint64_t* h_probes, uint64_t m, uint32_t* h_pairs,
                                 uint64_t* h_count, void* d_workspace, size_t workspace_bytes, void* stream) {
    return host_pairs("gj_inlj_pairs_host_unordered", false, index, h_probes, m, h_pairs, h_count, d_workspace,
                      workspace_bytes, stream);
}

int gj_inlj_pairs_status(const void* d_workspace, size_t workspace_bytes, uint64_t m, void* stream) {
    GJ_CHECK_ARG(d_workspace, "gj_inlj_pairs_status: null workspace");
    unsigned int flag = 0;
    GJ_TRY(pairs_error_flag(const_cast<void*>(d_workspace), workspace_bytes, m, &flag, as_stream(stream)));
    if (flag) {
        set_error("inlj pairs: a tile waited too long for its predecessors' counts; the pairs are incomplete");
        return GJ_ERR_TIMEOUT;
    }
    return GJ_OK;
}

}  // extern "C"
