// gpujoin/device.cuh -- device-side index views and per-probe lookups.
//
// The views are plain structs passed to kernels by value, like the
// reference's device_index_t members (src/indexes.cuh:18-22).  The lookup
// functions are what the library's own kernels run; user kernels written in
// the reference style call them through the device_index_t wrappers in
// gpujoin/indexes.cuh.
//
// All lookups are per-thread (no warp-collective requirement); results
// follow the reference's per-index semantics:
//   binary search / radix spline / learned: lower bound, GJ_INVALID_POS at n
//   B+tree / Harmonia: position of an equal key, else GJ_INVALID_POS.
#pragma once

#include <stdint.h>

#include "../gpujoin.h"

#ifndef GJ_DEVICE_INLINE
#define GJ_DEVICE_INLINE __device__ __forceinline__
#endif

namespace gj {

constexpr uint32_t kInvalid = GJ_INVALID_POS;
constexpr int kBtreeMaxLevels = 8;
constexpr int kHarmoniaKeys = 32;  // keys per Harmonia node (fanout 33, src/indexes.cuh:264)

// ---------------------------------------------------------------------------
// load helpers: read-only data through the non-coherent path
// ---------------------------------------------------------------------------
GJ_DEVICE_INLINE uint64_t ld_ro(const uint64_t* p) { return __ldg(reinterpret_cast<const unsigned long long*>(p)); }
GJ_DEVICE_INLINE uint32_t ld_ro(const uint32_t* p) { return __ldg(reinterpret_cast<const unsigned int*>(p)); }
GJ_DEVICE_INLINE double ld_ro(const double* p) { return __ldg(p); }

// count of a[0..2^k-1) entries < key for a sorted array of 2^k - 1 entries
// (a[2^k - 1] is never read): the child index of a B+tree node.
template <int STEPS>
GJ_DEVICE_INLINE uint32_t count_less_pow2m1(const uint64_t* a, uint64_t key) {
    uint32_t c = 0;
#pragma unroll
    for (int s = STEPS - 1; s >= 0; --s) {
        const uint32_t w = 1u << s;
        c += (ld_ro(a + c + w - 1) < key) ? w : 0u;
    }
    return c;
}

// shared-memory variant (no __ldg on shared addresses)
template <int STEPS>
GJ_DEVICE_INLINE uint32_t count_less_pow2m1_smem(const uint64_t* a, uint64_t key) {
    uint32_t c = 0;
#pragma unroll
    for (int s = STEPS - 1; s >= 0; --s) {
        const uint32_t w = 1u << s;
        c += (a[c + w - 1] < key) ? w : 0u;
    }
    return c;
}

// lower bound over arr[0, len) with len <= 2^STEPS - 1 (entries past len
// count as +infinity)
template <int STEPS>
GJ_DEVICE_INLINE uint32_t lower_bound_bounded(const uint64_t* arr, uint32_t len, uint64_t key) {
    uint32_t c = 0;
#pragma unroll
    for (int s = STEPS - 1; s >= 0; --s) {
        const uint32_t w = 1u << s;
        const uint32_t i = c + w - 1;
        c += (i < len && ld_ro(arr + i) < key) ? w : 0u;
    }
    return c;
}

// classic lower bound (count/step form of src/search.cuh:26-41)
GJ_DEVICE_INLINE uint64_t lower_bound_any(const uint64_t* arr, uint64_t n, uint64_t key) {
    uint64_t lower = 0, count = n;
    while (count > 0) {
        const uint64_t step = count >> 1;
        const uint64_t mid = lower + step;
        if (ld_ro(arr + mid) < key) {
            lower = mid + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    return lower;
}

// branch-free lower bound over any n >= 1 (power-of-two stride form of
// src/search.cuh:143-158, defined for n == 1 as well)
GJ_DEVICE_INLINE uint64_t lower_bound_branch_free(const uint64_t* arr, uint64_t n, uint64_t key) {
    if (n <= 1) return (n == 1 && ld_ro(arr) < key) ? 1 : 0;
    const unsigned steps = 63u - __clzll(n - 1);
    uint64_t mid = 1ull << steps;
    uint64_t ret = (ld_ro(arr + mid) < key) ? (n - mid) : 0;
    for (unsigned s = 1; s <= steps; ++s) {
        mid >>= 1;
        ret += (ld_ro(arr + ret + mid) < key) ? mid : 0;
    }
    ret += (ld_ro(arr + ret) < key) ? 1 : 0;
    return ret;
}

// ---------------------------------------------------------------------------
// binary search index (src/indexes.cuh:336-375)
// ---------------------------------------------------------------------------
// Optional sampled cache: fence[j] = col[j << fence_shift] for j < fence_used,
// padded with UINT64_MAX to fence_slots (a power of two).  The first
// log2(fence_slots) steps of the search then run against the fence (staged
// in shared memory by the library's kernels), the rest against the column.
struct bs_view {
    const uint64_t* col;
    uint64_t n;
    const uint64_t* fence;
    uint32_t fence_slots;  // 0 = no fence
    uint32_t fence_shift;
    uint32_t fence_steps;  // log2(fence_slots)
    uint32_t pad;
};

GJ_DEVICE_INLINE uint32_t bs_lookup(const bs_view& v, const uint64_t* fence, uint64_t key) {
    uint64_t lb;
    if (v.fence_slots == 0) {
        lb = lower_bound_branch_free(v.col, v.n, key);
    } else {
        // c = number of fence keys < key (branch-free over fence_slots entries)
        uint32_t c = 0;
        for (int s = (int)v.fence_steps - 1; s >= 0; --s) {
            const uint32_t w = 1u << s;
            c += (fence[c + w - 1] < key) ? w : 0u;
        }
        c += (fence[c] < key) ? 1u : 0u;
        if (c == 0) {
            lb = 0;
        } else {
            // lower bound lies in ((c-1) << shift, c << shift]
            const uint64_t lo = ((uint64_t)(c - 1) << v.fence_shift) + 1;
            uint64_t hi = (uint64_t)c << v.fence_shift;
            if (hi > v.n) hi = v.n;
            lb = lo + lower_bound_branch_free(v.col + lo, hi - lo, key);
        }
    }
    return lb < v.n ? (uint32_t)lb : kInvalid;
}

// ---------------------------------------------------------------------------
// clustered B+tree with implicit children (replaces src/btree.cuh)
// ---------------------------------------------------------------------------
// Leaves are slices of W keys of the sorted column (clustered, as
// src/btree.cuh:237-243).  Level l >= 1 holds ceil(n / W^(l+1)) nodes of W
// slots; slot c of node j = max key of child (j*W + c) (separator = max key
// of the child, src/btree.cuh:176-206), UINT64_MAX past the last child.
// Children are implicit (node j's children are j*W .. j*W+W-1 one level
// down), so a level is a strided gather of the column.
struct btree_view {
    const uint64_t* col;
    uint64_t n;
    uint64_t max_key;                       // col[n-1]
    const uint64_t* level[kBtreeMaxLevels]; // level[l] for l = 1..height (index 0 unused)
    uint32_t smem_offset[kBtreeMaxLevels];  // offset in keys inside the shared cache
    uint32_t height;                        // number of inner levels (>= 1)
    uint32_t cached_levels;                 // top levels staged in shared memory
    uint32_t cache_keys;                    // total keys staged
    uint32_t node_keys;                     // W
};

template <int LOGW>
GJ_DEVICE_INLINE uint32_t btree_lookup(const btree_view& v, const uint64_t* cache, uint64_t key) {
    constexpr uint32_t W = 1u << LOGW;
    if (key > v.max_key) return kInvalid;
    uint64_t j = 0;
    const int h = (int)v.height;
    const int first_global = h - (int)v.cached_levels;  // levels <= this come from global memory
    for (int l = h; l >= 1; --l) {
        uint32_t c;
        if (l > first_global) {
            c = count_less_pow2m1_smem<LOGW>(cache + v.smem_offset[l] + j * W, key);
        } else {
            c = count_less_pow2m1<LOGW>(v.level[l] + j * W, key);
        }
        j = j * W + c;
    }
    // leaf j: column slice [j*W, min(j*W + W, n))
    const uint64_t base = j * W;
    const uint64_t rem = v.n - base;
    const uint32_t len = rem < W ? (uint32_t)rem : W;
    const uint32_t lb = lower_bound_bounded<LOGW>(v.col + base, len, key);
    const uint64_t pos = base + lb;
    return (lb < len && ld_ro(v.col + pos) == key) ? (uint32_t)pos : kInvalid;
}

// ---------------------------------------------------------------------------
// Harmonia (src/harmonia.cuh: layout :69-89, lookup :740-786)
// ---------------------------------------------------------------------------
// keys: 32 keys per inner node in level order (UINT64_MAX padded); the leaf
// level is the column itself (Reuse_Input_Memory).  children[node] = index
// of the node's first child (inner) or of its first key (leaf level).
struct harmonia_view {
    const uint64_t* keys;
    const uint64_t* children;
    const uint64_t* col;
    uint64_t n;
    uint64_t inner_size;     // 32 * inner node count
    uint32_t depth;
    uint32_t cached_nodes;   // leading nodes (level order) staged in shared memory
    uint32_t cached_levels;  // the cached nodes are exactly the top cached_levels levels
    uint32_t pad;
};

// shared cache layout: cached_nodes * 32 keys, then cached_nodes children
GJ_DEVICE_INLINE uint32_t harmonia_lookup(const harmonia_view& v, const uint64_t* cache, uint64_t key) {
    constexpr uint32_t K = kHarmoniaKeys;
    uint64_t pos = 0;
    const uint32_t depth = v.depth;
    for (uint32_t d = 1; d < depth; ++d) {
        uint32_t lb;
        uint64_t child;
        if (pos < v.cached_nodes) {
            const uint64_t* node = cache + pos * K;
            lb = count_less_pow2m1_smem<5>(node, key);
            lb += (node[lb] < key) ? 1u : 0u;
            child = cache[(uint64_t)v.cached_nodes * K + pos];
        } else {
            const uint64_t* node = v.keys + pos * K;
            lb = count_less_pow2m1<5>(node, key);
            lb += (lb == K - 1 && ld_ro(node + lb) < key) ? 1u : 0u;
            child = ld_ro(v.children + pos);
        }
        pos = child + lb;
    }
    // leaf level: node pos covers column [32*(pos - leaf_prefix), +32)
    const uint64_t leaf_first = (depth > 1) ? (pos * K - v.inner_size) : 0;
    const uint64_t* node = v.col + leaf_first;
    uint32_t lb = count_less_pow2m1<5>(node, key);
    lb += (lb == K - 1 && ld_ro(node + lb) < key) ? 1u : 0u;
    const uint64_t p = leaf_first + lb;
    return (p < v.n && ld_ro(v.col + p) == key) ? (uint32_t)p : kInvalid;
}

// ---------------------------------------------------------------------------
// RadixSpline (src/rs.cuh:118-154, window src/indexes.cuh:205-215)
// ---------------------------------------------------------------------------
struct rs_view {
    const uint64_t* col;
    uint64_t n;
    const uint32_t* table;   // (1 << radix_bits) + 2 entries
    const uint64_t* sx;      // spline point keys
    const double* sy;        // spline point positions
    uint64_t min_key, max_key;
    uint32_t shift;
    uint32_t max_error;
};

GJ_DEVICE_INLINE double rs_estimate(const rs_view& v, uint64_t key) {
    if (key <= v.min_key) return 0.0;
    if (key >= v.max_key) return (double)(v.n - 1);
    const uint64_t prefix = (key - v.min_key) >> v.shift;
    const uint32_t b = ld_ro(v.table + prefix);
    const uint32_t e = ld_ro(v.table + prefix + 1);
    // first spline point with x >= key in [b, e)
    uint32_t lo = b, cnt = e - b;
    while (cnt > 0) {
        const uint32_t step = cnt >> 1, mid = lo + step;
        if (ld_ro(v.sx + mid) < key) {
            lo = mid + 1;
            cnt -= step + 1;
        } else {
            cnt = step;
        }
    }
    const uint64_t dx0 = ld_ro(v.sx + lo - 1), ux = ld_ro(v.sx + lo);
    const double dy0 = ld_ro(v.sy + lo - 1), uy = ld_ro(v.sy + lo);
    const double slope = (uy - dy0) / (double)(ux - dx0);
    return __dadd_rn(__dmul_rn((double)(key - dx0), slope), dy0);
}

GJ_DEVICE_INLINE uint32_t rs_lookup(const rs_view& v, uint64_t key) {
    const double est = rs_estimate(v, key);
    const double err = (double)v.max_error;
    uint64_t b = est < err ? 0 : (uint64_t)(est - err);
    uint64_t e = (est + err + 2 > (double)v.n) ? v.n : (uint64_t)(est + err + 2);
    if (b > e) b = e;
    uint64_t pos = b + lower_bound_branch_free(v.col + b, e - b, key);
    // the window must bracket the lower bound; otherwise search the column
    if ((pos == b && b > 0 && ld_ro(v.col + b - 1) >= key) || (pos == e && e < v.n && ld_ro(v.col + e) < key))
        pos = lower_bound_branch_free(v.col, v.n, key);
    return pos < v.n ? (uint32_t)pos : kInvalid;
}

// ---------------------------------------------------------------------------
// batched lookups: K independent probes per thread searched in lockstep
// ---------------------------------------------------------------------------
// A probe's search is a chain of dependent loads, so one probe per thread
// leaves the memory system idle while the thread waits.  The batched forms
// advance K probes one search step at a time: the K loads of a step are
// independent and are in flight together.  Results equal the single-probe
// functions above.

// branch-free lower bound of key[k] in arr[lo_k, lo_k + len_k) with
// len_k <= 2^steps - 1 for all k
template <int K>
GJ_DEVICE_INLINE void lower_bound_bounded_batch(const uint64_t* arr, const uint64_t (&lo)[K], const uint32_t (&len)[K],
                                                const uint64_t (&key)[K], int steps, uint32_t (&r)[K]) {
#pragma unroll
    for (int k = 0; k < K; ++k) r[k] = 0;
    for (int s = steps - 1; s >= 0; --s) {
        const uint32_t w = 1u << s;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const uint32_t i = r[k] + w - 1;
            r[k] += (i < len[k] && ld_ro(arr + lo[k] + i) < key[k]) ? w : 0u;
        }
    }
}

GJ_DEVICE_INLINE int steps_for(uint64_t len) {  // smallest s with len <= 2^s - 1
    return len == 0 ? 0 : 64 - __clzll(len);
}

template <int K>
GJ_DEVICE_INLINE void bs_lookup_batch(const bs_view& v, const uint64_t* fence, const uint64_t (&key)[K],
                                      uint32_t (&res)[K]) {
    uint64_t lo[K];
    uint32_t len[K];
    int steps;
    if (v.fence_slots == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            lo[k] = 0;
            len[k] = (uint32_t)v.n;
        }
        steps = steps_for(v.n);
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            uint32_t c = 0;
            for (int s = (int)v.fence_steps - 1; s >= 0; --s) {
                const uint32_t w = 1u << s;
                c += (fence[c + w - 1] < key[k]) ? w : 0u;
            }
            c += (fence[c] < key[k]) ? 1u : 0u;
            if (c == 0) {
                lo[k] = 0;
                len[k] = 0;
            } else {
                lo[k] = ((uint64_t)(c - 1) << v.fence_shift) + 1;
                uint64_t hi = (uint64_t)c << v.fence_shift;
                if (hi > v.n) hi = v.n;
                len[k] = (uint32_t)(hi - lo[k]);
            }
        }
        steps = (int)v.fence_shift;  // ranges hold at most 2^shift - 1 keys
    }
    uint32_t r[K];
    lower_bound_bounded_batch<K>(v.col, lo, len, key, steps, r);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const uint64_t lb = lo[k] + r[k];
        res[k] = lb < v.n ? (uint32_t)lb : kInvalid;
    }
}

template <int LOGW, int K>
GJ_DEVICE_INLINE void btree_lookup_batch(const btree_view& v, const uint64_t* cache, const uint64_t (&key)[K],
                                         uint32_t (&res)[K]) {
    constexpr uint32_t W = 1u << LOGW;
    uint64_t tk[K];  // probes above the largest key walk the rightmost path
    uint32_t j[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        tk[k] = key[k] > v.max_key ? v.max_key : key[k];
        j[k] = 0;
    }
    const int h = (int)v.height;
    const int first_global = h - (int)v.cached_levels;
    for (int l = h; l >= 1; --l) {
        uint32_t c[K];
#pragma unroll
        for (int k = 0; k < K; ++k) c[k] = 0;
        if (l > first_global) {
            const uint64_t* base = cache + v.smem_offset[l];
#pragma unroll
            for (int s = LOGW - 1; s >= 0; --s) {
#pragma unroll
                for (int k = 0; k < K; ++k) c[k] += (base[j[k] * W + c[k] + (1u << s) - 1] < tk[k]) ? (1u << s) : 0u;
            }
        } else {
            const uint64_t* base = v.level[l];
#pragma unroll
            for (int s = LOGW - 1; s >= 0; --s) {
#pragma unroll
                for (int k = 0; k < K; ++k)
                    c[k] += (ld_ro(base + (uint64_t)j[k] * W + c[k] + (1u << s) - 1) < tk[k]) ? (1u << s) : 0u;
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) j[k] = j[k] * W + c[k];
    }
    uint64_t lo[K];
    uint32_t len[K], r[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        lo[k] = (uint64_t)j[k] * W;
        const uint64_t rem = v.n - lo[k];
        len[k] = rem < W ? (uint32_t)rem : W;
    }
    lower_bound_bounded_batch<K>(v.col, lo, len, tk, LOGW, r);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const uint64_t pos = lo[k] + r[k];
        res[k] = (key[k] <= v.max_key && r[k] < len[k] && ld_ro(v.col + pos) == key[k]) ? (uint32_t)pos : kInvalid;
    }
}

template <int K>
GJ_DEVICE_INLINE void harmonia_lookup_batch(const harmonia_view& v, const uint64_t* cache, const uint64_t (&key)[K],
                                            uint32_t (&res)[K]) {
    constexpr uint32_t NK = kHarmoniaKeys;
    uint64_t pos[K];
#pragma unroll
    for (int k = 0; k < K; ++k) pos[k] = 0;
    const uint32_t depth = v.depth;
    for (uint32_t d = 1; d < depth; ++d) {
        uint64_t child[K];
        uint32_t lb[K];
#pragma unroll
        for (int k = 0; k < K; ++k) lb[k] = 0;
        if (d <= v.cached_levels) {
            const uint64_t* ch = cache + (uint64_t)v.cached_nodes * NK;
#pragma unroll
            for (int k = 0; k < K; ++k) child[k] = ch[pos[k]];
#pragma unroll
            for (int s = 4; s >= 0; --s) {
#pragma unroll
                for (int k = 0; k < K; ++k) lb[k] += (cache[pos[k] * NK + lb[k] + (1u << s) - 1] < key[k]) ? (1u << s) : 0u;
            }
#pragma unroll
            for (int k = 0; k < K; ++k) lb[k] += (cache[pos[k] * NK + lb[k]] < key[k]) ? 1u : 0u;
        } else {
            // the child offset only depends on the node: load it alongside the search
#pragma unroll
            for (int k = 0; k < K; ++k) child[k] = ld_ro(v.children + pos[k]);
#pragma unroll
            for (int s = 4; s >= 0; --s) {
#pragma unroll
                for (int k = 0; k < K; ++k)
                    lb[k] += (ld_ro(v.keys + pos[k] * NK + lb[k] + (1u << s) - 1) < key[k]) ? (1u << s) : 0u;
            }
#pragma unroll
            for (int k = 0; k < K; ++k)
                lb[k] += (lb[k] == NK - 1 && ld_ro(v.keys + pos[k] * NK + lb[k]) < key[k]) ? 1u : 0u;
        }
#pragma unroll
        for (int k = 0; k < K; ++k) pos[k] = child[k] + lb[k];
    }
    uint64_t lo[K];
    uint32_t len[K], r[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        lo[k] = (depth > 1) ? (pos[k] * NK - v.inner_size) : 0;
        len[k] = NK;
    }
    // 32 keys: 5 steps cover 31, the sixth decides between 31 and 32
    lower_bound_bounded_batch<K>(v.col, lo, len, key, 5, r);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        uint32_t rr = r[k];
        if (rr == NK - 1 && ld_ro(v.col + lo[k] + rr) < key[k]) rr = NK;
        const uint64_t p = lo[k] + rr;
        res[k] = (p < v.n && ld_ro(v.col + p) == key[k]) ? (uint32_t)p : kInvalid;
    }
}

template <int K>
GJ_DEVICE_INLINE void rs_lookup_batch(const rs_view& v, const uint64_t (&key)[K], uint32_t (&res)[K]) {
    // spline segment: radix table, then a short search over the segment's points
    uint32_t lo[K], cnt[K];
    bool inner[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        inner[k] = key[k] > v.min_key && key[k] < v.max_key;
        const uint64_t prefix = inner[k] ? (key[k] - v.min_key) >> v.shift : 0;
        lo[k] = ld_ro(v.table + prefix);
        cnt[k] = inner[k] ? ld_ro(v.table + prefix + 1) - lo[k] : 0;
    }
    bool more = true;
    while (more) {
        more = false;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (cnt[k] > 0) {
                const uint32_t step = cnt[k] >> 1, mid = lo[k] + step;
                if (ld_ro(v.sx + mid) < key[k]) {
                    lo[k] = mid + 1;
                    cnt[k] -= step + 1;
                } else {
                    cnt[k] = step;
                }
                more |= cnt[k] > 0;
            }
        }
    }
    uint64_t b[K], e[K];
    uint32_t len[K], r[K];
    const double err = (double)v.max_error;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double est;
        if (!inner[k]) {
            est = key[k] <= v.min_key ? 0.0 : (double)(v.n - 1);
        } else {
            const uint64_t dx0 = ld_ro(v.sx + lo[k] - 1), ux = ld_ro(v.sx + lo[k]);
            const double dy0 = ld_ro(v.sy + lo[k] - 1), uy = ld_ro(v.sy + lo[k]);
            const double slope = (uy - dy0) / (double)(ux - dx0);
            est = __dadd_rn(__dmul_rn((double)(key[k] - dx0), slope), dy0);
        }
        b[k] = est < err ? 0 : (uint64_t)(est - err);
        e[k] = (est + err + 2 > (double)v.n) ? v.n : (uint64_t)(est + err + 2);
        if (b[k] > e[k]) b[k] = e[k];
        len[k] = (uint32_t)(e[k] - b[k]);
    }
    lower_bound_bounded_batch<K>(v.col, b, len, key, steps_for(2ull * v.max_error + 3), r);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        uint64_t pos = b[k] + r[k];
        if ((pos == b[k] && b[k] > 0 && ld_ro(v.col + b[k] - 1) >= key[k]) ||
            (pos == e[k] && e[k] < v.n && ld_ro(v.col + e[k]) < key[k]))
            pos = lower_bound_branch_free(v.col, v.n, key[k]);
        res[k] = pos < v.n ? (uint32_t)pos : kInvalid;
    }
}

// ---------------------------------------------------------------------------
// learned index: root model -> linear leaf model -> bounded search
// ---------------------------------------------------------------------------
// x = (key - min_key) / (max_key - min_key) in float.  The root predicts the
// key's CDF r(x); leaf = clamp(floor(r * L), 0, L-1).  A leaf predicts
// pos = base + floor(slope * (key - x0)), and err_lo / err_hi are the largest
// under- and over-prediction over the build keys routed to it, measured with
// this same arithmetic, so every build key lies in
// [pred - err_lo, pred + err_hi].  Keys outside the column may fall outside
// that window; the window check below then falls back to the plain binary
// search, so the result is always the exact lower bound.
struct learned_leaf {
    uint64_t x0;      // reference key of the leaf (smallest routed key)
    uint32_t base;    // position of x0
    float slope;      // positions per unit key distance
    uint32_t err_lo;
    uint32_t err_hi;
};

struct learned_view {
    const uint64_t* col;
    uint64_t n;
    uint64_t min_key, max_key;
    float inv_range;            // 1 / (max_key - min_key) (0 if the range is empty)
    uint32_t num_leaves;
    uint32_t root_kind;         // GJ_LEARNED_ROOT_LINEAR or GJ_LEARNED_ROOT_MLP
    uint32_t hidden;            // MLP width H (<= 32)
    const float* root;          // [a, b] (linear) or MLP parameters [W1 b1 W2 b2 W3 b3]
    const learned_leaf* leaves;
};

// root MLP 1 -> H -> H -> 1 with ReLU, parameters [W1(H) b1(H) W2(HxH, out-major) b2(H) W3(H) b3]
GJ_DEVICE_INLINE float mlp_forward(const float* P, int H, float x) {
    const float* W1 = P;
    const float* b1 = P + H;
    const float* W2 = P + 2 * H;
    const float* b2 = W2 + H * H;
    const float* W3 = b2 + H;
    float h1[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const float a = (j < H) ? fmaf(W1[j], x, b1[j]) : 0.f;
        h1[j] = a > 0.f ? a : 0.f;
    }
    float out = W3[H];  // b3 directly follows W3
    for (int o = 0; o < H; ++o) {
        const float* w = W2 + o * H;
        float a = b2[o];
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if (j < H) a = fmaf(w[j], h1[j], a);
        out = fmaf(W3[o], a > 0.f ? a : 0.f, out);
    }
    return out;
}

GJ_DEVICE_INLINE float learned_norm(const learned_view& v, uint64_t key) {
    if (key <= v.min_key) return 0.f;
    if (key >= v.max_key) return 1.f;
    return (float)(key - v.min_key) * v.inv_range;
}

GJ_DEVICE_INLINE uint32_t learned_route(const learned_view& v, const float* root, float x) {
    const float r = (v.root_kind == GJ_LEARNED_ROOT_MLP) ? mlp_forward(root, (int)v.hidden, x)
                                                         : fmaf(root[0], x, root[1]);
    const float lf = floorf(r * (float)v.num_leaves);
    if (!(lf > 0.f)) return 0;  // also catches NaN
    if (lf >= (float)v.num_leaves) return v.num_leaves - 1;
    return (uint32_t)lf;
}

// leaf prediction (signed, may lie outside [0, n))
GJ_DEVICE_INLINE int64_t learned_predict(const learned_leaf& lf, uint64_t key) {
    const float dx = (key >= lf.x0) ? (float)(key - lf.x0) : -(float)(lf.x0 - key);
    // |offset| is kept below 2^62 so that pred +- err cannot overflow
    float off = floorf(lf.slope * dx);
    off = fminf(fmaxf(off, -4.0e18f), 4.0e18f);
    return (int64_t)lf.base + (int64_t)off;
}

GJ_DEVICE_INLINE uint32_t learned_lookup(const learned_view& v, const float* root, uint64_t key) {
    const uint32_t li = learned_route(v, root, learned_norm(v, key));
    const uint64_t* lp = reinterpret_cast<const uint64_t*>(v.leaves + li);
    learned_leaf lf;
    lf.x0 = ld_ro(lp);
    const uint64_t w1 = ld_ro(lp + 1), w2 = ld_ro(lp + 2);
    lf.base = (uint32_t)w1;
    lf.slope = __uint_as_float((uint32_t)(w1 >> 32));
    lf.err_lo = (uint32_t)w2;
    lf.err_hi = (uint32_t)(w2 >> 32);
    const int64_t pred = learned_predict(lf, key);
    const int64_t n = (int64_t)v.n;
    // window [pred - err_lo, pred + err_hi + 1) clamped to [0, n]; a probe far
    // outside the leaf's keys can push both ends below 0 or above n
    int64_t lo = pred - (int64_t)lf.err_lo;
    int64_t hi = pred + (int64_t)lf.err_hi + 1;
    lo = lo < 0 ? 0 : (lo > n ? n : lo);
    hi = hi < 0 ? 0 : (hi > n ? n : hi);
    if (lo > hi) lo = hi;
    const uint64_t b = (uint64_t)lo, e = (uint64_t)hi;
    uint64_t pos = b + lower_bound_branch_free(v.col + b, e - b, key);
    if ((pos == b && b > 0 && ld_ro(v.col + b - 1) >= key) || (pos == e && e < v.n && ld_ro(v.col + e) < key))
        pos = lower_bound_branch_free(v.col, v.n, key);  // exact fallback: the plain binary search
    return pos < v.n ? (uint32_t)pos : kInvalid;
}

template <int K>
GJ_DEVICE_INLINE void learned_lookup_batch(const learned_view& v, const float* root, const uint64_t (&key)[K],
                                           uint32_t (&res)[K]) {
    uint64_t b[K], e[K];
    uint32_t len[K], r[K], maxlen = 0;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const uint32_t li = learned_route(v, root, learned_norm(v, key[k]));
        const uint64_t* lp = reinterpret_cast<const uint64_t*>(v.leaves + li);
        learned_leaf lf;
        lf.x0 = ld_ro(lp);
        const uint64_t w1 = ld_ro(lp + 1), w2 = ld_ro(lp + 2);
        lf.base = (uint32_t)w1;
        lf.slope = __uint_as_float((uint32_t)(w1 >> 32));
        lf.err_lo = (uint32_t)w2;
        lf.err_hi = (uint32_t)(w2 >> 32);
        const int64_t pred = learned_predict(lf, key[k]);
        const int64_t n = (int64_t)v.n;
        int64_t lo = pred - (int64_t)lf.err_lo;
        int64_t hi = pred + (int64_t)lf.err_hi + 1;
        lo = lo < 0 ? 0 : (lo > n ? n : lo);  // clamp both ends to [0, n]
        hi = hi < 0 ? 0 : (hi > n ? n : hi);
        if (lo > hi) lo = hi;
        b[k] = (uint64_t)lo;
        e[k] = (uint64_t)hi;
        len[k] = (uint32_t)(e[k] - b[k]);
        maxlen = len[k] > maxlen ? len[k] : maxlen;
    }
    lower_bound_bounded_batch<K>(v.col, b, len, key, steps_for(maxlen), r);
#pragma unroll
    for (int k = 0; k < K; ++k) {
        uint64_t pos = b[k] + r[k];
        if ((pos == b[k] && b[k] > 0 && ld_ro(v.col + b[k] - 1) >= key[k]) ||
            (pos == e[k] && e[k] < v.n && ld_ro(v.col + e[k]) < key[k]))
            pos = lower_bound_branch_free(v.col, v.n, key[k]);  // exact fallback: the plain binary search
        res[k] = pos < v.n ? (uint32_t)pos : kInvalid;
    }
}

}  // namespace gj
