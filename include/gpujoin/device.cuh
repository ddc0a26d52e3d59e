// gpujoin/device.cuh -- device-side index views and per-probe lookups.
//
// The views are plain structs passed to kernels by value, like the
// reference's device_index_t members (src/indexes.cuh:18-22).  The lookup
// functions are what the library's own kernels run; reference-style kernels
// call them through the device_index_t wrappers in gpujoin/indexes.cuh.
//
// All lookups are per-thread (no warp-collective requirement), except the
// warp-cooperative searches near the end of this file, which mirror the
// reference's cooperative entry points; results follow the reference's
// per-index semantics:
//   binary search / radix spline / learned: lower bound, GJ_INVALID_POS at n
//   B+tree / Harmonia: position of an equal key, else GJ_INVALID_POS.
//
// Memory access: a probe touches random addresses, and on GB300 each
// scattered load costs one L1 wavefront per 32-byte sector whatever its
// width.  The searches therefore read whole sectors (four uint64 keys) with
// one 256-bit load and compare all four keys: a sector-granular binary
// search needs about log2(n/4) loads instead of log2(n).  Arrays the
// sector loads read must be 32-byte aligned; the views record whether the
// caller's column is, and fall back to 8-byte loads when it is not.
#pragma once

#include <stdint.h>

#include "../gpujoin.h"

#ifndef GJ_DEVICE_INLINE
#define GJ_DEVICE_INLINE __device__ __forceinline__
#endif

namespace gj {

constexpr uint32_t kInvalid = GJ_INVALID_POS;
constexpr int kBtreeMaxLevels = 16;
constexpr int kHarmoniaKeys = 32;  // keys per Harmonia node (fanout 33, src/indexes.cuh:264)

// ---------------------------------------------------------------------------
// loads
// ---------------------------------------------------------------------------
GJ_DEVICE_INLINE uint64_t ld_ro(const uint64_t* p) { return __ldg(reinterpret_cast<const unsigned long long*>(p)); }
GJ_DEVICE_INLINE uint32_t ld_ro(const uint32_t* p) { return __ldg(reinterpret_cast<const unsigned int*>(p)); }
GJ_DEVICE_INLINE double ld_ro(const double* p) { return __ldg(p); }

// one 32-byte sector (4 keys) through the non-coherent path; p 32-byte aligned
GJ_DEVICE_INLINE void ld_sector(const uint64_t* p, uint64_t (&k)[4]) {
    asm("ld.global.nc.v4.u64 {%0, %1, %2, %3}, [%4];"
        : "=l"(k[0]), "=l"(k[1]), "=l"(k[2]), "=l"(k[3])
        : "l"(p));
}

// one 32-byte sector, asking L2 to fill 64 bytes on a miss: a random sector
// read otherwise fills 128 bytes (measured: 122.5 against 62.6 bytes of DRAM
// reads per random load); for data without spatial locality
GJ_DEVICE_INLINE void ld_sector_64(const uint64_t* p, uint64_t (&k)[4]) {
    asm("ld.global.nc.L2::64B.v4.u64 {%0, %1, %2, %3}, [%4];"
        : "=l"(k[0]), "=l"(k[1]), "=l"(k[2]), "=l"(k[3])
        : "l"(p));
}

// L2 eviction classes for the two kinds of index data: the inner levels of a
// tree (tens of MB, read by every probe) are kept over the column sectors a
// probe reads once (hundreds of MB, random).  Loads carry an L2 cache policy;
// no device-wide setting is involved.  Both classes serve scattered probes,
// whose neighbouring sectors are of no use: their misses fill 64 bytes.
enum l2_class : int { kL2Default = 0, kL2Keep = 1, kL2Stream = 2 };

template <int kClass>
GJ_DEVICE_INLINE uint64_t l2_policy() {
    uint64_t p;
    if constexpr (kClass == kL2Keep)
        asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    else
        asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

template <int kClass>
GJ_DEVICE_INLINE void ld_sector_c(const uint64_t* p, uint64_t (&k)[4]) {
    if constexpr (kClass == kL2Default) {
        ld_sector(p, k);
    } else {
        asm("ld.global.nc.L2::cache_hint.L2::64B.v4.u64 {%0, %1, %2, %3}, [%4], %5;"
            : "=l"(k[0]), "=l"(k[1]), "=l"(k[2]), "=l"(k[3])
            : "l"(p), "l"(l2_policy<kClass>()));
    }
}

// 16 bytes (p 16-byte aligned) under the L2 class, 64-byte fill on a miss
template <int kClass>
GJ_DEVICE_INLINE void ld_pair_c(const uint64_t* p, uint64_t (&k)[2]) {
    if constexpr (kClass == kL2Default) {
        asm("ld.global.nc.v2.u64 {%0, %1}, [%2];" : "=l"(k[0]), "=l"(k[1]) : "l"(p));
    } else {
        asm("ld.global.nc.L2::cache_hint.L2::64B.v2.u64 {%0, %1}, [%2], %3;"
            : "=l"(k[0]), "=l"(k[1])
            : "l"(p), "l"(l2_policy<kClass>()));
    }
}

template <int kClass>
GJ_DEVICE_INLINE uint64_t ld_ro_c(const uint64_t* p) {
    if constexpr (kClass == kL2Default) {
        return ld_ro(p);
    } else {
        uint64_t v;
        asm("ld.global.nc.L2::cache_hint.L2::64B.u64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(l2_policy<kClass>()));
        return v;
    }
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

// k[i] for a run-time i < 4 without indexing the array (which would put it
// in local memory)
GJ_DEVICE_INLINE uint64_t pick4(const uint64_t (&k)[4], uint32_t i) {
    const uint64_t lo = (i & 1) ? k[1] : k[0];
    const uint64_t hi = (i & 1) ? k[3] : k[2];
    return (i & 2) ? hi : lo;
}

// Lower bound of key in arr[lo, hi) by a binary search over the 32-byte
// sectors that cover the range.  arr must be 32-byte aligned when aligned is
// set; arr_n is the number of valid entries of arr (a sector that reaches
// past it is read with 8-byte loads).  *eq tells whether arr[result] == key
// (result < hi).  Invariant: in-range keys of sectors below sl are < key,
// those of sectors above sr are >= key.
template <int kClass = kL2Default>
GJ_DEVICE_INLINE uint64_t lower_bound_sectors(const uint64_t* arr, uint64_t arr_n, uint64_t lo, uint64_t hi,
                                              uint64_t key, bool aligned, bool* eq) {
    *eq = false;
    if (lo >= hi) return lo;
    if (!aligned) {
        const uint64_t r = lo + lower_bound_branch_free(arr + lo, hi - lo, key);
        *eq = r < hi && ld_ro(arr + r) == key;
        return r;
    }
    // positions are below 2^32 - 1 (columns hold at most 2^32 - 2 keys), so
    // the search runs on 32-bit positions; hi <= arr_n keeps every sector
    // start below arr_n
    const uint32_t lo32 = (uint32_t)lo, hi32 = (uint32_t)hi, n32 = (uint32_t)arr_n;
    uint32_t sl = lo32 >> 2, sr = (hi32 - 1) >> 2;
    // first in-range position known to hold a key >= key, and that key: the
    // answer may end up there after the sector that holds it was ruled out
    uint32_t right_pos = hi32;
    uint64_t right_key = 0;
    for (;;) {
        const uint32_t s = (sl + sr) >> 1;
        const uint32_t s0 = s << 2;
        uint64_t k[4];
        if (n32 - s0 >= 4) {
            ld_sector_c<kClass>(arr + s0, k);
        } else {
#pragma unroll
            for (uint32_t i = 0; i < 4; ++i) k[i] = (i < n32 - s0) ? ld_ro_c<kClass>(arr + s0 + i) : ~0ull;
        }
        const uint32_t first = s0 > lo32 ? s0 : lo32;
        const uint32_t last = hi32 - s0 > 4 ? s0 + 4 : hi32;
        uint32_t below = 0;
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) below += (s0 + i >= first && s0 + i < last && k[i] < key) ? 1u : 0u;
        const uint32_t in_range = last - first;
        if (below == in_range) {  // every in-range key of the sector is < key
            if (s == sr) {
                *eq = last == right_pos && right_key == key;
                return last;
            }
            sl = s + 1;
        } else if (below == 0 && s != sl) {  // every in-range key is >= key, earlier sectors remain
            right_pos = first;
            right_key = pick4(k, first - s0);
            sr = s - 1;
        } else {
            const uint32_t r = first + below;
            *eq = pick4(k, r - s0) == key;
            return r;
        }
    }
}

// ---------------------------------------------------------------------------
// binary search index (src/indexes.cuh:336-375)
// ---------------------------------------------------------------------------
// Optional sampled cache: fence[j] = col[j << fence_shift], padded with
// UINT64_MAX to fence_slots (a power of two).  The first log2(fence_slots)
// steps of the search run against the fence (staged in shared memory by the
// library's kernels), the rest against the column.
struct bs_view {
    const uint64_t* col;
    uint64_t n;
    const uint64_t* fence;
    uint32_t fence_slots;  // 0 = no fence
    uint32_t fence_shift;
    uint32_t fence_steps;  // log2(fence_slots)
    uint32_t col_aligned;  // column base is 32-byte aligned
};

GJ_DEVICE_INLINE uint32_t bs_lookup(const bs_view& v, const uint64_t* fence, uint64_t key) {
    uint64_t lo = 0, hi = v.n;
    if (v.fence_slots != 0) {
        // c = number of fence keys < key (branch-free over fence_slots entries)
        uint32_t c = 0;
        for (int s = (int)v.fence_steps - 1; s >= 0; --s) {
            const uint32_t w = 1u << s;
            c += (fence[c + w - 1] < key) ? w : 0u;
        }
        c += (fence[c] < key) ? 1u : 0u;
        if (c == 0) return 0;  // col[0] >= key
        // the lower bound lies in ((c-1) << shift, c << shift]
        lo = ((uint64_t)(c - 1) << v.fence_shift) + 1;
        hi = (uint64_t)c << v.fence_shift;
        if (hi > v.n) hi = v.n;
    }
    bool eq;
    const uint64_t lb = lower_bound_sectors(v.col, v.n, lo, hi, key, v.col_aligned, &eq);
    return lb < v.n ? (uint32_t)lb : kInvalid;
}

// ---------------------------------------------------------------------------
// clustered B+tree with implicit children (replaces src/btree.cuh)
// ---------------------------------------------------------------------------
// Leaves are slices of L keys of the sorted column (clustered, as
// src/btree.cuh:237-243).  An inner node holds W separators and W+1
// children; separator c = max key of child c (src/btree.cuh:176-206), the
// last child has none (its max is the separator above), and slots past the
// last child hold UINT64_MAX.  Children are implicit: node j's children are
// j*(W+1) .. j*(W+1)+W one level down, so no pointers are stored and a level
// is a strided gather of the column.  With W = 4 a node is one 32-byte
// sector: one load per level.
struct btree_view {
    const uint64_t* col;
    uint64_t n;
    uint64_t min_key;                       // col[0]
    uint64_t max_key;                       // col[n-1]
    const uint64_t* level[kBtreeMaxLevels]; // level[l] for l = 1..height (index 0 unused)
    uint32_t smem_offset[kBtreeMaxLevels];  // offset in keys inside the shared cache
    uint32_t height;                        // number of inner levels (>= 1)
    uint32_t cached_levels;                 // top levels staged in shared memory
    uint32_t cache_keys;                    // total keys staged
    uint32_t node_keys;                     // W (separators per node)
    uint32_t leaf_keys;                     // L
    uint32_t col_aligned;                   // column base is 32-byte aligned
    // start table: the key range [min_key, max_key] cut into buckets of
    // 2^start_shift keys; entry b (16 bytes: base, node | level << 32) is the
    // deepest node every key of bucket b passes, where a lookup starts its
    // descent (null: from the root)
    const uint64_t* start;
    uint32_t start_shift;
    uint32_t start_entries;
};

// Compressed nodes (W = 7): a node is one 32-byte sector of 8 uint32 words,
// a header (the node's shift s) and 7 separators stored as deltas
// d_i = (sep_i - base) >> s, fanout 8.  The base of the root is col[0]; the
// base of child c of a node (base B, shift s) is B for c = 0 and
// B + (d_{c-1} << s) otherwise -- never above the child's smallest key.  s is
// the smallest shift that brings (node max - B) below 2^31, and a missing
// child's slot holds 0xFFFFFFFF.  With kd = (key - B) >> s, kd > d_i means
// key > sep_i and kd < d_i means key < sep_i; kd == d_i (same 2^s bucket) is
// open.
//
// The search sends an open slot left (key <= sep_i), which is right for
// every key equal to a separator -- the common case, probes being column keys
// -- and needs no extra load.  A wrong left turn (key > sep_i) only ever
// leads to a leaf whose keys are all below the key, while a correct descent
// ends in a leaf whose largest key is >= the key; so a leaf search that runs
// off the leaf's end (before n) reveals it, and only then the search runs
// again resolving open slots exactly, with the separator (the last key of
// child i's subtree) read from the column.  kd is clamped below 0xFFFFFFFF
// for keys that passed a wrong turn.
constexpr uint32_t kBtreeCompressed = 7;
constexpr uint32_t kBtreeAbsent = 0xFFFFFFFFu;

GJ_DEVICE_INLINE uint32_t pick8(const uint32_t (&w)[8], uint32_t i) {
    const uint32_t a = (i & 1) ? w[1] : w[0], b = (i & 1) ? w[3] : w[2];
    const uint32_t c = (i & 1) ? w[5] : w[4], d = (i & 1) ? w[7] : w[6];
    const uint32_t lo = (i & 2) ? b : a, hi = (i & 2) ? d : c;
    return (i & 4) ? hi : lo;
}

// child of compressed node j (words w, base *B) to descend into; updates *B
// to the child's base.  span = column keys under one child.
template <int kInner, bool kExact>
GJ_DEVICE_INLINE uint32_t btree_c7_child(const btree_view& v, const uint32_t (&w)[8], uint64_t j, uint64_t span,
                                         uint64_t key, uint64_t* B) {
    const uint32_t sh = w[0] & 63u;
    const uint64_t q = (key - *B) >> sh;
    const uint32_t kd = q < 0xFFFFFFFEull ? (uint32_t)q : 0xFFFFFFFEu;
    uint32_t c = 0, same = 0;
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        c += kd > w[i + 1] ? 1u : 0u;
        same |= (kd == w[i + 1] ? 1u : 0u) << i;
    }
    if constexpr (kExact) {
        while (same) {  // same 2^s bucket: compare with the exact separator
            const uint32_t i = __ffs(same) - 1;
            same &= same - 1;
            const uint64_t first = (j * 8 + (uint64_t)i) * span;
            const uint64_t last = first + span < v.n ? first + span : v.n;
            c += ld_ro_c<kInner>(v.col + last - 1) < key ? 1u : 0u;
        }
    }
    if (c) *B += (uint64_t)pick8(w, c) << sh;
    return c;
}

// Compressed nodes of 16 lanes (node width 15): lane 0 = 0xFFC0 | s, lanes
// 1..15 = 0x8000 | ((separator - B) >> s), a 14-bit delta of at most
// kBtreeMaxDelta16; 0xFFFF past the column's end.  Lane i sits in logical
// word i / 2, low half for even i.  With every lane in [0x8000, 0xFFFF] and
// the probe value kd at most 0x3FFE, one 32-bit subtraction compares two
// lanes with the probe: lane - kd stays in [0x4002, 0xFFFF], so no borrow
// crosses into the other lane, and bit 15 of a separator lane is set iff its
// delta >= kd.  The header and absent lanes always count as >= kd.
constexpr uint32_t kBtreeCompressed16 = 15;
constexpr uint32_t kBtreeAbsent16 = 0xFFFFu;
constexpr uint32_t kBtreeHeader16 = 0xFFC0u;
constexpr uint32_t kBtreeLaneBias16 = 0x8000u;
constexpr uint32_t kBtreeMaxDelta16 = 0x3FFEu;

// delta of lane i (bias removed)
GJ_DEVICE_INLINE uint32_t lane16(const uint32_t (&w)[8], uint32_t i) {
    return __byte_perm(pick8(w, i >> 1), 0, (i & 1) ? 0x4432u : 0x4410u) & 0x7FFFu;
}

template <int kInner, bool kExact>
GJ_DEVICE_INLINE uint32_t btree_c15_child(const btree_view& v, const uint32_t (&w)[8], uint64_t j, uint64_t span,
                                          uint64_t key, uint64_t* B) {
    const uint32_t sh = w[0] & 63u;
    const uint64_t q = (key - *B) >> sh;
    const uint32_t kd = q < kBtreeMaxDelta16 ? (uint32_t)q : kBtreeMaxDelta16;
    const uint32_t q2 = kd * 0x00010001u;
    uint32_t ge = 0;  // lanes >= kd (the header lane always)
#pragma unroll
    for (int i = 0; i < 8; ++i) ge += __popc((w[i] - q2) & 0x80008000u);
    uint32_t c = 16u - ge;
    if constexpr (kExact) {
        // separators equal to kd follow c (they are sorted): step right over
        // those whose exact key is below the probe
        for (uint32_t i = c; i < 15u; ++i) {
            if (lane16(w, i + 1) != kd) break;
            const uint64_t first = (j * 16 + (uint64_t)i) * span;
            const uint64_t last = first + span < v.n ? first + span : v.n;
            if (!(ld_ro_c<kInner>(v.col + last - 1) < key)) break;
            c = i + 1;
        }
    }
    if (c) *B += (uint64_t)lane16(w, c) << sh;
    return c;
}

// the 8 words of compressed node j of level l, from the shared cache or from
// global memory
template <int kInner>
GJ_DEVICE_INLINE void btree_cx_node(const btree_view& v, const uint64_t* cache, int l, uint32_t j, bool in_smem,
                                    uint32_t (&w)[8]) {
    if (in_smem) {
        const uint64_t* node = cache + v.smem_offset[l] + (uint64_t)j * 4;
        // halves in a node-dependent order (bank groups, see btree_node_search)
        const uint32_t hf = (uint32_t)(reinterpret_cast<uintptr_t>(node) >> 7) & 1u;
        const ulonglong2 x = reinterpret_cast<const ulonglong2*>(node)[hf];
        const ulonglong2 y = reinterpret_cast<const ulonglong2*>(node)[hf ^ 1u];
        const ulonglong2 lo = hf ? y : x, hi = hf ? x : y;
        w[0] = (uint32_t)lo.x, w[1] = (uint32_t)(lo.x >> 32), w[2] = (uint32_t)lo.y, w[3] = (uint32_t)(lo.y >> 32);
        w[4] = (uint32_t)hi.x, w[5] = (uint32_t)(hi.x >> 32), w[6] = (uint32_t)hi.y, w[7] = (uint32_t)(hi.y >> 32);
    } else {
        uint64_t k[4];
        ld_sector_c<kInner>(v.level[l] + (uint64_t)j * 4, k);
        w[0] = (uint32_t)k[0], w[1] = (uint32_t)(k[0] >> 32), w[2] = (uint32_t)k[1], w[3] = (uint32_t)(k[1] >> 32);
        w[4] = (uint32_t)k[2], w[5] = (uint32_t)(k[2] >> 32), w[6] = (uint32_t)k[3], w[7] = (uint32_t)(k[3] >> 32);
    }
}

template <int W>
constexpr int btree_cx_log = W == (int)kBtreeCompressed ? 3 : 4;  // log2 of a compressed node's fanout

template <int W, int kInner, bool kExact>
GJ_DEVICE_INLINE uint32_t btree_cx_child(const btree_view& v, const uint32_t (&w)[8], uint32_t j, uint64_t span,
                                         uint64_t key, uint64_t* B) {
    if constexpr (W == (int)kBtreeCompressed) return btree_c7_child<kInner, kExact>(v, w, j, span, key, B);
    else return btree_c15_child<kInner, kExact>(v, w, j, span, key, B);
}

// leaf reached for key through compressed nodes (open slots left, or exact),
// starting at node j (base B) of level l; l = 0 means j is the leaf
template <int W, int kInner, bool kExact>
GJ_DEVICE_INLINE uint32_t btree_cx_descend(const btree_view& v, const uint64_t* cache, uint64_t key, int l,
                                           uint32_t j, uint64_t B) {
    constexpr int kLog = btree_cx_log<W>;
    const int first_global = (int)v.height - (int)v.cached_levels;
    uint64_t span = l >= 1 ? (uint64_t)v.leaf_keys << (kLog * (l - 1)) : 0;  // column keys under one child
    uint32_t w[8];
    for (; l > first_global; --l, span >>= kLog) {
        btree_cx_node<kInner>(v, cache, l, j, true, w);
        j = (j << kLog) + btree_cx_child<W, kInner, kExact>(v, w, j, span, key, &B);
    }
    for (; l >= 1; --l, span >>= kLog) {
        btree_cx_node<kInner>(v, cache, l, j, false, w);
        j = (j << kLog) + btree_cx_child<W, kInner, kExact>(v, w, j, span, key, &B);
    }
    return j;
}

// children below a node: the count of separators < key, in [0, W]
template <int W, int kInner = kL2Keep>
GJ_DEVICE_INLINE uint32_t btree_node_search(const uint64_t* node, uint64_t key, bool in_smem) {
    if constexpr (W == 4) {
        uint64_t k[4];
        if (in_smem) {
            // A 16-byte shared load is served 8 lanes at a time, conflict
            // free when those lanes hit 8 different 16-byte bank groups.
            // Node j's halves sit in groups 2j and 2j+1 (mod 8), so loading
            // the low half first would use even groups only; every second
            // run of 4 nodes loads its high half first instead, and the
            // first loads of random nodes spread over all 8 groups.  The
            // count below does not depend on the order.
            const uint32_t h = (uint32_t)(reinterpret_cast<uintptr_t>(node) >> 7) & 1u;
            const ulonglong2 a = reinterpret_cast<const ulonglong2*>(node)[h];
            const ulonglong2 b = reinterpret_cast<const ulonglong2*>(node)[h ^ 1u];
            k[0] = a.x;
            k[1] = a.y;
            k[2] = b.x;
            k[3] = b.y;
        } else {
            ld_sector_c<kInner>(node, k);
        }
        return (k[0] < key) + (k[1] < key) + (k[2] < key) + (k[3] < key);
    } else {
        if (in_smem) {
            uint32_t c = 0;  // branch-free over W entries (power of two)
#pragma unroll
            for (int w = W / 2; w >= 1; w >>= 1) c += (node[c + w - 1] < key) ? w : 0u;
            return c + ((node[c] < key) ? 1u : 0u);
        }
        bool eq;
        return (uint32_t)lower_bound_sectors<kInner>(node, W, 0, W, key, true, &eq);
    }
}

// Where a descent starts: node `node` of level `level` (0: `node` is the
// leaf), whose base is `base` (compressed nodes).
struct btree_cursor {
    uint64_t base;
    uint32_t node;
    int32_t level;
};

GJ_DEVICE_INLINE btree_cursor btree_root(const btree_view& v) { return {v.min_key, 0u, (int32_t)v.height}; }

template <int W, int kInner>
GJ_DEVICE_INLINE uint32_t btree_plain_descend(const btree_view& v, const uint64_t* cache, uint64_t key, int l,
                                              uint32_t j) {
    constexpr uint32_t F = W + 1;
    // node and leaf numbers are below 2^32 (at most one leaf per key)
    const int first_global = (int)v.height - (int)v.cached_levels;  // levels <= this come from global memory
    for (; l > first_global; --l) j = j * F + btree_node_search<W>(cache + v.smem_offset[l] + j * W, key, true);
    for (; l >= 1; --l) j = j * F + btree_node_search<W, kInner>(v.level[l] + (uint64_t)j * W, key, false);
    return j;
}

// kScattered: probes arrive in random key order -- the inner levels are
// kept in L2 over the column sectors, which are streamed.  Partitioned
// probes (nearby keys in a row) reuse column sectors and touch only a slice
// of the inner levels: both use the default class then.
//
// The search starts at `from`, a node on the key's path (the root, or the
// deepest node shared by the paths of a run of sorted probes).
template <int W, bool kScattered = true>
GJ_DEVICE_INLINE uint32_t btree_lookup_from(const btree_view& v, const uint64_t* cache, uint64_t key,
                                            const btree_cursor& from) {
    constexpr int kInner = kScattered ? kL2Keep : kL2Default;
    constexpr int kColumn = kScattered ? kL2Stream : kL2Default;
    constexpr bool kCompressed = W == (int)kBtreeCompressed || W == (int)kBtreeCompressed16;
    if (key > v.max_key || key < v.min_key) return kInvalid;
    uint64_t j;
    if constexpr (kCompressed) j = btree_cx_descend<W, kInner, false>(v, cache, key, from.level, from.node, from.base);
    else j = btree_plain_descend<W, kInner>(v, cache, key, from.level, from.node);
    // leaf j: column slice [j*L, min(j*L + L, n))
    uint64_t base = j * v.leaf_keys;
    uint64_t end = base + v.leaf_keys < v.n ? base + v.leaf_keys : v.n;
    bool eq;
    uint64_t pos;
    if (v.leaf_keys == 4 && v.col_aligned && end == base + 4) {
        // a full leaf of one aligned sector: one load, four compares
        uint64_t k[4];
        ld_sector_c<kColumn>(v.col + base, k);
        const uint32_t below = (k[0] < key ? 1u : 0u) + (k[1] < key ? 1u : 0u) + (k[2] < key ? 1u : 0u) +
                               (k[3] < key ? 1u : 0u);
        pos = base + below;
        eq = below < 4 && pick4(k, below & 3u) == key;
    } else {
        pos = lower_bound_sectors<kColumn>(v.col, v.n, base, end, key, v.col_aligned, &eq);
    }
    if constexpr (kCompressed) {
        // a wrong left turn: search again, open slots resolved exactly
        if (pos == end && end < v.n) {  // a wrong left turn: search again, open slots resolved exactly
            j = btree_cx_descend<W, kInner, true>(v, cache, key, (int)v.height, 0u, v.min_key);
            base = j * v.leaf_keys;
            end = base + v.leaf_keys < v.n ? base + v.leaf_keys : v.n;
            pos = lower_bound_sectors<kColumn>(v.col, v.n, base, end, key, v.col_aligned, &eq);
        }
    }
    return eq ? (uint32_t)pos : kInvalid;
}

// A scattered lookup starts at its key bucket's entry of the start table:
// one 16-byte load in place of the levels above that node.
template <int W, bool kScattered = true>
GJ_DEVICE_INLINE uint32_t btree_lookup(const btree_view& v, const uint64_t* cache, uint64_t key) {
    if (key > v.max_key || key < v.min_key) return kInvalid;
    if (v.start == nullptr) return btree_lookup_from<W, kScattered>(v, cache, key, btree_root(v));
    uint64_t e[2];
    ld_pair_c<kScattered ? kL2Keep : kL2Default>(v.start + 2 * ((key - v.min_key) >> v.start_shift), e);
    return btree_lookup_from<W, kScattered>(v, cache, key, {e[0], (uint32_t)e[1], (int32_t)(e[1] >> 32)});
}

// The deepest node on the paths of both lo and hi (lo <= hi): every key in
// [lo, hi] passes through it, since the exact descent is monotonic in the
// key.  Used once per tile of sorted probes.
template <int W, bool kScattered = true>
GJ_DEVICE_INLINE btree_cursor btree_common_node(const btree_view& v, const uint64_t* cache, uint64_t lo,
                                                uint64_t hi) {
    constexpr int kInner = kScattered ? kL2Keep : kL2Default;
    btree_cursor c = btree_root(v);
    lo = lo < v.min_key ? v.min_key : lo;
    hi = hi > v.max_key ? v.max_key : hi;
    if (lo > hi) return c;
    const int first_global = (int)v.height - (int)v.cached_levels;
    if constexpr (W == (int)kBtreeCompressed || W == (int)kBtreeCompressed16) {
        constexpr int kLog = btree_cx_log<W>;
        uint64_t span = (uint64_t)v.leaf_keys << (kLog * (c.level - 1));
        for (; c.level >= 1; --c.level, span >>= kLog) {
            uint32_t w[8];
            btree_cx_node<kInner>(v, cache, c.level, c.node, c.level > first_global, w);
            uint64_t b_lo = c.base, b_hi = c.base;
            const uint32_t a = btree_cx_child<W, kInner, true>(v, w, c.node, span, lo, &b_lo);
            const uint32_t b = btree_cx_child<W, kInner, true>(v, w, c.node, span, hi, &b_hi);
            if (a != b) break;
            c.node = (c.node << kLog) + a;
            c.base = b_lo;
        }
    } else {
        for (; c.level >= 1; --c.level) {
            const bool sm = c.level > first_global;
            const uint64_t* node = sm ? cache + v.smem_offset[c.level] + (uint64_t)c.node * W
                                      : v.level[c.level] + (uint64_t)c.node * W;
            const uint32_t a = btree_node_search<W, kInner>(node, lo, sm);
            const uint32_t b = btree_node_search<W, kInner>(node, hi, sm);
            if (a != b) break;
            c.node = c.node * (W + 1) + a;
        }
    }
    return c;
}

// ---------------------------------------------------------------------------
// Linear-probing hash table: the build side of the reference's hash join
// (src/linear_probing_hashtable.cuh:13-73, src/generic_hj.cu:7-50), kept as
// an index kind so that every probe operator can run against it.
// ---------------------------------------------------------------------------
// Slots of 16 bytes (key, position, pad); the capacity is a power of two of
// at least twice the key count (load factor <= 0.5, as the reference's
// max_load_factor).  A slot whose position is 0xFFFFFFFF is empty: positions
// are below n < 2^32 - 1, so every 64-bit key can be stored, UINT64_MAX (the
// reference's empty key marker) included.  The home of a key is MurmurHash3's
// 64-bit finaliser of the key (the reference hashes with murmur3 as well).
// Linear probing runs over buckets of two slots -- one 32-byte sector, read
// with one load: a key goes to the first free slot of its home bucket, then
// of the next bucket, and so on (the reference probes slot by slot).
struct hash_slot {
    uint64_t key;
    uint32_t pos;
    uint32_t pad;
};
struct hash_view {
    const hash_slot* slots;
    uint64_t mask;  // buckets - 1 (a bucket = 2 slots)
    uint64_t n;
};
constexpr uint32_t kHashEmpty = 0xFFFFFFFFu;

// fmix64 of MurmurHash3 (Austin Appleby, public domain)
__host__ __device__ __forceinline__ uint64_t murmur3_fmix64(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// position of the slot holding key, else kInvalid; the table always has an
// empty slot, and the walk is bounded by the bucket count besides
GJ_DEVICE_INLINE uint32_t hash_lookup(const hash_view& v, uint64_t key) {
    uint64_t b = murmur3_fmix64(key) & v.mask;
    for (uint64_t step = 0; step <= v.mask; ++step) {
        uint64_t w[4];  // slot 0: key, pos | pad << 32; slot 1: key, pos | pad << 32
        ld_sector_64(reinterpret_cast<const uint64_t*>(v.slots + 2 * b), w);
        const uint32_t p0 = (uint32_t)w[1], p1 = (uint32_t)w[3];
        if (p0 == kHashEmpty) return kInvalid;
        if (w[0] == key) return p0;
        if (p1 == kHashEmpty) return kInvalid;
        if (w[2] == key) return p1;
        b = (b + 1) & v.mask;
    }
    return kInvalid;
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
    uint32_t col_aligned;    // column base is 32-byte aligned
    // start table: the key range [min_key, max key] cut into buckets of
    // 2^start_shift keys; entry b (8 bytes: node | level << 56) is the
    // deepest node every key of bucket b passes, where a lookup starts its
    // descent (null: from the root)
    uint64_t min_key;
    const uint64_t* start;
    uint32_t start_shift;
    uint32_t start_entries;
};

// Shared cache layout: cached_nodes * 32 keys, then cached_nodes children.
// A node's child offset does not depend on the search, so it is loaded
// alongside the node's keys.
template <bool kScattered = true>
GJ_DEVICE_INLINE uint32_t harmonia_lookup(const harmonia_view& v, const uint64_t* cache, uint64_t key) {
    constexpr int kInner = kScattered ? kL2Keep : kL2Default;
    constexpr int kColumn = kScattered ? kL2Stream : kL2Default;
    constexpr uint32_t K = kHarmoniaKeys;
    uint64_t pos = 0;
    uint32_t d0 = 1;
    const uint32_t depth = v.depth;
    if (v.start != nullptr && key >= v.min_key) {
        // one 8-byte load in place of the levels above the bucket's node
        const uint64_t b = (key - v.min_key) >> v.start_shift;
        if (b < v.start_entries) {
            const uint64_t e = ld_ro_c<kInner>(v.start + b);
            pos = e & ((1ull << 56) - 1);
            d0 = (uint32_t)(e >> 56);
        }
    }
    for (uint32_t d = d0; d < depth; ++d) {
        uint32_t lb;
        uint64_t child;
        if (d <= v.cached_levels) {
            const uint64_t* node = cache + pos * K;
            uint32_t c = 0;
#pragma unroll
            for (int w = 16; w >= 1; w >>= 1) c += (node[c + w - 1] < key) ? w : 0u;
            lb = c + ((node[c] < key) ? 1u : 0u);
            child = cache[(uint64_t)v.cached_nodes * K + pos];
        } else {
            child = ld_ro_c<kInner>(v.children + pos);
            bool eq;
            lb = (uint32_t)lower_bound_sectors<kInner>(v.keys + pos * K, K, 0, K, key, true, &eq);
        }
        pos = child + lb;
    }
    // leaf level: node pos covers column [32*pos - inner_size, +32)
    const uint64_t leaf_first = (depth > 1) ? (pos * K - v.inner_size) : 0;
    bool eq;
    const uint64_t p =
        lower_bound_sectors<kColumn>(v.col, v.n, leaf_first, leaf_first + K, key, v.col_aligned, &eq);
    return eq ? (uint32_t)p : kInvalid;
}

// ---------------------------------------------------------------------------
// Warp-cooperative searches: the counterparts of the reference's
// cooperative_binary_search (src/search.cuh:296-386) and
// harmonia_tree::lookup<Degree> (src/harmonia.cuh:740-786).  Groups of
// 2^kDegree lanes serve their members' queries one after another; every
// round each lane of the group loads one key (or one 2^(5-kDegree)-key slice
// of a Harmonia node) and a ballot or a reduction combines them.  All 32
// lanes of the warp must call together, converged; inactive lanes only lend
// their loads.  Results equal the per-thread searches'.  For a stream of
// independent probes the per-thread searches are the faster form on GB300 (a
// warp keeps 32 searches in flight instead of 32 / 2^kDegree); these serve
// code written against the reference's cooperative calls.
// ---------------------------------------------------------------------------
GJ_DEVICE_INLINE uint32_t lane_index() {
    uint32_t l;
    asm("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

template <unsigned kDegree>
GJ_DEVICE_INLINE uint32_t group_mask_of(uint32_t first) {
    return kDegree >= 5 ? 0xffffffffu : (((1u << (1u << kDegree)) - 1u) << first);
}

// Lower bound of x in arr[0, size) (size if every key is below x) by a
// (G + 1)-ary search, G = 2^kDegree: each round the G lanes test the G
// pivots lo + (i + 1) * len / (G + 1) of the candidate range [lo, hi], and
// the number of pivots below x selects one of the G + 1 parts (the keys are
// sorted, so the tests below x are a prefix of the lanes); a range of at most
// G positions is finished in one last round.  log_{G+1}(size) + 1 rounds.
template <unsigned kDegree = 4>
GJ_DEVICE_INLINE uint64_t cooperative_lower_bound(bool active, uint64_t x, const uint64_t* arr, uint64_t size) {
    static_assert(kDegree >= 1 && kDegree <= 5, "groups of 2 to 32 lanes");
    constexpr uint32_t G = 1u << kDegree;
    const uint32_t lane = lane_index();
    const uint32_t first = lane & ~(G - 1u), me = lane - first;
    const uint32_t mask = group_mask_of<kDegree>(first);
    uint64_t result = size;
    for (uint32_t s = 0; s < G; ++s) {
        const uint32_t leader = first + s;
        if (!__shfl_sync(mask, active ? 1 : 0, leader)) continue;  // the same answer on every lane of the group
        const uint64_t lx = __shfl_sync(mask, (unsigned long long)x, leader);
        const uint64_t* la =
            reinterpret_cast<const uint64_t*>(__shfl_sync(mask, (unsigned long long)(uintptr_t)arr, leader));
        uint64_t lo = 0, hi = __shfl_sync(mask, (unsigned long long)size, leader);
        while (hi - lo > G) {
            // the answer lies in [lo, hi]; pivot i = lo + (i + 1) * len / (G + 1)
            const uint64_t len = hi - lo, lo0 = lo;
            const uint64_t p = lo0 + (uint64_t)(me + 1) * len / (G + 1);
            const uint32_t below = __popc(__ballot_sync(mask, ld_ro(la + p) < lx));
            // pivots 0 .. below - 1 are below x, pivot `below` (if any) is not
            if (below > 0) lo = lo0 + (uint64_t)below * len / (G + 1) + 1;
            if (below < G) hi = lo0 + (uint64_t)(below + 1) * len / (G + 1);
        }
        const uint64_t p = lo + me;
        const uint32_t below = __popc(__ballot_sync(mask, p < hi && ld_ro(la + p) < lx));
        if (lane == leader) result = lo + below;
    }
    return active ? result : size;
}

// Where the descents of lo and hi (lo <= hi) part: the deepest node both
// pass, as (node | level << 56) -- level d means the node is searched at
// loop level d, depth means it is the leaf node.  Every key in [lo, hi]
// passes through it (the descent is monotonic in the key).
GJ_DEVICE_INLINE uint64_t harmonia_common_node(const harmonia_view& v, uint64_t lo, uint64_t hi) {
    constexpr uint32_t K = kHarmoniaKeys;
    uint64_t pos = 0;
    uint32_t d = 1;
    for (; d < v.depth; ++d) {
        bool eq;
        const uint64_t* node = v.keys + pos * K;
        const uint32_t a = (uint32_t)lower_bound_sectors(node, K, 0, K, lo, true, &eq);
        const uint32_t b = (uint32_t)lower_bound_sectors(node, K, 0, K, hi, true, &eq);
        if (a != b) break;
        pos = ld_ro(v.children + pos) + a;
    }
    return pos | ((uint64_t)d << 56);
}

// Harmonia lookup (exact match, as harmonia_lookup) with a group of
// 2^kDegree lanes per node: each lane reads a 32 / 2^kDegree-key slice of the
// 32-key node and the group sums the counts of keys below the probe (the
// node's lower bound, one round of loads per level instead of about three
// dependent sector loads).
template <unsigned kDegree = 4>
GJ_DEVICE_INLINE uint32_t harmonia_lookup_cooperative(bool active, const harmonia_view& v, uint64_t key) {
    static_assert(kDegree >= 1 && kDegree <= 5, "groups of 2 to 32 lanes");
    constexpr uint32_t G = 1u << kDegree, kSlice = kHarmoniaKeys / G;
    const uint32_t lane = lane_index();
    const uint32_t first = lane & ~(G - 1u), me = lane - first;
    const uint32_t mask = group_mask_of<kDegree>(first);
    uint32_t result = kInvalid;
    for (uint32_t s = 0; s < G; ++s) {
        const uint32_t leader = first + s;
        if (!__shfl_sync(mask, active ? 1 : 0, leader)) continue;
        const uint64_t lx = __shfl_sync(mask, (unsigned long long)key, leader);
        uint64_t pos = 0;
        for (uint32_t d = 1; d < v.depth; ++d) {
            const uint64_t* node = v.keys + pos * kHarmoniaKeys + me * kSlice;
            uint32_t c = 0;
#pragma unroll
            for (uint32_t j = 0; j < kSlice; ++j) c += ld_ro(node + j) < lx ? 1u : 0u;
            const uint32_t lb = __reduce_add_sync(mask, c);
            pos = ld_ro(v.children + pos) + lb;
        }
        // leaf level: node pos covers column [32 * pos - inner_size, +32)
        const uint64_t leaf_first = (v.depth > 1) ? (pos * kHarmoniaKeys - v.inner_size) : 0;
        const uint64_t* leaf = v.col + leaf_first + me * kSlice;
        uint32_t c = 0;
        bool eq = false;
#pragma unroll
        for (uint32_t j = 0; j < kSlice; ++j) {
            const bool in = leaf_first + me * kSlice + j < v.n;
            const uint64_t k = in ? ld_ro(leaf + j) : ~0ull;
            c += in && k < lx ? 1u : 0u;
            eq |= in && k == lx;
        }
        const uint32_t lb = __reduce_add_sync(mask, c);
        const bool found = __ballot_sync(mask, eq) != 0;
        if (lane == leader && found) result = (uint32_t)(leaf_first + lb);
    }
    return active ? result : kInvalid;
}

// ---------------------------------------------------------------------------
// RadixSpline (src/rs.cuh:118-154, window src/indexes.cuh:205-215)
// ---------------------------------------------------------------------------
// A spline point (src/rs.cuh:22-52: Coord{x, y}) with the slope of the
// segment to the next point, computed at build with the same double
// division the estimate would make: one 32-byte sector, one load per segment.
struct rs_point {
    uint64_t x;
    double y;
    double slope;  // (y[i+1] - y[i]) / (x[i+1] - x[i]); 0 for the last point
    uint64_t pad;
};
static_assert(sizeof(rs_point) == 32, "a spline point is one sector");

struct rs_view {
    const uint64_t* col;
    uint64_t n;
    const uint32_t* table;   // (1 << radix_bits) + 2 entries
    const rs_point* pts;     // spline points, 32-byte aligned
    uint64_t min_key, max_key;
    uint32_t shift;
    uint32_t max_error;
    uint32_t col_aligned;    // column base is 32-byte aligned
    uint32_t pad;
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
        if (ld_ro(&v.pts[mid].x) < key) {
            lo = mid + 1;
            cnt -= step + 1;
        } else {
            cnt = step;
        }
    }
    // segment [lo - 1, lo]: its left point and precomputed slope
    uint64_t w[4];
    ld_sector(reinterpret_cast<const uint64_t*>(v.pts + lo - 1), w);
    return __dadd_rn(__dmul_rn((double)(key - w[0]), __longlong_as_double((long long)w[2])),
                     __longlong_as_double((long long)w[1]));
}

// lower bound inside [b, e), widened to the whole column when the window
// does not bracket it (possible only for keys outside the column)
template <bool kScattered = true>
GJ_DEVICE_INLINE uint64_t window_lower_bound(const uint64_t* col, uint64_t n, uint64_t b, uint64_t e, uint64_t key,
                                             bool aligned) {
    bool eq;
    uint64_t pos = lower_bound_sectors<kScattered ? kL2Stream : kL2Default>(col, n, b, e, key, aligned, &eq);
    if ((pos == b && b > 0 && ld_ro(col + b - 1) >= key) || (pos == e && e < n && ld_ro(col + e) < key))
        pos = lower_bound_sectors(col, n, 0, n, key, aligned, &eq);
    return pos;
}

template <bool kScattered = true>
GJ_DEVICE_INLINE uint32_t rs_lookup(const rs_view& v, uint64_t key) {
    const double est = rs_estimate(v, key);
    const double err = (double)v.max_error;
    uint64_t b = est < err ? 0 : (uint64_t)(est - err);
    uint64_t e = (est + err + 2 > (double)v.n) ? v.n : (uint64_t)(est + err + 2);
    if (b > e) b = e;
    const uint64_t pos = window_lower_bound<kScattered>(v.col, v.n, b, e, key, v.col_aligned);
    return pos < v.n ? (uint32_t)pos : kInvalid;
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
// that window; the window check then falls back to a search of the whole
// column, so the result is always the exact lower bound.
struct learned_leaf {
    uint64_t x0;      // reference key of the leaf (smallest routed key)
    uint32_t base;    // position of x0
    float slope;      // positions per unit key distance
    uint32_t err_lo;
    uint32_t err_hi;
    uint64_t pad;     // one 32-byte sector per leaf: a single load
};
static_assert(sizeof(learned_leaf) == 32, "a leaf is one sector");

// The root MLP is stored 32 wide: 1 -> 32 -> 32 -> 1 with ReLU over
// [W1(32) b1(32) W2(32x32, out-major) b2(32) W3(32) b3].  Narrower trained
// networks are stored zero-padded; the padding adds exact zeros, so the
// result is the narrower network's, and one of at most 16 units is
// evaluated over its first 16 lanes only.
constexpr int kMlpWidth = 32;
constexpr int kMlpParams = 2 * kMlpWidth + kMlpWidth * kMlpWidth + 2 * kMlpWidth + 1;  // 1153

struct learned_view {
    const uint64_t* col;
    uint64_t n;
    uint64_t min_key, max_key;
    float inv_range;            // 1 / (max_key - min_key) (0 if the range is empty)
    uint32_t num_leaves;
    uint32_t root_kind;         // GJ_LEARNED_ROOT_LINEAR, _MLP or _SEGMENTS
    uint32_t hidden;            // trained MLP width H (<= 32), stored padded to 32
    const float* root;          // [a, b] (linear), kMlpParams MLP parameters or
                                // the segment table ({y, dy} per segment)
    const learned_leaf* leaves; // 32-byte aligned
    uint32_t col_aligned;       // column base is 32-byte aligned
    uint32_t segments;          // segment-table root: number of segments
};

// segments of the segment-table root (a 32 KB table: it stays in L1)
constexpr uint32_t kLearnedSegments = 4096;

// root parameters carried by value (a kernel argument): the forward pass then
// reads its weights as constant-bank operands of its FMAs
struct alignas(8) learned_root_params {
    float w[kMlpParams];
};

// two fused multiply-adds in one instruction (each lane rounds like fmaf)
GJ_DEVICE_INLINE float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// The lookup's root function.  Layer 2 sums even and odd inputs in two lanes
// of packed FMAs (out = b2 + even + odd), half the instructions of a scalar
// chain; the build routes keys with this same function, so the recorded
// error windows hold for it.  P must be 8-byte aligned.
template <int H>
GJ_DEVICE_INLINE float mlp_forward(const float* P, float x) {
    // H: evaluated width (16 or 32) over the 32-wide stored layout; for a
    // network of at most 16 units the lanes 16..31 are exact zeros, so both
    // widths give the same result and the 16-wide one a quarter of layer 2
    constexpr int W = kMlpWidth;
    const float2* W1 = reinterpret_cast<const float2*>(P);
    const float2* b1 = reinterpret_cast<const float2*>(P + W);
    float2 h1[H / 2];
#pragma unroll
    for (int j = 0; j < H / 2; ++j) {
        const float2 a = fma2(W1[j], make_float2(x, x), b1[j]);
        h1[j] = make_float2(a.x > 0.f ? a.x : 0.f, a.y > 0.f ? a.y : 0.f);
    }
    float out = P[4 * W + W * W];  // b3
#pragma unroll
    for (int o = 0; o < H; ++o) {
        const float2* w = reinterpret_cast<const float2*>(P + 2 * W + o * W);
        float2 s = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < H / 2; ++j) s = fma2(w[j], h1[j], s);
        const float a = P[2 * W + W * W + o] + s.x + s.y;  // b2[o] + even + odd
        out = fmaf(P[3 * W + W * W + o], a > 0.f ? a : 0.f, out);
    }
    return out;
}

GJ_DEVICE_INLINE float learned_norm(const learned_view& v, uint64_t key) {
    if (key <= v.min_key) return 0.f;
    if (key >= v.max_key) return 1.f;
    return (float)(key - v.min_key) * v.inv_range;
}

// The segment-table root is r(x) = y[i] + (xS - i) * dy[i] with i = floor(xS)
// over S equal-width segments of the normalised key, y[i] the fraction of keys
// below segment i's first key: the key CDF, exact at every segment end and
// linear in between.  It reads the table from global memory (v.root), not
// from `root`, which holds the by-value parameters of the other kinds.
GJ_DEVICE_INLINE uint32_t learned_route(const learned_view& v, const float* root, float x) {
    float r;
    if (v.root_kind == GJ_LEARNED_ROOT_SEGMENTS) {
        const float t = x * (float)v.segments;
        const uint32_t i = min((uint32_t)t, v.segments - 1);
        const float2 s = __ldg(reinterpret_cast<const float2*>(v.root) + i);
        r = fmaf(t - (float)i, s.y, s.x);
    } else if (v.root_kind == GJ_LEARNED_ROOT_MLP)
        r = v.hidden <= 16 ? mlp_forward<16>(root, x) : mlp_forward<32>(root, x);
    else
        r = fmaf(root[0], x, root[1]);
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

template <bool kScattered = true>
GJ_DEVICE_INLINE uint32_t learned_lookup(const learned_view& v, const float* root, uint64_t key) {
    const uint32_t li = learned_route(v, root, learned_norm(v, key));
    uint64_t w[4];
    ld_sector_c<kScattered ? kL2Keep : kL2Default>(reinterpret_cast<const uint64_t*>(v.leaves + li), w);
    learned_leaf lf;
    lf.x0 = w[0];
    lf.base = (uint32_t)w[1];
    lf.slope = __uint_as_float((uint32_t)(w[1] >> 32));
    lf.err_lo = (uint32_t)w[2];
    lf.err_hi = (uint32_t)(w[2] >> 32);
    const int64_t pred = learned_predict(lf, key);
    const int64_t n = (int64_t)v.n;
    // window [pred - err_lo, pred + err_hi + 1) clamped to [0, n]; a probe far
    // outside the leaf's keys can push both ends below 0 or above n
    int64_t lo = pred - (int64_t)lf.err_lo;
    int64_t hi = pred + (int64_t)lf.err_hi + 1;
    lo = lo < 0 ? 0 : (lo > n ? n : lo);
    hi = hi < 0 ? 0 : (hi > n ? n : hi);
    if (lo > hi) lo = hi;
    const uint64_t pos = window_lower_bound<kScattered>(v.col, v.n, (uint64_t)lo, (uint64_t)hi, key, v.col_aligned);
    return pos < v.n ? (uint32_t)pos : kInvalid;
}

}  // namespace gj
