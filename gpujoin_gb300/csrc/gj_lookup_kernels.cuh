// gj_lookup_kernels.cuh -- the probe kernels and their launchers, shared by
// the translation units that instantiate them: each index kind (and B+tree
// node width) is compiled in one unit (gj_lookup*.cu), so the units build in
// parallel.  Everything but the call interface has internal linkage.
//
// Replaces lookup_kernel (src/index_lookup_common.cuh:217-245),
// partitioned_lookup_kernel (src/index_lookup_partitioning.cu:218-248) and
// ij_lookup_kernel (src/tpch/tpch_14_ij.cu:371-407).
//
// Each kernel stages the upper part of the index (B+tree top levels,
// Harmonia top nodes, the sampled binary-search keys) into shared memory once
// per block.  Probe keys are streamed with evict-first loads, results with
// streaming stores.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <type_traits>
#include <utility>

#include "gj_internal.h"

namespace gj {

// one launch of a probe kernel for an index, as passed between the units
enum class lookup_action { positions, scatter, pairs, sorted_pairs, sorted_positions };
struct lookup_call {
    lookup_action action;
    const uint64_t* keys;  // probes, or the keys of a partitioned relation
    const uint32_t* rows;  // row ids (partitioned relation) or null
    uint64_t m;
    uint32_t* out;         // positions (positions, scatter) or pairs
    const uint64_t* d_base;
    uint64_t* d_count;
    void* ws;
    size_t ws_bytes;
    uint32_t* stash;       // pairs: two-pass positions buffer, or null
    cudaStream_t s;
    // test hook of the bounded waits (gj_debug_inlj_pairs_stalled): a spin
    // limit other than kSpinLimit (0 = default) and a first tile left
    // unclaimed, so that every look-back runs out
    uint32_t spin_limit;
    bool skip_first_tile;
    // pairs (single pass): tiles placed by one atomicAdd each instead of in
    // probe order
    bool unordered;
};

// per-kind entry points, each defined in one unit
int lookup_call_bs(const gj_index* idx, const lookup_call& c);
int lookup_call_noop(const gj_index* idx, const lookup_call& c);
int lookup_call_harmonia(const gj_index* idx, const lookup_call& c);
int lookup_call_rs(const gj_index* idx, const lookup_call& c);
int lookup_call_learned(const gj_index* idx, const lookup_call& c);
int lookup_call_hash(const gj_index* idx, const lookup_call& c);
template <int W>
int lookup_call_btree(const gj_index* idx, const lookup_call& c);  // the widths of btree_dispatch:
template <> int lookup_call_btree<4>(const gj_index* idx, const lookup_call& c);
template <> int lookup_call_btree<7>(const gj_index* idx, const lookup_call& c);
template <> int lookup_call_btree<8>(const gj_index* idx, const lookup_call& c);
template <> int lookup_call_btree<15>(const gj_index* idx, const lookup_call& c);
template <> int lookup_call_btree<16>(const gj_index* idx, const lookup_call& c);
template <> int lookup_call_btree<32>(const gj_index* idx, const lookup_call& c);
template <> int lookup_call_btree<64>(const gj_index* idx, const lookup_call& c);

namespace {


constexpr int kBlock = 256;
// Resident blocks per SM each lookup kernel is compiled for: the register
// cap.  A search is a chain of dependent loads and the warps of an SM are
// what keeps loads in flight, so the tree and search kinds are capped at 32
// registers (8 blocks of 256 threads, full occupancy), which they meet
// without spilling; the learned index keeps 64 for its MLP root.
// GJ_MIN_BLOCKS overrides every kind (tuning builds).
#ifdef GJ_MIN_BLOCKS
#define GJ_BLOCKS(n) GJ_MIN_BLOCKS
#else
#define GJ_BLOCKS(n) (n)
#endif

// ---------------------------------------------------------------------------
// per-index lookup functors
// ---------------------------------------------------------------------------
struct stage_desc {
    const uint64_t* src0;
    const uint64_t* src1;
    uint32_t words0;
    uint32_t words1;
};

// Each op searches one probe.  lookup<kScattered> picks the L2 classes:
// scattered probes (operator()) keep the inner levels and stream the
// column; the partitioned kernels, whose nearby probes reuse column sectors
// and touch a slice of the tree, use the default class.
struct op_bs {
    static constexpr int kMinBlocks = GJ_BLOCKS(8);
    bs_view v;
    template <bool kScattered = true>
    __device__ __forceinline__ uint32_t lookup(const uint64_t* cache, uint64_t key) const {
        return bs_lookup(v, cache, key);
    }
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const { return lookup(cache, key); }
};
// Sorted tiles: an op with a tile_hint searches once per tile for what all
// keys of the tile's range share (for the B+tree: the deepest node on every
// path) and starts each probe's search there.
template <int W>
struct op_btree {
    static constexpr int kMinBlocks = GJ_BLOCKS(8);
    btree_view v;
    template <bool kScattered = true>
    __device__ __forceinline__ uint32_t lookup(const uint64_t* cache, uint64_t key) const {
        return btree_lookup<W, kScattered>(v, cache, key);
    }
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const { return lookup(cache, key); }
    using tile_hint = btree_cursor;
    __device__ __forceinline__ tile_hint tile(const uint64_t* cache, uint64_t lo, uint64_t hi) const {
        return btree_common_node<W, false>(v, cache, lo, hi);
    }
    __device__ __forceinline__ uint32_t lookup_in_tile(const uint64_t* cache, uint64_t key, const tile_hint& h) const {
        return btree_lookup_from<W, false>(v, cache, key, h);
    }
};

struct no_tile_hint {};
template <class Op, class = void>
struct tile_hint_of {
    using type = no_tile_hint;
};
template <class Op>
struct tile_hint_of<Op, std::void_t<typename Op::tile_hint>> {
    using type = typename Op::tile_hint;
};
struct op_harmonia {
    static constexpr int kMinBlocks = GJ_BLOCKS(8);
    harmonia_view v;
    template <bool kScattered = true>
    __device__ __forceinline__ uint32_t lookup(const uint64_t* cache, uint64_t key) const {
        return harmonia_lookup<kScattered>(v, cache, key);
    }
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const { return lookup(cache, key); }
};
struct op_rs {
    static constexpr int kMinBlocks = GJ_BLOCKS(8);
    rs_view v;
    template <bool kScattered = true>
    __device__ __forceinline__ uint32_t lookup(const uint64_t*, uint64_t key) const {
        return rs_lookup<kScattered>(v, key);
    }
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const { return lookup(cache, key); }
};
struct op_hash {
    static constexpr int kMinBlocks = GJ_BLOCKS(8);
    hash_view v;
    template <bool kScattered = true>
    __device__ __forceinline__ uint32_t lookup(const uint64_t*, uint64_t key) const {
        return hash_lookup(v, key);
    }
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const { return lookup(cache, key); }
};
struct op_noop {
    static constexpr int kMinBlocks = GJ_BLOCKS(8);
    template <bool kScattered = true>
    __device__ __forceinline__ uint32_t lookup(const uint64_t*, uint64_t) const { return kInvalid; }
    __device__ __forceinline__ uint32_t operator()(const uint64_t*, uint64_t) const { return kInvalid; }
};
// the root parameters travel inside the op (a kernel argument): the MLP's
// FMAs read their weights from the constant bank
struct op_learned {
    static constexpr int kMinBlocks = GJ_BLOCKS(4);
    learned_view v;
    learned_root_params p;
    template <bool kScattered = true>
    __device__ __forceinline__ uint32_t lookup(const uint64_t*, uint64_t key) const {
        return learned_lookup<kScattered>(v, p.w, key);
    }
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const { return lookup(cache, key); }
};

__device__ __forceinline__ void stage_cache(uint64_t* dst, const stage_desc& sd) {
    for (uint32_t i = threadIdx.x; i < sd.words0; i += blockDim.x) dst[i] = __ldg(reinterpret_cast<const unsigned long long*>(sd.src0) + i);
    for (uint32_t i = threadIdx.x; i < sd.words1; i += blockDim.x)
        dst[sd.words0 + i] = __ldg(reinterpret_cast<const unsigned long long*>(sd.src1) + i);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// plain lookup: out[i] = lookup(probes[i])
// ---------------------------------------------------------------------------
// One block per tile of kLookupItems * kBlock probes (item k of thread t is
// probe tile + k * kBlock + t: coalesced).  The grid is not persistent: the
// hardware hands tiles to SMs as they free up, which balances SMs that run
// at different speeds (near and far HBM of the two dies) without a counter.
// A thread searches its probes one after another (a search is a chain of
// dependent loads; occupancy, not per-thread interleaving, keeps many loads
// in flight) and loads the next probe key before it searches the current
// one.  No per-thread arrays: the search runs with few live registers.
#ifndef GJ_LOOKUP_ITEMS
#define GJ_LOOKUP_ITEMS 8
#endif
constexpr int kLookupItems = GJ_LOOKUP_ITEMS;
constexpr uint32_t kLookupTile = kBlock * kLookupItems;

__device__ __forceinline__ uint64_t load_probe(const uint64_t* p, uint64_t i, uint64_t m) {
    return i < m ? __ldcs(reinterpret_cast<const unsigned long long*>(p + i)) : 0ull;
}

template <class Op>
__global__ void __launch_bounds__(kBlock, Op::kMinBlocks) k_lookup(const __grid_constant__ Op op, const stage_desc sd,
                                                   const uint64_t* __restrict__ probes, uint64_t m,
                                                   uint32_t* __restrict__ out) {
    extern __shared__ __align__(16) uint64_t cache[];
    stage_cache(cache, sd);
    const uint64_t t0 = (uint64_t)blockIdx.x * kLookupTile + threadIdx.x;
    uint64_t next = load_probe(probes, t0, m);
#pragma unroll 1
    for (int k = 0; k < kLookupItems; ++k) {
        const uint64_t i = t0 + (uint64_t)k * kBlock;
        if (i >= m) break;
        const uint64_t key = next;
        if (k + 1 < kLookupItems) next = load_probe(probes, i + kBlock, m);
        __stcs(out + i, op(cache, key));
    }
}

// scattered lookup over a partitioned relation: out[rows[i]] = lookup(keys[i])
template <class Op>
__global__ void __launch_bounds__(kBlock, Op::kMinBlocks) k_scatter_lookup(const __grid_constant__ Op op, const stage_desc sd,
                                                           const uint64_t* __restrict__ keys,
                                                           const uint32_t* __restrict__ rows, uint64_t m,
                                                           uint32_t* __restrict__ out) {
    extern __shared__ __align__(16) uint64_t cache[];
    stage_cache(cache, sd);
    const uint64_t t0 = (uint64_t)blockIdx.x * kLookupTile + threadIdx.x;
    uint64_t next = load_probe(keys, t0, m);
#pragma unroll 1
    for (int k = 0; k < kLookupItems; ++k) {
        const uint64_t i = t0 + (uint64_t)k * kBlock;
        if (i >= m) break;
        const uint64_t key = next;
        if (k + 1 < kLookupItems) next = load_probe(keys, i + kBlock, m);
        const uint32_t r = op.template lookup<false>(cache, key);
        out[__ldcs(rows + i)] = r;
    }
}

// ---------------------------------------------------------------------------
// join pairs with decoupled look-back compaction
// ---------------------------------------------------------------------------
// Pairs are emitted in probe order.  Tiles of kBlock * items probes are
// claimed in order through an atomic counter, so every predecessor of a tile
// is already running when the tile looks back: each wait ends.  Waits are
// bounded anyway; on expiry the kernel raises the error flag (GJ_ERR_TIMEOUT
// on the host) and stops writing.
//
// Plain probes take two passes: k_lookup writes the positions to the upper
// half of the pairs buffer (the caller provides 2m u32), then
// k_compact_pairs turns them into pairs.  The search pass has no block
// barriers, and the compaction is a streaming pass.  Probes of a partitioned
// relation (row ids, appended behind *d_base) take the single-pass k_pairs.
// k_pairs items per thread (8 measured fastest for gj_inlj_pairs_host, whose
// tiles read their probes from and write their pairs to host memory: 15.2 ms
// per 2^28 probes, against 18.7 with 4 and 21.4 with 16); GJ_PAIRS_ITEMS
// overrides it in tuning builds
#ifndef GJ_PAIRS_ITEMS
#define GJ_PAIRS_ITEMS GJ_LOOKUP_ITEMS
#endif
constexpr int kItems = GJ_PAIRS_ITEMS;
constexpr int kCompactItems = 16;                // k_compact_pairs items per thread
static_assert(kItems >= 4 && (kItems & (kItems - 1)) == 0, "the pairs scan needs a power-of-two item count >= 4");
constexpr uint32_t kTile = kBlock * kItems;
// the workspace holds one state per kStateTile probes: enough for the
// smallest tile of any pairs kernel, at the same offsets for all of them
constexpr uint32_t kStateTile = kBlock * 4;
constexpr uint32_t kCompactTile = kBlock * kCompactItems;
constexpr unsigned long long kFlagAggregate = 1ull << 62;
constexpr unsigned long long kFlagPrefix = 2ull << 62;
constexpr unsigned long long kValueMask = (1ull << 62) - 1;
constexpr uint32_t kSpinLimit = 1u << 22;

struct pairs_ws {
    unsigned long long* tile_state;  // num_tiles
    unsigned int* tile_counter;      // 1
    unsigned int* error;             // 1
    unsigned long long* totals;      // 2: pairs placed and tiles done (unordered pairs)
    uint32_t spin_limit;             // polls before a look-back gives up
};

// the workspace layout of every pairs kernel; false when it is too small
inline bool carve_pairs_ws(void* ws, size_t ws_bytes, uint64_t m, pairs_ws* pw, size_t* used) {
    const uint64_t states = (m + kStateTile - 1) / kStateTile;
    workspace_carver wc(ws, ws_bytes);
    pw->tile_state = wc.take<unsigned long long>(states ? states : 1);
    pw->tile_counter = wc.take<unsigned int>(2);
    pw->error = pw->tile_counter ? pw->tile_counter + 1 : nullptr;
    pw->totals = wc.take<unsigned long long>(2);
    pw->spin_limit = kSpinLimit;
    *used = wc.used;
    return pw->tile_state && pw->tile_counter && pw->totals;
}

// Exclusive prefix of tile `tile` (> 0) from the states of its predecessors,
// read 32 at a time by the calling warp: lane i reads tile j - i, and the
// window is summed up to its nearest published prefix.  Returns false when
// the wait ran out.
__device__ __forceinline__ bool look_back(const pairs_ws& ws, uint32_t tile, uint32_t lane,
                                          unsigned long long* prefix_out) {
    unsigned long long prefix = 0;
    int64_t j = (int64_t)tile - 1;
    uint32_t spins = 0;
    for (;;) {
        const int64_t idx = j - (int64_t)lane;
        const unsigned long long st =
            idx >= 0 ? *reinterpret_cast<volatile unsigned long long*>(&ws.tile_state[idx]) : (kFlagPrefix | 0ull);
        const unsigned long long flag = st & ~kValueMask;
        const uint32_t not_ready = __ballot_sync(0xffffffffu, flag == 0);
        const uint32_t has_prefix = __ballot_sync(0xffffffffu, flag == kFlagPrefix);
        // lanes up to (and including) the nearest prefix must all be published
        const uint32_t need = has_prefix ? (2u << (__ffs(has_prefix) - 1)) - 1u : 0xffffffffu;
        if (not_ready & need) {
            if (++spins > ws.spin_limit) return false;
            continue;
        }
        unsigned long long v = ((need >> lane) & 1u) ? (st & kValueMask) : 0ull;
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
        prefix += v;
        if (has_prefix) break;
        j -= 32;
    }
    *prefix_out = prefix;
    return true;
}

// One block-tile of the ordered compaction: fill(t0, s_pos) writes the
// result of tile item j into s_pos[j] (kInvalid for no pair) for the tile's
// kBlock * kIt items; the block then emits the pairs of the tile, in item
// order, at the tile's prefix.  row_of(k, i) is the probe row of item k of
// the calling thread (i = t0 + k * kBlock + thread).  Returns false when the
// kernel must stop (look-back timed out).  Unordered (kOrdered false), the
// tile's place comes from one atomicAdd instead of the look-back -- tiles
// in the order they finish, as the reference's join kernels place their
// pairs (src/tpch/tpch_14_ij.cu:371-407) -- and the last tile to finish
// writes the count.
template <int kIt, bool kOrdered = true, class Fill, class RowOf>
__device__ __forceinline__ bool pairs_tile(Fill&& fill, RowOf&& row_of, uint32_t tile, uint2* pairs, uint64_t base,
                                           uint64_t* __restrict__ d_count, const pairs_ws& ws, uint32_t num_tiles) {
    constexpr int kWarps = kBlock / 32;
    constexpr uint32_t kT = kBlock * kIt;
    __shared__ uint32_t s_cnt[kIt * kWarps];
    __shared__ uint32_t s_ballot[kIt * kWarps];
    __shared__ uint32_t s_pos[kT];
    __shared__ unsigned long long s_prefix;
    __shared__ int s_abort;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t t0 = (uint64_t)tile * kT;
    // item k of thread t is probe t0 + k * kBlock + t; output order is probe
    // order, i.e. (k, warp, lane) order
    fill(t0, s_pos);
    uint32_t flags = 0;
#pragma unroll
    for (int k = 0; k < kIt; ++k) {
        const bool hit = s_pos[k * kBlock + threadIdx.x] != kInvalid;
        const uint32_t ballot = __ballot_sync(0xffffffffu, hit);
        if (hit) flags |= 1u << k;
        if (lane == 0) {
            s_cnt[k * kWarps + warp] = __popc(ballot);
            s_ballot[k * kWarps + warp] = ballot;
        }
    }
    __syncthreads();
    if (warp == 0) {
        // exclusive scan of the kIt * kWarps counts in (k, warp) order
        constexpr int kPerLane = kIt * kWarps / 32;
        uint32_t v[kPerLane];
        uint32_t sum = 0;
#pragma unroll
        for (int j = 0; j < kPerLane; ++j) {
            v[j] = s_cnt[lane * kPerLane + j];
            sum += v[j];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += t;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (int j = 0; j < kPerLane; ++j) {
            s_cnt[lane * kPerLane + j] = run;
            run += v[j];
        }
        // publish the tile aggregate, then resolve the tile prefix
        const unsigned long long total = __shfl_sync(0xffffffffu, incl, 31);
        unsigned long long prefix = 0;
        bool ok = true;
        if constexpr (!kOrdered) {
            if (lane == 0) {
                prefix = atomicAdd(&ws.totals[0], total);
                __threadfence();  // this tile's total is counted before it counts as done
                if (atomicAdd(&ws.totals[1], 1ull) == (unsigned long long)num_tiles - 1ull) {
                    __threadfence();
                    *d_count = base + atomicAdd(&ws.totals[0], 0ull);
                }
            }
        } else if (tile == 0) {
            if (lane == 0) atomicExch(&ws.tile_state[0], kFlagPrefix | total);
        } else {
            if (lane == 0) atomicExch(&ws.tile_state[tile], kFlagAggregate | total);
            ok = look_back(ws, tile, lane, &prefix);
            if (lane == 0) {
                if (ok)
                    atomicExch(&ws.tile_state[tile], kFlagPrefix | (prefix + total));
                else
                    atomicExch(ws.error, 1u);
            }
        }
        if (lane == 0) {
            s_abort = ok ? 0 : 1;
            s_prefix = prefix;
            if (kOrdered && ok && tile == num_tiles - 1) *d_count = base + prefix + total;
        }
    }
    __syncthreads();
    if (s_abort) return false;
    const uint64_t tile_base = base + s_prefix;
#pragma unroll
    for (int k = 0; k < kIt; ++k) {
        if (flags & (1u << k)) {
            const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
            const uint32_t rank = __popc(s_ballot[k * kWarps + warp] & ((1u << lane) - 1u));
            const uint64_t o = tile_base + s_cnt[k * kWarps + warp] + rank;
            const uint32_t row = row_of(k, i);
            const uint32_t pos = s_pos[k * kBlock + threadIdx.x];
            __stcs(reinterpret_cast<unsigned long long*>(pairs + o), ((unsigned long long)pos << 32) | row);
        }
    }
    __syncthreads();
    return true;
}

__device__ __forceinline__ uint32_t claim_tile(const pairs_ws& ws) {
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(ws.tile_counter, 1u);
    __syncthreads();
    return s_tile;
}


// single pass: search and compact tile by tile (partitioned relations, whose
// pairs are appended behind *d_base)
template <class Op, bool kOrdered>
__global__ void __launch_bounds__(kBlock, Op::kMinBlocks) k_pairs(const __grid_constant__ Op op, const stage_desc sd, const uint64_t* __restrict__ probes,
                                                  const uint32_t* __restrict__ rows, uint64_t m,
                                                  uint2* __restrict__ pairs, const uint64_t* __restrict__ d_base,
                                                  uint64_t* __restrict__ d_count, pairs_ws ws, uint32_t num_tiles) {
    extern __shared__ __align__(16) uint64_t cache[];
    stage_cache(cache, sd);
    const uint64_t base = d_base ? *d_base : 0ull;
    auto search = [&](uint64_t t0, uint32_t* s_pos) {
        uint64_t next = load_probe(probes, t0 + threadIdx.x, m);
#pragma unroll 1
        for (int k = 0; k < kItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
            const uint64_t key = next;
            if (k + 1 < kItems) next = load_probe(probes, i + kBlock, m);
            s_pos[k * kBlock + threadIdx.x] = i < m ? op(cache, key) : kInvalid;
        }
    };
    auto row_of = [&](int, uint64_t i) { return rows ? __ldcs(rows + i) : (uint32_t)i; };
    for (;;) {
        const uint32_t tile = claim_tile(ws);
        if (tile >= num_tiles) break;
        if (!pairs_tile<kItems, kOrdered>(search, row_of, tile, pairs, base, d_count, ws, num_tiles)) break;
    }
}

// Second pass of the two-pass pairs: compact the positions k_lookup wrote
// to the stash into pairs at *d_base + (rank of the match).  The stash lies
// inside the pairs buffer, placed so that the u32 words of pair o only reach
// stash entries j <= o: a tile writes pairs only after every earlier tile
// has published its count, i.e. after every earlier tile has read its
// positions, so no position is overwritten before it is read.  (stash and
// pairs alias, so neither is __restrict__.)
__global__ void __launch_bounds__(kBlock) k_compact_pairs(const uint32_t* stash, const uint32_t* __restrict__ rows,
                                                          uint64_t m, uint2* pairs,
                                                          const uint64_t* __restrict__ d_base,
                                                          uint64_t* __restrict__ d_count, pairs_ws ws,
                                                          uint32_t num_tiles) {
    const uint64_t base = d_base ? *d_base : 0ull;
    auto load = [&](uint64_t t0, uint32_t* s_pos) {
#pragma unroll
        for (int k = 0; k < kCompactItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
            s_pos[k * kBlock + threadIdx.x] = i < m ? __ldcs(stash + i) : kInvalid;
        }
    };
    for (;;) {
        const uint32_t tile = claim_tile(ws);
        if (tile >= num_tiles) break;
        auto row_of = [&](int, uint64_t i) { return rows ? __ldcs(rows + i) : (uint32_t)i; };
        if (!pairs_tile<kCompactItems>(load, row_of, tile, pairs, base, d_count, ws, num_tiles)) break;
    }
}

// Pairs of a partitioned relation (probes grouped by key range, rows
// attached).  Each tile of kTile probes is first sorted by key in shared
// memory -- a counting sort over kSortBuckets equal-width buckets of the
// tile's key range -- and then searched in that order: neighbouring lanes
// follow the same path through the upper index levels, and a warp-wide load
// of one sector serves all lanes that ask for it.  Pairs leave in tile order
// (sorted within a tile, in the relation's order across tiles); the order of
// equal-bucket keys inside a tile is not fixed.
constexpr int kSortItems = 4;                        // probes per thread and tile
constexpr uint32_t kSortTile = kBlock * kSortItems;  // 1024
constexpr uint32_t kSortBuckets = kSortTile;
static_assert(kStateTile <= kSortTile && kStateTile <= kTile && kStateTile <= kCompactTile,
              "the workspace needs a state per tile of every pairs kernel");

__device__ __forceinline__ unsigned bit_length(uint64_t v) { return v ? 64u - (unsigned)__clzll(v) : 0u; }

// Shared memory of one sorted tile (about 21 KB with the kernels' caches).
template <class Hint>
struct sorted_tile_smem {
    static constexpr int kWarps = kBlock / 32;
    uint64_t key[kSortTile];
    uint32_t row[kSortTile];
    __align__(16) uint32_t bucket[kSortBuckets];  // read as uint4
    unsigned long long lo[kWarps], hi[kWarps];
    uint32_t wsum[kWarps];
    Hint hint;
};

// Sorts the tile keys[t0 .. t0 + tn) by key into t.key, with row_of(j) (j =
// item inside the tile) beside each in t.row, and (for an op with a tile
// hint) leaves the hint of the tile's key range in t.hint.  Ends with a
// barrier.  The caller's previous reads of t must be behind a barrier.
template <class Op, class RowOf>
__device__ __forceinline__ void sort_tile(const Op& op, const uint64_t* cache, const uint64_t* __restrict__ keys,
                                          uint64_t t0, uint32_t tn, RowOf&& row_of,
                                          sorted_tile_smem<typename tile_hint_of<Op>::type>& t) {
    constexpr int kWarps = kBlock / 32;
    constexpr bool kHinted = !std::is_same<typename tile_hint_of<Op>::type, no_tile_hint>::value;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t key[kSortItems];
    unsigned long long lo = ~0ull, hi = 0ull;
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t j = k * kBlock + threadIdx.x;
        key[k] = j < tn ? __ldcs(reinterpret_cast<const unsigned long long*>(keys) + t0 + j) : 0ull;
        if (j < tn) {
            lo = key[k] < lo ? key[k] : lo;
            hi = key[k] > hi ? key[k] : hi;
        }
    }
    // key range of the tile
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, d);
        const unsigned long long b = __shfl_xor_sync(0xffffffffu, hi, d);
        lo = a < lo ? a : lo;
        hi = b > hi ? b : hi;
    }
    if (lane == 0) {
        t.lo[warp] = lo;
        t.hi[warp] = hi;
    }
    for (uint32_t b = threadIdx.x; b < kSortBuckets; b += kBlock) t.bucket[b] = 0;
    __syncthreads();
    lo = t.lo[0];
    hi = t.hi[0];
#pragma unroll
    for (int w = 1; w < kWarps; ++w) {
        lo = t.lo[w] < lo ? t.lo[w] : lo;
        hi = t.hi[w] > hi ? t.hi[w] : hi;
    }
    if constexpr (kHinted) {
        if (threadIdx.x == 0) t.hint = op.tile(cache, lo, hi);  // read after the barriers below
    }
    const unsigned used = bit_length(hi - lo);
    constexpr unsigned kBucketBits = 10;  // kSortBuckets = 2^10
    const unsigned sh = used > kBucketBits ? used - kBucketBits : 0;  // (hi - lo) >> sh < kSortBuckets
    // counting sort: ranks inside a bucket from shared-memory atomics
    uint32_t rank[kSortItems];
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t j = k * kBlock + threadIdx.x;
        rank[k] = j < tn ? atomicAdd(&t.bucket[(uint32_t)((key[k] - lo) >> sh)], 1u) : 0u;
    }
    __syncthreads();
    {
        // exclusive scan of the buckets: kSortBuckets / kBlock consecutive per thread
        static_assert(kSortBuckets / kBlock == 4, "one uint4 per thread");
        uint4* sb = reinterpret_cast<uint4*>(t.bucket) + threadIdx.x;
        const uint4 c0 = sb[0];
        const uint32_t sum = c0.x + c0.y + c0.z + c0.w;
        uint32_t incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += v;
        }
        if (lane == 31) t.wsum[warp] = incl;
        __syncthreads();
        uint32_t run = incl - sum;
        for (int w = 0; w < (int)warp; ++w) run += t.wsum[w];
        uint4 o0;
        o0.x = run; run += c0.x;
        o0.y = run; run += c0.y;
        o0.z = run; run += c0.z;
        o0.w = run;
        sb[0] = o0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kSortItems; ++k) {
        const uint32_t j = k * kBlock + threadIdx.x;
        if (j < tn) {
            const uint32_t q = t.bucket[(uint32_t)((key[k] - lo) >> sh)] + rank[k];
            t.key[q] = key[k];
            t.row[q] = row_of(j);
        }
    }
    __syncthreads();
}

// item j of a sorted tile: its search, from the tile's hint when the op has one
template <class Op>
__device__ __forceinline__ uint32_t sorted_lookup(const Op& op, const uint64_t* cache, uint64_t key,
                                                  const typename tile_hint_of<Op>::type& h) {
    if constexpr (std::is_same<typename tile_hint_of<Op>::type, no_tile_hint>::value)
        return op.template lookup<false>(cache, key);
    else
        return op.lookup_in_tile(cache, key, h);
}

// about 21 KB of shared memory per block; 6 resident blocks (40 registers),
// fewer for index kinds compiled for fewer.  kRows = false: no row ids, the
// row of probe i is i (plain probes in sorted tiles).
template <class Op, bool kRows>
__global__ void __launch_bounds__(kBlock, Op::kMinBlocks < 6 ? Op::kMinBlocks : 6) k_sorted_pairs(const __grid_constant__ Op op, const stage_desc sd,
                                                         const uint64_t* __restrict__ keys,
                                                         const uint32_t* __restrict__ rows, uint64_t m,
                                                         uint2* __restrict__ pairs,
                                                         const uint64_t* __restrict__ d_base,
                                                         uint64_t* __restrict__ d_count, pairs_ws ws,
                                                         uint32_t num_tiles) {
    extern __shared__ __align__(16) uint64_t cache[];
    using hint_t = typename tile_hint_of<Op>::type;
    __shared__ sorted_tile_smem<hint_t> t;
    stage_cache(cache, sd);
    const uint64_t base = d_base ? *d_base : 0ull;
    auto fill = [&](uint64_t t0, uint32_t* s_pos) {
        const uint32_t tn = m - t0 < kSortTile ? (uint32_t)(m - t0) : kSortTile;
        sort_tile(op, cache, keys, t0, tn,
                  [&](uint32_t j) {
                      if constexpr (kRows) return __ldcs(rows + t0 + j);
                      else return (uint32_t)(t0 + j);
                  },
                  t);
        const hint_t h = t.hint;
#pragma unroll 1
        for (int k = 0; k < kSortItems; ++k) {
            const uint32_t j = k * kBlock + threadIdx.x;
            s_pos[j] = j < tn ? sorted_lookup(op, cache, t.key[j], h) : kInvalid;
        }
    };
    auto row_of = [&](int k, uint64_t) { return t.row[k * kBlock + threadIdx.x]; };
    for (;;) {
        const uint32_t tile = claim_tile(ws);
        if (tile >= num_tiles) break;
        if (!pairs_tile<kSortItems>(fill, row_of, tile, pairs, base, d_count, ws, num_tiles)) break;
    }
}

// Block-wise sorted lookup (the reference's bws_lookup,
// src/index_lookup_common.cuh:398-549): each tile of kSortTile probes is
// sorted by key, searched in that order, and the positions are put back in
// probe order through shared memory: out[i] = lookup(probes[i]).  A block
// takes kSortedLookupTiles consecutive tiles (the shared cache is staged
// once for them).
constexpr uint32_t kSortedLookupTiles = 4;
template <class Op>
__global__ void __launch_bounds__(kBlock, Op::kMinBlocks < 6 ? Op::kMinBlocks : 6) k_sorted_lookup(const __grid_constant__ Op op, const stage_desc sd,
                                                          const uint64_t* __restrict__ probes, uint64_t m,
                                                          uint32_t* __restrict__ out) {
    extern __shared__ __align__(16) uint64_t cache[];
    using hint_t = typename tile_hint_of<Op>::type;
    __shared__ sorted_tile_smem<hint_t> t;
    __shared__ uint32_t s_pos[kSortTile];
    stage_cache(cache, sd);
    for (uint32_t r = 0; r < kSortedLookupTiles; ++r) {
        const uint64_t t0 = ((uint64_t)blockIdx.x * kSortedLookupTiles + r) * kSortTile;
        if (t0 >= m) break;
        const uint32_t tn = m - t0 < kSortTile ? (uint32_t)(m - t0) : kSortTile;
        sort_tile(op, cache, probes, t0, tn, [](uint32_t j) { return j; }, t);
        const hint_t h = t.hint;
#pragma unroll 1
        for (int k = 0; k < kSortItems; ++k) {
            const uint32_t j = k * kBlock + threadIdx.x;
            if (j < tn) s_pos[t.row[j]] = sorted_lookup(op, cache, t.key[j], h);
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kSortItems; ++k) {
            const uint32_t j = k * kBlock + threadIdx.x;
            if (j < tn) __stcs(out + t0 + j, s_pos[j]);
        }
        __syncthreads();  // t and s_pos are reused by the next tile
    }
}

// ---------------------------------------------------------------------------
// dispatch helpers
// ---------------------------------------------------------------------------
stage_desc make_stage(const gj_index* idx) {
    stage_desc sd{};
    switch (idx->type) {
        case GJ_INDEX_BINARY_SEARCH:
            if (idx->bs.fence_slots) {
                sd.src0 = idx->bs.fence;
                sd.words0 = idx->bs.fence_slots;
            }
            break;
        case GJ_INDEX_BTREE:
            if (idx->bt.cached_levels) {
                sd.src0 = idx->bt.level[idx->bt.height];
                sd.words0 = idx->bt.cache_keys;
            }
            break;
        case GJ_INDEX_HARMONIA:
            if (idx->hm.cached_nodes) {
                sd.src0 = idx->hm.keys;
                sd.words0 = idx->hm.cached_nodes * kHarmoniaKeys;
                sd.src1 = idx->hm.children;
                sd.words1 = idx->hm.cached_nodes;
            }
            break;
        default:
            break;
    }
    return sd;
}

size_t stage_bytes(const stage_desc& sd) { return (size_t)(sd.words0 + sd.words1) * sizeof(uint64_t); }

template <class Kernel>
int prepare_smem(Kernel kernel, size_t smem) {
    // Static plus dynamic shared memory above 48 KB needs the kernel's
    // dynamic limit raised first; the limit set so far is remembered per
    // (device, kernel), so the attribute call is made once per new maximum.
    if (smem == 0) return GJ_OK;
    int dev = 0;
    GJ_CUDA_TRY(cudaGetDevice(&dev));
    static std::mutex mu;
    static std::map<std::pair<int, const void*>, size_t> raised;
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = raised[{dev, reinterpret_cast<const void*>(kernel)}];
    if (smem > cur) {
        GJ_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        cur = smem;
    }
    return GJ_OK;
}

template <class Kernel>
int grid_for(Kernel kernel, size_t smem, uint64_t work_items, int* grid) {
    device_info di;
    GJ_TRY(current_device_info(&di));
    GJ_TRY(prepare_smem(kernel, smem));
    int per_sm = 0;
    GJ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem));
    if (per_sm < 1) per_sm = 1;
    uint64_t g = (uint64_t)di.sm_count * per_sm;
    const uint64_t need = (work_items + kBlock - 1) / kBlock;
    if (need < g) g = need ? need : 1;
    *grid = (int)g;
    return GJ_OK;
}

template <class Op>
int run_lookup(const Op& op, const stage_desc& sd, const uint64_t* probes, uint64_t m, uint32_t* out, cudaStream_t s) {
    const size_t smem = stage_bytes(sd);
    GJ_TRY(prepare_smem(k_lookup<Op>, smem));
    const uint64_t grid = (m + kLookupTile - 1) / kLookupTile;
    k_lookup<Op><<<(unsigned)grid, kBlock, smem, s>>>(op, sd, probes, m, out);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

template <class Op>
int run_sorted_lookup(const Op& op, const stage_desc& sd, const uint64_t* probes, uint64_t m, uint32_t* out,
                      cudaStream_t s) {
    const size_t smem = stage_bytes(sd);
    GJ_TRY(prepare_smem(k_sorted_lookup<Op>, smem));
    const uint64_t per_block = (uint64_t)kSortTile * kSortedLookupTiles;
    const uint64_t grid = (m + per_block - 1) / per_block;
    k_sorted_lookup<Op><<<(unsigned)grid, kBlock, smem, s>>>(op, sd, probes, m, out);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

template <class Op>
int run_scatter(const Op& op, const stage_desc& sd, const uint64_t* keys, const uint32_t* rows, uint64_t m,
                uint32_t* out, cudaStream_t s) {
    const size_t smem = stage_bytes(sd);
    GJ_TRY(prepare_smem(k_scatter_lookup<Op>, smem));
    const uint64_t grid = (m + kLookupTile - 1) / kLookupTile;
    k_scatter_lookup<Op><<<(unsigned)grid, kBlock, smem, s>>>(op, sd, keys, rows, m, out);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

template <class Op>
int run_pairs(const Op& op, const stage_desc& sd, const uint64_t* probes, const uint32_t* rows, uint64_t m,
              uint32_t* pairs, const uint64_t* d_base, uint64_t* d_count, void* ws, size_t ws_bytes, uint32_t* stash,
              cudaStream_t s, uint32_t spin_limit = 0, bool skip_first_tile = false, bool unordered = false) {
    const uint32_t num_tiles = (uint32_t)((m + kTile - 1) / kTile);
    pairs_ws pw;
    size_t used = 0;
    if (!carve_pairs_ws(ws, ws_bytes, m, &pw, &used)) {
        set_error("inlj pairs: workspace of %zu bytes is smaller than the %zu required", ws_bytes,
                  pairs_workspace_bytes(m));
        return GJ_ERR_WORKSPACE;
    }
    if (m == 0) {
        if (d_base && d_base != d_count)
            GJ_CUDA_TRY(cudaMemcpyAsync(d_count, d_base, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
        else if (!d_base)
            GJ_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(uint64_t), s));
        return GJ_OK;
    }
    GJ_CUDA_TRY(cudaMemsetAsync(ws, 0, used, s));
    if (spin_limit) pw.spin_limit = spin_limit;
    // test hook: the tile counter starts at 1, so tile 0 is never claimed and
    // never publishes; every later tile's look-back runs out
    if (skip_first_tile) GJ_CUDA_TRY(cudaMemsetAsync(pw.tile_counter, 1, 1, s));
    if (stash) {
        GJ_TRY(run_lookup(op, sd, probes, m, stash, s));
        const uint32_t compact_tiles = (uint32_t)((m + kCompactTile - 1) / kCompactTile);
        int grid = 0;
        GJ_TRY(grid_for(k_compact_pairs, 0, (uint64_t)compact_tiles * kBlock, &grid));
        k_compact_pairs<<<grid, kBlock, 0, s>>>(stash, rows, m, reinterpret_cast<uint2*>(pairs), d_base, d_count, pw,
                                                compact_tiles);
        GJ_CUDA_TRY(cudaGetLastError());
        return GJ_OK;
    }
    const size_t smem = stage_bytes(sd);
    int grid = 0;
    if (unordered) {
        GJ_TRY(grid_for(k_pairs<Op, false>, smem, (uint64_t)num_tiles * kBlock, &grid));
        k_pairs<Op, false><<<grid, kBlock, smem, s>>>(op, sd, probes, rows, m, reinterpret_cast<uint2*>(pairs), d_base,
                                                      d_count, pw, num_tiles);
    } else {
        GJ_TRY(grid_for(k_pairs<Op, true>, smem, (uint64_t)num_tiles * kBlock, &grid));
        k_pairs<Op, true><<<grid, kBlock, smem, s>>>(op, sd, probes, rows, m, reinterpret_cast<uint2*>(pairs), d_base,
                                                     d_count, pw, num_tiles);
    }
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

template <class Op>
int run_sorted_pairs(const Op& op, const stage_desc& sd, const uint64_t* keys, const uint32_t* rows, uint64_t m,
                     uint32_t* pairs, const uint64_t* d_base, uint64_t* d_count, void* ws, size_t ws_bytes,
                     cudaStream_t s) {
    const uint32_t num_tiles = (uint32_t)((m + kSortTile - 1) / kSortTile);
    pairs_ws pw;
    size_t used = 0;
    if (!carve_pairs_ws(ws, ws_bytes, m, &pw, &used)) {
        set_error("partitioned pairs: workspace of %zu bytes is smaller than the %zu required", ws_bytes,
                  pairs_workspace_bytes(m));
        return GJ_ERR_WORKSPACE;
    }
    if (m == 0) {
        if (d_base && d_base != d_count)
            GJ_CUDA_TRY(cudaMemcpyAsync(d_count, d_base, sizeof(uint64_t), cudaMemcpyDeviceToDevice, s));
        else if (!d_base)
            GJ_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(uint64_t), s));
        return GJ_OK;
    }
    GJ_CUDA_TRY(cudaMemsetAsync(ws, 0, used, s));
    const size_t smem = stage_bytes(sd);
    int grid = 0;
    if (rows) {
        GJ_TRY(grid_for(k_sorted_pairs<Op, true>, smem, (uint64_t)num_tiles * kBlock, &grid));
        k_sorted_pairs<Op, true><<<grid, kBlock, smem, s>>>(op, sd, keys, rows, m, reinterpret_cast<uint2*>(pairs),
                                                            d_base, d_count, pw, num_tiles);
    } else {
        GJ_TRY(grid_for(k_sorted_pairs<Op, false>, smem, (uint64_t)num_tiles * kBlock, &grid));
        k_sorted_pairs<Op, false><<<grid, kBlock, smem, s>>>(op, sd, keys, rows, m, reinterpret_cast<uint2*>(pairs),
                                                             d_base, d_count, pw, num_tiles);
    }
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

template <class Op>
int run_call(const Op& op, const gj_index* idx, const lookup_call& c) {
    const stage_desc sd = make_stage(idx);
    switch (c.action) {
        case lookup_action::positions: return run_lookup(op, sd, c.keys, c.m, c.out, c.s);
        case lookup_action::scatter: return run_scatter(op, sd, c.keys, c.rows, c.m, c.out, c.s);
        case lookup_action::pairs:
            return run_pairs(op, sd, c.keys, c.rows, c.m, c.out, c.d_base, c.d_count, c.ws, c.ws_bytes, c.stash, c.s,
                             c.spin_limit, c.skip_first_tile, c.unordered);
        case lookup_action::sorted_pairs:
            return run_sorted_pairs(op, sd, c.keys, c.rows, c.m, c.out, c.d_base, c.d_count, c.ws, c.ws_bytes, c.s);
        case lookup_action::sorted_positions: return run_sorted_lookup(op, sd, c.keys, c.m, c.out, c.s);
    }
    set_error("probe kernels: unknown action");
    return GJ_ERR_INVALID_ARGUMENT;
}

}  // namespace
}  // namespace gj
