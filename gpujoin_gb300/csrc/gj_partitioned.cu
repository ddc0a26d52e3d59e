// gj_partitioned.cu -- the windowed partitioned INLJ.
//
// Replaces partitioning_approach::run with its window loop
// (src/index_lookup_partitioning.cu:436-507) and partitioned_lookup_kernel
// (:218-248): the probe side of each window is range-partitioned on the
// index's key range (gj_partition.cu), then every partition is probed against
// its own slice of the sorted build column.
//
// Partition directory.  Partition p covers the keys
// [min_key + p * 2^shift, min_key + (p + 1) * 2^shift) and so one contiguous
// slice [c_p, c_{p+1}) of the column (the leaf level of the clustered B+tree,
// the leaf level of Harmonia, the array of binary search and RadixSpline).
// The directory cuts each partition's key range into D = 2^d equal buckets
// and records, per bucket, the 32-byte column sector that holds the lower
// bound of the bucket's first key, as a 16-bit offset from the partition's
// first sector -- D + 1 entries per partition (the last one the next
// partition's start).  d is chosen for about one bucket per sector, so the
// lower bound of a probe key in bucket b lies in the sectors named by
// entries b and b + 1, usually one or two sectors apart.  The directory
// depends only on the index and the partition geometry; it is built once per
// call (one pass over the column) into the workspace.
//
// A probe block takes one chunk of one partition (up to kChunk probes),
// copies that partition's directory (at most 64 KB) into shared memory and
// searches each probe with one shared-memory read and, usually, one or two
// independent sector loads from L2 (the partition's column slice is read by
// every block of that partition at about the same time).  A partition whose
// slice spans more than 65534 sectors (a directory offset would not fit 16
// bits: skewed key distributions) is searched by a sector-granular binary
// search over its whole slice instead.  The search returns the lower bound,
// from which each index kind's result follows (src/indexes.cuh): the lower
// bound (binary search, RadixSpline, learned; invalid at n), the position of
// an equal key (B+tree, Harmonia, hash; else invalid), or nothing (no-op).
//
// Pairs of a window are emitted per block tile: one atomicAdd on *d_count
// per tile gives the tile's place, so pairs come out grouped by tile in an
// order that is not fixed (the reference's order follows its atomics as
// well, src/tpch/tpch_14_ij.cu:371-407); the count and the set of pairs are.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "gj_internal.h"

namespace gj {
namespace {

constexpr uint32_t kMaxRadixBits = 12;
constexpr uint32_t kMaxDirBits = 15;       // 2^15 u16 entries = 64 KB of shared memory: 3 blocks per SM
constexpr uint32_t kDirPad = 8;            // D + 1 entries rounded up to a multiple of 8 (16 bytes)
constexpr uint16_t kDirUnset = 0xFFFF;     // not yet written / offset above 65534
constexpr uint32_t kDirKeyCap = 16;        // entries one key thread writes; the rest by the fill pass
constexpr int kProbeBlock = 256;
constexpr int kProbeItems = 4;             // probes per thread in flight
constexpr uint32_t kProbeTile = kProbeBlock * kProbeItems;
constexpr uint32_t kChunk = 1u << 14;      // probes per block (directory copied once per chunk)

enum probe_semantics : int { kSemNone = 0, kSemLowerBound = 1, kSemExact = 2 };

struct pgeom {
    uint64_t min_key;
    uint64_t span;      // max_key - min_key
    uint32_t shift;     // partition width 2^shift
    uint32_t fanout;
    uint32_t dbits;     // buckets per partition 2^dbits, dbits <= shift
    uint32_t bshift;    // shift - dbits
};

// entries per partition: D + 1, rounded up to whole 16-byte words
__host__ __device__ __forceinline__ uint32_t dir_stride(uint32_t dbits) { return ((1u << dbits) + kDirPad) & ~7u; }

// partition and bucket of a key (the partition function of the scatter)
__device__ __forceinline__ void part_bucket(uint64_t k, const pgeom& g, uint32_t* p_out, uint32_t* b_out) {
    if (k <= g.min_key) {
        *p_out = 0;
        *b_out = 0;
        return;
    }
    const uint64_t off = k - g.min_key;
    uint64_t p = off >> g.shift;
    if (p >= g.fanout) p = g.fanout - 1;
    uint64_t b = (off - (p << g.shift)) >> g.bshift;  // p << shift <= off: no overflow
    const uint64_t nb = 1ull << g.dbits;
    if (b >= nb) b = nb - 1;
    *p_out = (uint32_t)p;
    *b_out = (uint32_t)b;
}

__device__ __forceinline__ uint32_t global_bucket(uint64_t k, const pgeom& g) {
    uint32_t p, b;
    part_bucket(k, g, &p, &b);
    return (p << g.dbits) | b;
}

// first column position of partition p (c_0 = 0, c_F = n)
__device__ __forceinline__ uint64_t partition_start(const uint64_t* col, uint64_t n, const pgeom& g, uint32_t p) {
    if (p == 0) return 0;
    if (p >= g.fanout) return n;
    const uint64_t off = (uint64_t)p << g.shift;
    if (off > g.span) return n;
    return lower_bound_branch_free(col, n, g.min_key + off);
}

// bound[p] = c_p for p in [0, F]; directory entry D of partition p = the
// offset of the sector of c_{p+1}; wide[p] = 1 when that offset does not fit
__global__ void k_dir_bounds(const uint64_t* __restrict__ col, uint64_t n, pgeom g, uint32_t* __restrict__ bound,
                             uint16_t* __restrict__ dir, uint32_t* __restrict__ wide) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > g.fanout) return;
    const uint64_t c0 = partition_start(col, n, g, p);
    bound[p] = (uint32_t)c0;
    if (p == g.fanout) return;
    const uint64_t c1 = partition_start(col, n, g, p + 1);
    const uint64_t rel = (c1 >> 2) - (c0 >> 2);
    wide[p] = rel >= kDirUnset ? 1u : 0u;
    dir[(uint64_t)p * dir_stride(g.dbits) + (1u << g.dbits)] = rel >= kDirUnset ? kDirUnset : (uint16_t)rel;
}

__device__ __forceinline__ void dir_put(uint16_t* dir, const uint32_t* bound, uint32_t* wide, const pgeom& g,
                                        uint32_t gb, uint64_t pos) {
    const uint32_t p = gb >> g.dbits, b = gb & ((1u << g.dbits) - 1);
    const uint64_t rel = (pos >> 2) - (bound[p] >> 2);
    if (rel >= kDirUnset) {
        wide[p] = 1u;
        return;
    }
    dir[(uint64_t)p * dir_stride(g.dbits) + b] = (uint16_t)rel;
}

// One thread per column position i in [0, n]: the buckets whose first key's
// lower bound is i are those in (G(col[i-1]), G(col[i])] (G = global bucket
// of a key, monotone); after the last key, every bucket up to F * D - 1 has
// lower bound n.  A thread writes at most kDirKeyCap of them; k_dir_fill
// completes longer runs (gaps in the column).  kDirKeysPer positions per
// thread, kDirKeysBlock apart (coalesced loads, several in flight).
constexpr int kDirKeysBlock = 256;
constexpr int kDirKeysPer = 8;
__global__ void __launch_bounds__(kDirKeysBlock) k_dir_keys(const uint64_t* __restrict__ col, uint64_t n, pgeom g,
                                                            const uint32_t* __restrict__ bound,
                                                            uint16_t* __restrict__ dir, uint32_t* __restrict__ wide) {
    const uint64_t i0 = (uint64_t)blockIdx.x * (kDirKeysBlock * kDirKeysPer) + threadIdx.x;
    const uint32_t total = g.fanout << g.dbits;
    uint32_t cur[kDirKeysPer], prev[kDirKeysPer];
#pragma unroll
    for (int k = 0; k < kDirKeysPer; ++k) {
        const uint64_t i = i0 + (uint64_t)k * kDirKeysBlock;
        cur[k] = i < n ? global_bucket(__ldcs(reinterpret_cast<const unsigned long long*>(col) + i), g) : total - 1u;
        prev[k] = (i >= 1 && i - 1 < n) ? global_bucket(ld_ro(col + i - 1), g) + 1u : 0u;
    }
#pragma unroll
    for (int k = 0; k < kDirKeysPer; ++k) {
        const uint64_t i = i0 + (uint64_t)k * kDirKeysBlock;
        if (i > n) break;
        const uint32_t lo = i == 0 ? 0u : prev[k], hi = cur[k];
        if (lo > hi) continue;
        const uint32_t end = hi - lo >= kDirKeyCap ? lo + kDirKeyCap - 1 : hi;
        for (uint32_t gb = lo; gb <= end; ++gb) dir_put(dir, bound, wide, g, gb, i);
    }
}

// Entries left unset by k_dir_keys: the lower bound of the bucket's first
// key by a binary search over the partition's slice.
__global__ void k_dir_fill(const uint64_t* __restrict__ col, uint64_t n, pgeom g, const uint32_t* __restrict__ bound,
                           uint16_t* __restrict__ dir, uint32_t* __restrict__ wide) {
    const uint32_t gb = blockIdx.x * blockDim.x + threadIdx.x;
    if (gb >= (g.fanout << g.dbits)) return;
    const uint32_t p = gb >> g.dbits, b = gb & ((1u << g.dbits) - 1);
    uint16_t* e = dir + (uint64_t)p * dir_stride(g.dbits) + b;
    if (*e != kDirUnset || wide[p]) return;
    const uint64_t first = g.min_key + ((uint64_t)p << g.shift) + ((uint64_t)b << g.bshift);
    const uint64_t c0 = bound[p], c1 = bound[p + 1];
    const uint64_t pos = c0 + lower_bound_branch_free(col + c0, c1 - c0, first);
    dir_put(dir, bound, wide, g, gb, pos);
}

// chunk_begin[p] = number of chunks of the partitions before p (F + 1
// entries; chunk_begin[F] = total) and chunk_part[c] = the partition of
// chunk c, one block of 1024 threads
__global__ void __launch_bounds__(1024) k_chunk_map(const uint64_t* __restrict__ offsets, uint32_t fanout,
                                                    uint32_t* __restrict__ chunk_begin,
                                                    uint32_t* __restrict__ chunk_part) {
    __shared__ uint32_t s_warp[32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t per = (fanout + 1023) / 1024;
    const uint32_t begin = threadIdx.x * per;
    uint32_t sum = 0;
    for (uint32_t q = 0; q < per; ++q) {
        const uint32_t p = begin + q;
        if (p < fanout) sum += (uint32_t)((offsets[p + 1] - offsets[p] + kChunk - 1) / kChunk);
    }
    uint32_t incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (uint32_t)d) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        const uint32_t v = s_warp[lane];
        uint32_t w = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= (uint32_t)d) w += t;
        }
        s_warp[lane] = w - v;
    }
    __syncthreads();
    uint32_t run = s_warp[warp] + incl - sum;
    for (uint32_t q = 0; q < per; ++q) {
        const uint32_t p = begin + q;
        if (p < fanout) {
            chunk_begin[p] = run;
            const uint32_t nc = (uint32_t)((offsets[p + 1] - offsets[p] + kChunk - 1) / kChunk);
            for (uint32_t c = 0; c < nc; ++c) chunk_part[run + c] = p;
            run += nc;
        }
    }
    if (threadIdx.x == 1023) chunk_begin[fanout] = run;
}

// Lower bound of key when it lies in the sectors [s_lo, s_hi] of the column
// (s_lo <= s_hi; the sector of every key before it holds only smaller keys
// or the lower bound itself).  The first two sectors are loaded together;
// the rest, if any, by a binary search over sectors.  *eq: col[result] == key.
template <bool kAligned>
__device__ __forceinline__ uint64_t lb_in_sectors(const uint64_t* __restrict__ col, uint64_t n, uint64_t s_lo,
                                                  uint64_t s_hi, uint64_t key, bool* eq) {
    *eq = false;
    const uint64_t b0 = s_lo << 2;
    if (b0 >= n) return n;
    if constexpr (kAligned) {
        if (n - b0 >= 8 || (n - b0 >= 4 && s_hi == s_lo)) {
            uint64_t k[4], k2[4];
            ld_sector(col + b0, k);
            const bool two = s_hi > s_lo;
            if (two) ld_sector(col + b0 + 4, k2);
            const uint32_t below = (k[0] < key) + (k[1] < key) + (k[2] < key) + (k[3] < key);
            if (below < 4) {
                *eq = pick4(k, below) == key;
                return b0 + below;
            }
            if (two) {
                const uint32_t below2 = (k2[0] < key) + (k2[1] < key) + (k2[2] < key) + (k2[3] < key);
                if (below2 < 4) {
                    *eq = pick4(k2, below2) == key;
                    return b0 + 4 + below2;
                }
                if (s_hi == s_lo + 1) return b0 + 8 < n ? b0 + 8 : n;
                const uint64_t hi = ((s_hi + 1) << 2) < n ? ((s_hi + 1) << 2) : n;
                return lower_bound_sectors(col, n, b0 + 8, hi, key, true, eq);
            }
            return b0 + 4 < n ? b0 + 4 : n;
        }
    }
    const uint64_t hi = ((s_hi + 1) << 2) < n ? ((s_hi + 1) << 2) : n;
    return lower_bound_sectors(col, n, b0, hi, key, kAligned, eq);
}

struct probe_args {
    const uint64_t* pkeys;       // partitioned keys of the window
    const uint32_t* prows;       // their probe rows
    const uint64_t* offsets;     // partition starts in the window (F + 1)
    const uint32_t* chunk_begin; // F + 1
    const uint32_t* chunk_part;  // partition of each chunk
    const uint16_t* dir;         // F x dir_stride(dbits)
    const uint32_t* bound;       // c_p, F + 1
    const uint32_t* wide;        // F
    const uint64_t* col;
    uint64_t n;
    pgeom g;
    uint32_t* positions;         // positions[row] = result, or null
    uint2* pairs;                // (row, result) of the matches, or null
    unsigned long long* count;   // pairs appended at atomicAdd(count, ...)
};

template <int kSem, bool kAligned>
__global__ void __launch_bounds__(kProbeBlock, 3) k_part_probe(const __grid_constant__ probe_args a) {
    extern __shared__ __align__(16) uint16_t s_dir[];
    constexpr int kWarps = kProbeBlock / 32;
    __shared__ uint32_t s_cnt[kWarps * kProbeItems];
    __shared__ unsigned long long s_base;
    const uint32_t c = blockIdx.x;
    const uint32_t F = a.g.fanout;
    if (c >= __ldg(a.chunk_begin + F)) return;
    const uint32_t p = __ldg(a.chunk_part + c);
    const uint64_t pbeg = __ldg(reinterpret_cast<const unsigned long long*>(a.offsets) + p) +
                          (uint64_t)(c - __ldg(a.chunk_begin + p)) * kChunk;
    const uint64_t pend0 = __ldg(reinterpret_cast<const unsigned long long*>(a.offsets) + p + 1);
    const uint64_t pend = pend0 - pbeg < kChunk ? pend0 : pbeg + kChunk;
    const bool wide = kSem != kSemNone && __ldg(a.wide + p) != 0;
    const uint64_t c_lo = __ldg(a.bound + p), c_hi = __ldg(a.bound + p + 1);
    const uint64_t sbase = c_lo >> 2;
    if (kSem != kSemNone && !wide) {
        const uint32_t words = dir_stride(a.g.dbits) / 8;  // uint4 = 8 entries
        const uint4* src = reinterpret_cast<const uint4*>(a.dir + (uint64_t)p * dir_stride(a.g.dbits));
        uint4* dst = reinterpret_cast<uint4*>(s_dir);
        for (uint32_t w = threadIdx.x; w < words; w += kProbeBlock) dst[w] = __ldg(src + w);
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t t0 = pbeg; t0 < pend; t0 += kProbeTile) {
        // The items of a thread go through each phase together, so their
        // loads are in flight at the same time: probe keys and rows, then
        // the first sector of each probe's range, then (for the probes whose
        // lower bound lies further on) the next sector; anything else (a
        // longer range, a partial last sector, a wide partition, an
        // unaligned column) takes the sector binary search.
        uint64_t key[kProbeItems];
        uint32_t res[kProbeItems], row[kProbeItems], slo[kProbeItems], shi[kProbeItems];
        bool valid[kProbeItems], todo[kProbeItems];
#pragma unroll
        for (int k = 0; k < kProbeItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kProbeBlock + threadIdx.x;
            valid[k] = i < pend;
            key[k] = valid[k] ? __ldcs(reinterpret_cast<const unsigned long long*>(a.pkeys) + i) : 0ull;
            row[k] = valid[k] ? __ldcs(a.prows + i) : 0u;
            res[k] = kInvalid;
            todo[k] = kSem != kSemNone && valid[k];
            slo[k] = shi[k] = 0;
        }
        if constexpr (kSem != kSemNone) {
            if (!wide) {
#pragma unroll
                for (int k = 0; k < kProbeItems; ++k) {
                    uint32_t pp, b;
                    part_bucket(key[k], a.g, &pp, &b);
                    slo[k] = (uint32_t)sbase + s_dir[b];
                    shi[k] = (uint32_t)sbase + s_dir[b + 1];
                }
                if constexpr (kAligned) {
#pragma unroll
                    for (int step = 0; step < 2; ++step) {
                        uint64_t w[kProbeItems][4];
                        bool load[kProbeItems];
#pragma unroll
                        for (int k = 0; k < kProbeItems; ++k) {
                            const uint32_t sct = slo[k] + (uint32_t)step;
                            load[k] = todo[k] && sct <= shi[k] && ((uint64_t)sct << 2) + 4 <= a.n;
                            if (load[k]) ld_sector(a.col + ((uint64_t)sct << 2), w[k]);
                        }
#pragma unroll
                        for (int k = 0; k < kProbeItems; ++k) {
                            if (!load[k]) continue;
                            const uint64_t x = key[k];
                            const uint32_t below = (w[k][0] < x) + (w[k][1] < x) + (w[k][2] < x) + (w[k][3] < x);
                            if (below < 4) {
                                todo[k] = false;
                                if (kSem == kSemLowerBound || pick4(w[k], below) == x)
                                    res[k] = (((uint32_t)slo[k] + (uint32_t)step) << 2) + below;
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < kProbeItems; ++k) {
                if (!todo[k]) continue;
                bool eq = false;
                const uint64_t lo = wide ? c_lo : (uint64_t)slo[k] << 2;
                const uint64_t hi = wide ? c_hi : ((((uint64_t)shi[k] + 1) << 2) < a.n ? ((uint64_t)shi[k] + 1) << 2 : a.n);
                const uint64_t lb = lower_bound_sectors(a.col, a.n, lo, hi, key[k], kAligned, &eq);
                if (lb < a.n && (kSem == kSemLowerBound || eq)) res[k] = (uint32_t)lb;
            }
        }
        if (a.positions) {
#pragma unroll
            for (int k = 0; k < kProbeItems; ++k)
                if (valid[k]) a.positions[row[k]] = res[k];
        }
        if (a.pairs) {
            uint32_t ballot[kProbeItems];
#pragma unroll
            for (int k = 0; k < kProbeItems; ++k) {
                ballot[k] = __ballot_sync(0xffffffffu, valid[k] && res[k] != kInvalid);
                if (lane == 0) s_cnt[k * kWarps + warp] = __popc(ballot[k]);
            }
            __syncthreads();
            if (warp == 0) {
                // exclusive scan of the kWarps * kProbeItems counts in (k, warp) order
                constexpr int kPer = kWarps * kProbeItems / 32;
                uint32_t v[kPer];
                uint32_t sum = 0;
#pragma unroll
                for (int j = 0; j < kPer; ++j) {
                    v[j] = s_cnt[lane * kPer + j];
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
                for (int j = 0; j < kPer; ++j) {
                    s_cnt[lane * kPer + j] = run;
                    run += v[j];
                }
                const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
                if (lane == 0) s_base = total ? atomicAdd(a.count, (unsigned long long)total) : 0ull;
            }
            __syncthreads();
            const unsigned long long base = s_base;
#pragma unroll
            for (int k = 0; k < kProbeItems; ++k) {
                if ((ballot[k] >> lane) & 1u) {
                    const unsigned long long o =
                        base + s_cnt[k * kWarps + warp] + __popc(ballot[k] & ((1u << lane) - 1u));
                    __stcs(reinterpret_cast<unsigned long long*>(a.pairs + o),
                           ((unsigned long long)res[k] << 32) | row[k]);
                }
            }
            __syncthreads();  // s_cnt and s_base are reused by the next tile
        }
    }
}
static_assert(kProbeBlock / 32 * kProbeItems % 32 == 0, "the tile scan gives each lane whole counts");

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int semantics_of(const gj_index* idx) {
    switch (idx->type) {
        case GJ_INDEX_BTREE:
        case GJ_INDEX_HARMONIA:
        case GJ_INDEX_HASH: return kSemExact;
        case GJ_INDEX_NO_OP: return kSemNone;
        default: return kSemLowerBound;
    }
}

// directory bits: about one bucket per 32-byte sector of a partition's slice
uint32_t dir_bits_for(uint64_t n, uint32_t radix_bits, uint32_t shift) {
    const uint64_t sectors_per_part = std::max<uint64_t>(1, (n >> radix_bits) >> 2);
    uint32_t d = 4;
    while (d < kMaxDirBits && (1ull << d) < sectors_per_part) ++d;
    return std::min(d, shift);
}

struct partitioned_layout {
    uint64_t window;
    uint32_t radix_bits, fanout, dbits;
    size_t dir_entries;  // F x stride
};

partitioned_layout layout_for(const gj_index* idx, uint64_t window, uint32_t radix_bits) {
    partitioned_layout L;
    L.window = window;
    L.radix_bits = radix_bits;
    L.fanout = 1u << radix_bits;
    const uint32_t shift = shift_for(idx->min_key, idx->max_key, radix_bits);
    L.dbits = dir_bits_for(idx->n, radix_bits, shift);
    L.dir_entries = (size_t)L.fanout * dir_stride(L.dbits);
    return L;
}

// chunks of a window of w probes: at most one partial chunk per partition
uint64_t max_chunks(uint64_t w, uint32_t fanout) { return (w + kChunk - 1) / kChunk + fanout; }

size_t partitioned_ws_bytes(const partitioned_layout& L, int sm_count) {
    const uint64_t w = L.window;
    return workspace_carver::need({w * sizeof(uint64_t), w * sizeof(uint32_t), (L.fanout + 1) * sizeof(uint64_t),
                                   partition_ws_bytes(w, L.radix_bits, sm_count), L.dir_entries * sizeof(uint16_t),
                                   (L.fanout + 1) * sizeof(uint32_t), L.fanout * sizeof(uint32_t),
                                   (L.fanout + 1) * sizeof(uint32_t), max_chunks(w, L.fanout) * sizeof(uint32_t)});
}

template <class Kernel>
int raise_smem(Kernel k, size_t smem) {
    if (smem > 48 * 1024) GJ_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return GJ_OK;
}

template <int kSem, bool kAligned>
int launch_probe(const probe_args& a, uint64_t len, cudaStream_t s) {
    const size_t smem = kSem == kSemNone ? 0 : (size_t)dir_stride(a.g.dbits) * sizeof(uint16_t);
    GJ_TRY(raise_smem(k_part_probe<kSem, kAligned>, smem));
    const uint64_t grid = max_chunks(len, a.g.fanout);
    k_part_probe<kSem, kAligned><<<(unsigned)grid, kProbeBlock, smem, s>>>(a);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

int dispatch_probe(int sem, bool aligned, const probe_args& a, uint64_t len, cudaStream_t s) {
    if (sem == kSemNone) return launch_probe<kSemNone, true>(a, len, s);
    if (sem == kSemExact) return aligned ? launch_probe<kSemExact, true>(a, len, s) : launch_probe<kSemExact, false>(a, len, s);
    return aligned ? launch_probe<kSemLowerBound, true>(a, len, s) : launch_probe<kSemLowerBound, false>(a, len, s);
}

}  // namespace
}  // namespace gj

using namespace gj;

extern "C" {

int gj_index_key_range(const gj_index* index, uint64_t* min_key, uint64_t* max_key) {
    GJ_CHECK_ARG(index && min_key && max_key, "gj_index_key_range: null argument");
    *min_key = index->min_key;
    *max_key = index->max_key;
    return GJ_OK;
}

int gj_partition_shift(uint64_t min_key, uint64_t max_key, uint32_t radix_bits, uint32_t* shift) {
    GJ_CHECK_ARG(shift, "gj_partition_shift: null argument");
    GJ_CHECK_ARG(min_key <= max_key, "gj_partition_shift: min_key > max_key");
    GJ_CHECK_ARG(radix_bits >= 1 && radix_bits <= kMaxRadixBits, "gj_partition_shift: radix_bits not in [1, 12]");
    *shift = shift_for(min_key, max_key, radix_bits);
    return GJ_OK;
}

int gj_partitioned_inlj_workspace_size(const gj_index* index, uint64_t window_size, uint32_t radix_bits,
                                       size_t* bytes) {
    GJ_CHECK_ARG(index && bytes, "gj_partitioned_inlj_workspace_size: null argument");
    GJ_CHECK_ARG(window_size > 0, "gj_partitioned_inlj_workspace_size: window_size must be > 0");
    if (radix_bits == 0) radix_bits = default_radix_bits(index->n);
    GJ_CHECK_ARG(radix_bits <= kMaxRadixBits, "gj_partitioned_inlj_workspace_size: radix_bits > 12");
    device_info di;
    GJ_TRY(current_device_info(&di));
    *bytes = partitioned_ws_bytes(layout_for(index, window_size, radix_bits), di.sm_count);
    return GJ_OK;
}

int gj_partitioned_inlj(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint64_t window_size,
                        uint32_t radix_bits, uint32_t* d_positions, uint32_t* d_pairs, uint64_t* d_count,
                        void* d_workspace, size_t workspace_bytes, void* stream) {
    GJ_CHECK_ARG(index, "gj_partitioned_inlj: null index");
    GJ_CHECK_ARG(d_positions || d_pairs, "gj_partitioned_inlj: no output requested");
    GJ_CHECK_ARG(!d_pairs || d_count, "gj_partitioned_inlj: d_count is required with d_pairs");
    GJ_CHECK_ARG(m == 0 || d_probes, "gj_partitioned_inlj: null probes");
    GJ_CHECK_ARG(window_size > 0, "gj_partitioned_inlj: window_size must be > 0");
    if (m > (uint64_t)UINT32_MAX) {
        set_error("gj_partitioned_inlj: probe rows must fit 32 bits");
        return GJ_ERR_TOO_LARGE;
    }
    if (radix_bits == 0) radix_bits = default_radix_bits(index->n);
    GJ_CHECK_ARG(radix_bits <= kMaxRadixBits, "gj_partitioned_inlj: radix_bits > 12");
    cudaStream_t s = as_stream(stream);
    device_info di;
    GJ_TRY(current_device_info(&di));
    const partitioned_layout L = layout_for(index, window_size, radix_bits);
    const uint64_t w = window_size;
    workspace_carver wc(d_workspace, workspace_bytes);
    uint64_t* pkeys = wc.take<uint64_t>(w);
    uint32_t* prows = wc.take<uint32_t>(w);
    uint64_t* offsets = wc.take<uint64_t>(L.fanout + 1);
    const size_t pws_bytes = partition_ws_bytes(w, radix_bits, di.sm_count);
    void* pws = wc.take<char>(pws_bytes);
    uint16_t* dir = wc.take<uint16_t>(L.dir_entries);
    uint32_t* bound = wc.take<uint32_t>(L.fanout + 1);
    uint32_t* wide = wc.take<uint32_t>(L.fanout);
    uint32_t* chunk_begin = wc.take<uint32_t>(L.fanout + 1);
    uint32_t* chunk_part = wc.take<uint32_t>(max_chunks(w, L.fanout));
    if (!pkeys || !prows || !offsets || !pws || !dir || !bound || !wide || !chunk_begin || !chunk_part) {
        set_error("gj_partitioned_inlj: workspace of %zu bytes is smaller than the %zu required", workspace_bytes,
                  partitioned_ws_bytes(L, di.sm_count));
        return GJ_ERR_WORKSPACE;
    }
    if (d_pairs) GJ_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(uint64_t), s));
    if (m == 0) return GJ_OK;

    const int sem = semantics_of(index);
    pgeom g;
    g.min_key = index->min_key;
    g.span = index->max_key - index->min_key;
    g.shift = shift_for(index->min_key, index->max_key, radix_bits);
    g.fanout = L.fanout;
    g.dbits = L.dbits;
    g.bshift = g.shift - g.dbits;
    const uint64_t n = index->n;
    const uint64_t* col = index->d_col;
    // the partition directory (once per call)
    if (sem != kSemNone) {
        GJ_CUDA_TRY(cudaMemsetAsync(dir, 0xFF, L.dir_entries * sizeof(uint16_t), s));
        k_dir_bounds<<<(L.fanout + 1 + 255) / 256, 256, 0, s>>>(col, n, g, bound, dir, wide);
        GJ_CUDA_TRY(cudaGetLastError());
        const uint64_t per_block = (uint64_t)kDirKeysBlock * kDirKeysPer;
        k_dir_keys<<<(unsigned)((n + 1 + per_block - 1) / per_block), kDirKeysBlock, 0, s>>>(col, n, g, bound, dir,
                                                                                          wide);
        GJ_CUDA_TRY(cudaGetLastError());
        const uint64_t buckets = (uint64_t)L.fanout << L.dbits;
        k_dir_fill<<<(unsigned)((buckets + 255) / 256), 256, 0, s>>>(col, n, g, bound, dir, wide);
        GJ_CUDA_TRY(cudaGetLastError());
    } else {
        GJ_CUDA_TRY(cudaMemsetAsync(bound, 0, (L.fanout + 1) * sizeof(uint32_t), s));
        GJ_CUDA_TRY(cudaMemsetAsync(wide, 0, L.fanout * sizeof(uint32_t), s));
    }
    const bool aligned = (reinterpret_cast<uintptr_t>(col) & 31) == 0;
    probe_args a;
    a.pkeys = pkeys;
    a.prows = prows;
    a.offsets = offsets;
    a.chunk_begin = chunk_begin;
    a.chunk_part = chunk_part;
    a.dir = dir;
    a.bound = bound;
    a.wide = wide;
    a.col = col;
    a.n = n;
    a.g = g;
    a.positions = d_positions;
    a.pairs = reinterpret_cast<uint2*>(d_pairs);
    a.count = reinterpret_cast<unsigned long long*>(d_count);
    for (uint64_t off = 0; off < m; off += w) {
        const uint64_t len = std::min<uint64_t>(w, m - off);
        GJ_TRY(range_partition_impl(d_probes + off, len, g.min_key, g.shift, radix_bits, off, pkeys, prows, offsets,
                                    pws, pws_bytes, s));
        k_chunk_map<<<1, 1024, 0, s>>>(offsets, L.fanout, chunk_begin, chunk_part);
        GJ_CUDA_TRY(cudaGetLastError());
        GJ_TRY(dispatch_probe(sem, aligned, a, len, s));
    }
    return GJ_OK;
}

}  // extern "C"
