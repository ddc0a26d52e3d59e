// gj_partitioned.cu -- the windowed partitioned INLJ.
//
// Replaces partitioning_approach::run with its window loop
// (src/index_lookup_partitioning.cu:436-507) and partitioned_lookup_kernel
// (:218-248): the probe side of each window is range-partitioned on the
// index's key range (gj_partition.cu), then the partitions are probed, in
// partition order, against the index's sorted column -- the leaf level of the
// clustered B+tree and of Harmonia, the array of binary search, RadixSpline
// and the learned index.
//
// Directory.  For probes that arrive grouped by key range, the inner levels
// of a tree are replaced by a flat radix directory over the column: the key
// range [min, max] of the index cut into 2^B equal buckets (about four per
// 32-byte column sector), and per bucket the sector that holds the lower
// bound of the bucket's first key (u32).  The lower bound of a probe key in
// bucket g then lies in the sectors named by entries g and g + 1 -- for
// uniform keys mostly the first, else the next, rarely a third.  The probe reads
// the two entries (one 32-byte sector of the directory, mostly) and the
// column sector(s): two dependent loads, both L2 hits because the probes of a
// partition touch one slice of the directory and the column, which stay in
// L2 while the partition is probed.  The directory depends only on the
// index, so gj_index_prepare_partitioned builds it once and keeps it with
// the index (like the B+tree's start table); an index that was not prepared
// gets it built per call into the workspace.  Each column position marks the
// first bucket whose lower bound it is, and a prefix maximum fills the
// buckets in between (gaps of any length, in linear time).
//
// The search returns the lower bound, from which each index kind's result
// follows (src/indexes.cuh): the lower bound (binary search, RadixSpline,
// learned; invalid at n), the position of an equal key (B+tree, Harmonia,
// hash; else invalid), or nothing (no-op).
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
int device_alloc_for(gj_index* idx, size_t bytes, void** out);  // gj_index.cu

namespace {

constexpr uint32_t kMaxRadixBits = 12;
// at most 2^28 buckets (1 GiB of entries); GJ_MAX_DIR_BITS overrides it in
// tuning builds (at most 31)
#ifndef GJ_MAX_DIR_BITS
#define GJ_MAX_DIR_BITS 28
#endif
constexpr uint32_t kMaxDirBits = GJ_MAX_DIR_BITS;
static_assert(kMaxDirBits <= 31, "bucket indexes and the closing entry fit 32 bits");
constexpr int kDirBlock = 256;
constexpr int kDirPer = 8;                 // column positions (and directory entries) per thread
constexpr int kScanBlock = 1024;
constexpr int kScanPer = 4;
constexpr uint32_t kScanTile = kScanBlock * kScanPer;
// load the second sector of a bucket's range together with the first (1),
// or only when the first holds no key >= the probe (0, measured faster:
// 12.11 against 12.45 ms per 2^29 probes -- the kernel is partly bound by
// the L1 data pipe, which the speculative sector loads fill);
// GJ_PROBE_SPECULATE overrides it in tuning builds
#ifndef GJ_PROBE_SPECULATE
#define GJ_PROBE_SPECULATE 0
#endif
constexpr int kProbeBlock = 256;
// probes per thread searched together (loads in flight) and resident
// blocks per SM (the register cap); GJ_PROBE_BATCH / GJ_PROBE_BLOCKS override
// them in tuning builds
#ifndef GJ_PROBE_BATCH
#define GJ_PROBE_BATCH 2
#endif
#ifndef GJ_PROBE_BLOCKS
#define GJ_PROBE_BLOCKS 3
#endif
constexpr int kProbeBatch = GJ_PROBE_BATCH;
constexpr int kProbeItems = 8;             // probes per thread and tile (one atomicAdd per tile)
constexpr uint32_t kProbeTile = kProbeBlock * kProbeItems;
constexpr uint32_t kChunk = 4 * kProbeTile;  // probes per block

enum probe_semantics : int { kSemNone = 0, kSemLowerBound = 1, kSemExact = 2 };

// bucket of a key: (key - min) >> shift, clamped to [0, buckets - 1]
struct dir_geom {
    uint64_t min_key;
    uint32_t shift;
    uint32_t buckets;  // 2^B
};

__device__ __forceinline__ uint32_t bucket_of(uint64_t k, const dir_geom& g) {
    if (k <= g.min_key) return 0;
    const uint64_t b = (k - g.min_key) >> g.shift;
    return b >= g.buckets ? g.buckets - 1 : (uint32_t)b;
}

// Marks: dir[b] = sector(i) + 1 for the first bucket b whose first key has
// lower bound i, i in [0, n] (buckets (G(col[i-1]), G(col[i])] all have lower
// bound i; after the last key, lower bound n).  Every other entry stays 0 and
// takes the value of the nearest marked entry to its left (k_dir_max_*):
// lower bounds are monotone in the bucket, so that is a prefix maximum.
// dir[buckets] = sector(n) + 1 closes the table.
__global__ void __launch_bounds__(kDirBlock) k_dir_mark(const uint64_t* __restrict__ col, uint64_t n, dir_geom g,
                                                        uint32_t* __restrict__ dir) {
    const uint64_t i0 = (uint64_t)blockIdx.x * (kDirBlock * kDirPer) + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t cur[kDirPer];
#pragma unroll
    for (int k = 0; k < kDirPer; ++k) {
        const uint64_t i = i0 + (uint64_t)k * kDirBlock;
        cur[k] = i < n ? bucket_of(__ldcs(reinterpret_cast<const unsigned long long*>(col) + i), g) : g.buckets;
    }
#pragma unroll
    for (int k = 0; k < kDirPer; ++k) {
        const uint64_t i = i0 + (uint64_t)k * kDirBlock;
        // the bucket of key i - 1 is the previous lane's; lane 0 loads its own
        uint32_t prev = __shfl_up_sync(0xffffffffu, cur[k], 1);
        if (lane == 0 && i >= 1 && i - 1 < n) prev = bucket_of(ld_ro(col + i - 1), g);
        if (i > n) continue;
        const uint32_t lo = i == 0 ? 0u : prev + 1u;
        const uint32_t hi = cur[k];  // i == n: g.buckets (the closing entry)
        if (lo <= hi && lo <= g.buckets) dir[lo] = (uint32_t)(i >> 2) + 1u;
    }
}

// In-place inclusive prefix maximum over dir[0 .. count) (a decoupled-free
// three-kernel scan: tile maxima, their exclusive prefix in one block, then
// the tiles), turning marks into entries; the result is stored minus one
// (entry = sector index).
__global__ void __launch_bounds__(kScanBlock) k_dir_max_tiles(const uint32_t* __restrict__ dir, uint64_t count,
                                                              uint32_t* __restrict__ tile_max) {
    __shared__ uint32_t s_warp[kScanBlock / 32];
    const uint64_t t0 = (uint64_t)blockIdx.x * kScanTile;
    uint32_t m = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        const uint64_t i = t0 + (uint64_t)k * kScanBlock + threadIdx.x;
        if (i < count) m = max(m, __ldcs(dir + i));
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, d));
    if ((threadIdx.x & 31) == 0) s_warp[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = s_warp[threadIdx.x];
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, d));
        if (threadIdx.x == 0) tile_max[blockIdx.x] = m;
    }
}

// exclusive prefix maximum of the tile maxima, one block
__global__ void __launch_bounds__(kScanBlock) k_dir_max_prefix(uint32_t* __restrict__ tile_max, uint32_t tiles) {
    __shared__ uint32_t s_warp[kScanBlock / 32];
    __shared__ uint32_t s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint32_t base = 0; base < tiles; base += kScanBlock) {
        const uint32_t i = base + threadIdx.x;
        const uint32_t v = i < tiles ? tile_max[i] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl = max(incl, t);
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = s_warp[lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, w, d);
                if (lane >= (uint32_t)d) w = max(w, t);
            }
            s_warp[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const uint32_t carry = s_carry;
        const uint32_t before_warp = warp ? s_warp[warp - 1] : 0u;
        const uint32_t excl_in_warp = __shfl_up_sync(0xffffffffu, incl, 1);
        uint32_t excl = max(carry, max(before_warp, lane ? excl_in_warp : 0u));
        if (i < tiles) tile_max[i] = excl;
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) s_carry = max(carry, s_warp[kScanBlock / 32 - 1]);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanBlock) k_dir_max_apply(uint32_t* __restrict__ dir, uint64_t count,
                                                              const uint32_t* __restrict__ tile_excl) {
    __shared__ uint32_t s_warp[kScanBlock / 32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // thread t holds entries t0 + t * kScanPer .. + kScanPer - 1 (consecutive)
    const uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanPer;
    uint32_t v[kScanPer];
    uint32_t run = 0;
#pragma unroll
    for (int k = 0; k < kScanPer; ++k) {
        v[k] = base + k < count ? dir[base + k] : 0u;
        run = max(run, v[k]);
        v[k] = run;
    }
    uint32_t incl = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (uint32_t)d) incl = max(incl, t);
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= (uint32_t)d) w = max(w, t);
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    const uint32_t excl_lane = __shfl_up_sync(0xffffffffu, incl, 1);
    const uint32_t before = max(tile_excl[blockIdx.x],
                                max(warp ? s_warp[warp - 1] : 0u, lane ? excl_lane : 0u));
#pragma unroll
    for (int k = 0; k < kScanPer; ++k)
        if (base + k < count) dir[base + k] = max(before, v[k]) - 1u;  // every entry is >= 1 here
}

// Lower bound of a probe (full 32-byte sectors of an aligned column, the
// common case): the sectors of entries g and g + 1 bracket it.
struct probe_args {
    const uint64_t* pkeys;       // partitioned keys of the window
    const uint32_t* prows;       // their probe rows
    uint64_t len;                // probes in the window
    const uint32_t* dir;         // buckets + 1 entries
    const uint64_t* col;
    uint64_t n;
    dir_geom g;
    uint32_t* positions;         // positions[row] = result, or null
    uint2* pairs;                // (row, result) of the matches, or null
    unsigned long long* count;   // pairs appended at atomicAdd(count, ...)
};

template <int kSem, bool kAligned>
__global__ void __launch_bounds__(kProbeBlock, GJ_PROBE_BLOCKS) k_part_probe(const __grid_constant__ probe_args a) {
    constexpr int kWarps = kProbeBlock / 32;
    __shared__ uint32_t s_cnt[kWarps * kProbeItems];
    __shared__ unsigned long long s_base;
    const uint64_t pbeg = (uint64_t)blockIdx.x * kChunk;
    const uint64_t pend = a.len - pbeg < kChunk ? a.len : pbeg + kChunk;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (uint64_t t0 = pbeg; t0 < pend; t0 += kProbeTile) {
        uint32_t res[kProbeItems];
        bool valid[kProbeItems];
        // keys of the first batch; each batch loads the next one's before it searches
        uint64_t nkey[kProbeBatch];
#pragma unroll
        for (int k = 0; k < kProbeBatch; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kProbeBlock + threadIdx.x;
            nkey[k] = i < pend ? __ldcs(reinterpret_cast<const unsigned long long*>(a.pkeys) + i) : 0ull;
        }
#pragma unroll
        for (int r = 0; r < kProbeItems; r += kProbeBatch) {
            // kProbeBatch probes of the thread go through each phase
            // together, so that their loads are in flight at the same time:
            // directory entries; the sector of the first entry (the lower
            // bound lies there for about 7 in 8 uniform keys at four buckets
            // per sector); the next sector when the range goes on; anything
            // else (a longer range, a partial last sector, an unaligned
            // column) takes the sector binary search.
            uint64_t key[kProbeBatch];
            uint32_t slo[kProbeBatch], shi[kProbeBatch];
            bool todo[kProbeBatch];
#pragma unroll
            for (int k = 0; k < kProbeBatch; ++k) {
                const uint64_t i = t0 + (uint64_t)(r + k) * kProbeBlock + threadIdx.x;
                key[k] = nkey[k];
                valid[r + k] = i < pend;
                res[r + k] = kInvalid;
                todo[k] = kSem != kSemNone && valid[r + k];
                slo[k] = shi[k] = 0;
                if (kSem != kSemNone && todo[k]) {
                    // entries b and b + 1: one 16-byte load unless b is the
                    // last of its four (the directory is padded to whole
                    // groups of four, so the aligned load stays inside it)
                    const uint32_t b = bucket_of(key[k], a.g);
                    const uint4 e = __ldg(reinterpret_cast<const uint4*>(a.dir) + (b >> 2));
                    const uint32_t q = b & 3u;
                    slo[k] = q == 0 ? e.x : q == 1 ? e.y : q == 2 ? e.z : e.w;
                    shi[k] = q == 0 ? e.y : q == 1 ? e.z : q == 2 ? e.w : __ldg(a.dir + b + 1);
                }
            }
            if (r + kProbeBatch < kProbeItems) {
#pragma unroll
                for (int k = 0; k < kProbeBatch; ++k) {
                    const uint64_t i = t0 + (uint64_t)(r + kProbeBatch + k) * kProbeBlock + threadIdx.x;
                    nkey[k] = i < pend ? __ldcs(reinterpret_cast<const unsigned long long*>(a.pkeys) + i) : 0ull;
                }
            }
            if constexpr (kSem != kSemNone) {
                if constexpr (kAligned) {
                    uint64_t w0[kProbeBatch][4], w1[kProbeBatch][4];
                    bool l0[kProbeBatch], l1[kProbeBatch];
#pragma unroll
                    for (int k = 0; k < kProbeBatch; ++k) {
                        l0[k] = todo[k] && ((uint64_t)slo[k] << 2) + 4 <= a.n;
                        l1[k] = GJ_PROBE_SPECULATE && l0[k] && shi[k] > slo[k] && ((uint64_t)slo[k] << 2) + 8 <= a.n;
                        if (l0[k]) ld_sector(a.col + ((uint64_t)slo[k] << 2), w0[k]);
                        if (l1[k]) ld_sector(a.col + ((uint64_t)slo[k] << 2) + 4, w1[k]);
                    }
#pragma unroll
                    for (int k = 0; k < kProbeBatch; ++k) {
                        const uint64_t x = key[k];
                        if (l0[k]) {
                            const uint32_t b0 = (w0[k][0] < x) + (w0[k][1] < x) + (w0[k][2] < x) + (w0[k][3] < x);
                            if (b0 < 4) {
                                todo[k] = false;
                                if (kSem == kSemLowerBound || pick4(w0[k], b0) == x) res[r + k] = (slo[k] << 2) + b0;
                                continue;
                            }
                            if (!l1[k]) slo[k] += 1;  // first sector below the key, second not loaded yet
                        }
                        if (l1[k]) {
                            const uint32_t b1 = (w1[k][0] < x) + (w1[k][1] < x) + (w1[k][2] < x) + (w1[k][3] < x);
                            if (b1 < 4) {
                                todo[k] = false;
                                if (kSem == kSemLowerBound || pick4(w1[k], b1) == x)
                                    res[r + k] = (slo[k] << 2) + 4 + b1;
                                continue;
                            }
                            slo[k] += 2;  // both sectors below the key: go on from the third
                        }
                    }
                    // the next sector (the third, or the second when it was
                    // not loaded with the first), for the probes that got this far
#pragma unroll
                    for (int k = 0; k < kProbeBatch; ++k) {
                        l0[k] = todo[k] && l0[k] && slo[k] <= shi[k] && ((uint64_t)slo[k] << 2) + 4 <= a.n;
                        if (l0[k]) ld_sector(a.col + ((uint64_t)slo[k] << 2), w0[k]);
                    }
#pragma unroll
                    for (int k = 0; k < kProbeBatch; ++k) {
                        if (!l0[k]) continue;
                        const uint64_t x = key[k];
                        const uint32_t b0 = (w0[k][0] < x) + (w0[k][1] < x) + (w0[k][2] < x) + (w0[k][3] < x);
                        if (b0 < 4) {
                            todo[k] = false;
                            if (kSem == kSemLowerBound || pick4(w0[k], b0) == x) res[r + k] = (slo[k] << 2) + b0;
                        } else {
                            slo[k] += 1;
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < kProbeBatch; ++k) {
                    if (!todo[k]) continue;
                    bool eq = false;
                    const uint64_t lo = (uint64_t)slo[k] << 2;
                    const uint64_t hi = (((uint64_t)shi[k] + 1) << 2) < a.n ? ((uint64_t)shi[k] + 1) << 2 : a.n;
                    const uint64_t lb = lower_bound_sectors(a.col, a.n, lo, hi, key[k], kAligned, &eq);
                    if (lb < a.n && (kSem == kSemLowerBound || eq)) res[r + k] = (uint32_t)lb;
                }
            }
        }
        // probe rows are read only now, when the results are written
        uint32_t row[kProbeItems];
#pragma unroll
        for (int k = 0; k < kProbeItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kProbeBlock + threadIdx.x;
            row[k] = valid[k] ? __ldcs(a.prows + i) : 0u;
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
static_assert(kProbeItems % kProbeBatch == 0, "whole batches per tile");

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

// directory buckets: about four per 32-byte sector of the column (2^B >= n):
// 10.64 against 10.90 ms per 2^29 probes into 2^28 keys with two per sector
// (the second sector is needed less often), 12.27 with one.
// GJ_DIR_BITS_DELTA (tuning builds) shifts it by powers of two
#ifndef GJ_DIR_BITS_DELTA
#define GJ_DIR_BITS_DELTA 1
#endif
uint32_t dir_bits_for(uint64_t n) {
    uint32_t b = 4;
    while (b < kMaxDirBits && (1ull << b) < n / 2) ++b;
    const int d = (int)b + GJ_DIR_BITS_DELTA;
    return d < 4 ? 4u : d > (int)kMaxDirBits ? kMaxDirBits : (uint32_t)d;
}

struct partitioned_layout {
    uint64_t window;
    uint32_t radix_bits;
    uint32_t dir_bits;
    uint64_t dir_entries;  // buckets + 1
    uint64_t scan_tiles;
};

partitioned_layout layout_for(const gj_index* idx, uint64_t window, uint32_t radix_bits) {
    partitioned_layout L;
    L.window = window;
    L.radix_bits = radix_bits;
    L.dir_bits = dir_bits_for(idx->n);
    L.dir_entries = (1ull << L.dir_bits) + 4;  // the closing entry, then padding to whole 16-byte groups
    L.scan_tiles = (L.dir_entries + kScanTile - 1) / kScanTile;
    return L;
}

size_t partitioned_ws_bytes(const partitioned_layout& L, int sm_count, bool prepared) {
    const uint64_t w = L.window;
    return workspace_carver::need({w * sizeof(uint64_t), w * sizeof(uint32_t),
                                   partition_ws_bytes(w, L.radix_bits, sm_count),
                                   prepared ? 0 : L.dir_entries * sizeof(uint32_t),
                                   prepared ? 0 : L.scan_tiles * sizeof(uint32_t)});
}

template <int kSem, bool kAligned>
int launch_probe(const probe_args& a, cudaStream_t s) {
    const uint64_t grid = (a.len + kChunk - 1) / kChunk;
    k_part_probe<kSem, kAligned><<<(unsigned)grid, kProbeBlock, 0, s>>>(a);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

int dispatch_probe(int sem, bool aligned, const probe_args& a, cudaStream_t s) {
    if (sem == kSemNone) return launch_probe<kSemNone, true>(a, s);
    if (sem == kSemExact) return aligned ? launch_probe<kSemExact, true>(a, s) : launch_probe<kSemExact, false>(a, s);
    return aligned ? launch_probe<kSemLowerBound, true>(a, s) : launch_probe<kSemLowerBound, false>(a, s);
}

// the directory of an index into dir (L.dir_entries entries)
int build_directory(const gj_index* idx, const partitioned_layout& L, uint32_t* dir, uint32_t* tiles,
                    cudaStream_t s) {
    dir_geom g;
    g.min_key = idx->min_key;
    g.shift = shift_for(idx->min_key, idx->max_key, L.dir_bits);
    g.buckets = 1u << L.dir_bits;
    const uint64_t n = idx->n;
    GJ_CUDA_TRY(cudaMemsetAsync(dir, 0, L.dir_entries * sizeof(uint32_t), s));
    const uint64_t per_block = (uint64_t)kDirBlock * kDirPer;
    k_dir_mark<<<(unsigned)((n + 1 + per_block - 1) / per_block), kDirBlock, 0, s>>>(idx->d_col, n, g, dir);
    GJ_CUDA_TRY(cudaGetLastError());
    k_dir_max_tiles<<<(unsigned)L.scan_tiles, kScanBlock, 0, s>>>(dir, L.dir_entries, tiles);
    GJ_CUDA_TRY(cudaGetLastError());
    k_dir_max_prefix<<<1, kScanBlock, 0, s>>>(tiles, (uint32_t)L.scan_tiles);
    GJ_CUDA_TRY(cudaGetLastError());
    k_dir_max_apply<<<(unsigned)L.scan_tiles, kScanBlock, 0, s>>>(dir, L.dir_entries, tiles);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
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
    *bytes = partitioned_ws_bytes(layout_for(index, window_size, radix_bits), di.sm_count, index->pdir != nullptr);
    return GJ_OK;
}

int gj_index_prepare_partitioned(gj_index* index, void* stream) {
    GJ_CHECK_ARG(index, "gj_index_prepare_partitioned: null index");
    if (index->pdir || semantics_of(index) == kSemNone) return GJ_OK;
    const partitioned_layout L = layout_for(index, 1, 8);
    void* dir = nullptr;
    void* tiles = nullptr;
    GJ_TRY(device_alloc_for(index, L.dir_entries * sizeof(uint32_t), &dir));
    GJ_TRY(device_alloc_for(index, L.scan_tiles * sizeof(uint32_t), &tiles));
    cudaStream_t s = as_stream(stream);
    GJ_TRY(build_directory(index, L, static_cast<uint32_t*>(dir), static_cast<uint32_t*>(tiles), s));
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    index->pdir = static_cast<const uint32_t*>(dir);
    index->pdir_bits = L.dir_bits;
    index->bytes += (L.dir_entries + L.scan_tiles) * sizeof(uint32_t);
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
    const size_t pws_bytes = partition_ws_bytes(w, radix_bits, di.sm_count);
    void* pws = wc.take<char>(pws_bytes);
    const bool prepared = index->pdir != nullptr;
    uint32_t* dir = prepared ? nullptr : wc.take<uint32_t>(L.dir_entries);
    uint32_t* tiles = prepared ? nullptr : wc.take<uint32_t>(L.scan_tiles);
    if (!pkeys || !prows || !pws || (!prepared && (!dir || !tiles))) {
        set_error("gj_partitioned_inlj: workspace of %zu bytes is smaller than the %zu required", workspace_bytes,
                  partitioned_ws_bytes(L, di.sm_count, prepared));
        return GJ_ERR_WORKSPACE;
    }
    if (d_pairs) GJ_CUDA_TRY(cudaMemsetAsync(d_count, 0, sizeof(uint64_t), s));
    if (m == 0) return GJ_OK;

    const int sem = semantics_of(index);
    if (sem != kSemNone && !prepared) GJ_TRY(build_directory(index, L, dir, tiles, s));
    const uint32_t pshift = shift_for(index->min_key, index->max_key, radix_bits);
    probe_args a;
    a.pkeys = pkeys;
    a.prows = prows;
    a.dir = prepared ? index->pdir : dir;
    a.col = index->d_col;
    a.n = index->n;
    a.g.min_key = index->min_key;
    a.g.shift = shift_for(index->min_key, index->max_key, L.dir_bits);
    a.g.buckets = 1u << L.dir_bits;
    a.positions = d_positions;
    a.pairs = reinterpret_cast<uint2*>(d_pairs);
    a.count = reinterpret_cast<unsigned long long*>(d_count);
    const bool aligned = (reinterpret_cast<uintptr_t>(index->d_col) & 31) == 0;
    for (uint64_t off = 0; off < m; off += w) {
        const uint64_t len = std::min<uint64_t>(w, m - off);
        GJ_TRY(range_partition_impl(d_probes + off, len, index->min_key, pshift, radix_bits, off, pkeys, prows,
                                    nullptr, pws, pws_bytes, s));
        a.len = len;
        GJ_TRY(dispatch_probe(sem, aligned, a, s));
    }
    return GJ_OK;
}

}  // extern "C"
