// gj_lookup.cu -- probe kernels: plain lookup (positions), scattered lookup
// (partitioned relations) and join-pair materialisation with a deterministic
// single-pass compaction.
//
// Replaces lookup_kernel (src/index_lookup_common.cuh:217-245),
// partitioned_lookup_kernel (src/index_lookup_partitioning.cu:218-248) and
// ij_lookup_kernel (src/tpch/tpch_14_ij.cu:371-407).
//
// Each kernel is persistent (grid = SMs x resident blocks) and stages the
// upper part of the index (B+tree top levels, Harmonia top nodes, the sampled
// binary-search keys) into shared memory once per block.  Probe keys are
// streamed with evict-first loads, results with streaming stores.
#include <cuda_runtime.h>

#include <cstdint>

#include "gj_internal.h"

namespace gj {
namespace {

constexpr int kBlock = 256;
// resident blocks per SM the lookup kernels are compiled for (register cap)
#ifndef GJ_MIN_BLOCKS
#define GJ_MIN_BLOCKS 1
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

struct op_bs {
    bs_view v;
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const {
        return bs_lookup(v, cache, key);
    }
};
template <int W>
struct op_btree {
    btree_view v;
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const {
        return btree_lookup<W>(v, cache, key);
    }
};
struct op_harmonia {
    harmonia_view v;
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const {
        return harmonia_lookup(v, cache, key);
    }
};
struct op_rs {
    rs_view v;
    __device__ __forceinline__ uint32_t operator()(const uint64_t*, uint64_t key) const { return rs_lookup(v, key); }
};
struct op_noop {
    __device__ __forceinline__ uint32_t operator()(const uint64_t*, uint64_t) const { return kInvalid; }
};
struct op_learned {
    learned_view v;
    __device__ __forceinline__ uint32_t operator()(const uint64_t* cache, uint64_t key) const {
        return learned_lookup(v, reinterpret_cast<const float*>(cache), key);
    }
};

// the items of a thread are searched one after another: a search is a
// chain of dependent loads, and occupancy (not per-thread interleaving)
// keeps the loads of many probes in flight
template <class Op, int K>
__device__ __forceinline__ void run_items(const Op& op, const uint64_t* cache, const uint64_t (&key)[K],
                                          uint32_t (&res)[K]) {
#pragma unroll 1
    for (int k = 0; k < K; ++k) res[k] = op(cache, key[k]);
}

__device__ __forceinline__ void stage_cache(uint64_t* dst, const stage_desc& sd) {
    for (uint32_t i = threadIdx.x; i < sd.words0; i += blockDim.x) dst[i] = __ldg(reinterpret_cast<const unsigned long long*>(sd.src0) + i);
    for (uint32_t i = threadIdx.x; i < sd.words1; i += blockDim.x)
        dst[sd.words0 + i] = __ldg(reinterpret_cast<const unsigned long long*>(sd.src1) + i);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// plain lookup: out[i] = lookup(probes[i])
// ---------------------------------------------------------------------------
// A block processes tiles of kLookupItems * kBlock probes; item k of thread t
// is probe tile + k * kBlock + t (coalesced), and the kLookupItems probes of a
// thread are searched in lockstep.
#ifndef GJ_LOOKUP_ITEMS
#define GJ_LOOKUP_ITEMS 8
#endif
constexpr int kLookupItems = GJ_LOOKUP_ITEMS;

template <class Op>
__global__ void __launch_bounds__(kBlock, GJ_MIN_BLOCKS) k_lookup(const Op op, const stage_desc sd,
                                                   const uint64_t* __restrict__ probes, uint64_t m,
                                                   uint32_t* __restrict__ out) {
    extern __shared__ uint64_t cache[];
    stage_cache(cache, sd);
    constexpr uint64_t tile = (uint64_t)kLookupItems * kBlock;
    for (uint64_t t0 = (uint64_t)blockIdx.x * tile; t0 < m; t0 += (uint64_t)gridDim.x * tile) {
        uint64_t key[kLookupItems];
        uint32_t res[kLookupItems];
#pragma unroll
        for (int k = 0; k < kLookupItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
            key[k] = i < m ? __ldcs(reinterpret_cast<const unsigned long long*>(probes + i)) : 0ull;
        }
        run_items<Op, kLookupItems>(op, cache, key, res);
#pragma unroll
        for (int k = 0; k < kLookupItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
            if (i < m) __stcs(out + i, res[k]);
        }
    }
}

// scattered lookup over a partitioned relation: out[rows[i]] = lookup(keys[i])
template <class Op>
__global__ void __launch_bounds__(kBlock, GJ_MIN_BLOCKS) k_scatter_lookup(const Op op, const stage_desc sd,
                                                           const uint64_t* __restrict__ keys,
                                                           const uint32_t* __restrict__ rows, uint64_t m,
                                                           uint32_t* __restrict__ out) {
    extern __shared__ uint64_t cache[];
    stage_cache(cache, sd);
    constexpr uint64_t tile = (uint64_t)kLookupItems * kBlock;
    for (uint64_t t0 = (uint64_t)blockIdx.x * tile; t0 < m; t0 += (uint64_t)gridDim.x * tile) {
        uint64_t key[kLookupItems];
        uint32_t res[kLookupItems];
#pragma unroll
        for (int k = 0; k < kLookupItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
            key[k] = i < m ? __ldcs(reinterpret_cast<const unsigned long long*>(keys + i)) : 0ull;
        }
        run_items<Op, kLookupItems>(op, cache, key, res);
#pragma unroll
        for (int k = 0; k < kLookupItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
            if (i < m) out[__ldcs(rows + i)] = res[k];
        }
    }
}

// ---------------------------------------------------------------------------
// join pairs with decoupled look-back compaction
// ---------------------------------------------------------------------------
// Tiles of kBlock * kItems probes are claimed in order through an atomic
// counter, so every predecessor of a tile is already running when the tile
// looks back: each wait ends.  Waits are bounded anyway; on expiry the kernel
// raises the error flag (GJ_ERR_TIMEOUT on the host) and stops writing.
constexpr int kItems = GJ_LOOKUP_ITEMS;
static_assert(kItems >= 4 && (kItems & (kItems - 1)) == 0, "the pairs scan needs a power-of-two item count >= 4");
constexpr uint32_t kTile = kBlock * kItems;
constexpr unsigned long long kFlagAggregate = 1ull << 62;
constexpr unsigned long long kFlagPrefix = 2ull << 62;
constexpr unsigned long long kValueMask = (1ull << 62) - 1;
constexpr uint32_t kSpinLimit = 1u << 22;

struct pairs_ws {
    unsigned long long* tile_state;  // num_tiles
    unsigned int* tile_counter;      // 1
    unsigned int* error;             // 1
};

template <class Op>
__global__ void __launch_bounds__(kBlock, GJ_MIN_BLOCKS) k_pairs(const Op op, const stage_desc sd, const uint64_t* __restrict__ probes,
                                                  const uint32_t* __restrict__ rows, uint64_t m,
                                                  uint2* __restrict__ pairs, const uint64_t* __restrict__ d_base,
                                                  uint64_t* __restrict__ d_count, pairs_ws ws, uint32_t num_tiles) {
    extern __shared__ uint64_t cache[];
    constexpr int kWarps = kBlock / 32;
    __shared__ uint32_t s_tile;
    __shared__ uint32_t s_cnt[kItems * kWarps];
    __shared__ unsigned long long s_prefix;
    __shared__ int s_abort;
    stage_cache(cache, sd);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t base = d_base ? *d_base : 0ull;

    for (;;) {
        if (threadIdx.x == 0) {
            s_tile = atomicAdd(ws.tile_counter, 1u);
            s_abort = 0;
        }
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= num_tiles) break;
        const uint64_t t0 = (uint64_t)tile * kTile;

        // item k of thread t is probe t0 + k * kBlock + t: coalesced loads;
        // output order is probe order, i.e. (k, warp, lane) order
        uint32_t pos[kItems];
        uint32_t lane_rank[kItems];
        uint32_t flags = 0;
        uint64_t key[kItems];
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
            key[k] = i < m ? __ldcs(reinterpret_cast<const unsigned long long*>(probes + i)) : 0ull;
        }
        run_items<Op, kItems>(op, cache, key, pos);
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
            if (i >= m) pos[k] = kInvalid;
            const bool hit = pos[k] != kInvalid;
            const uint32_t ballot = __ballot_sync(0xffffffffu, hit);
            lane_rank[k] = __popc(ballot & ((1u << lane) - 1u));
            if (hit) flags |= 1u << k;
            if (lane == 0) s_cnt[k * kWarps + warp] = __popc(ballot);
        }
        __syncthreads();
        if (warp == 0) {
            // exclusive scan of the kItems * kWarps counts in (k, warp) order
            constexpr int kPerLane = kItems * kWarps / 32;
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
            if (lane == 31) {
                // publish the tile aggregate, then resolve the tile prefix
                const unsigned long long total = incl;
                unsigned long long prefix = 0;
                if (tile == 0) {
                    atomicExch(&ws.tile_state[0], kFlagPrefix | total);
                } else {
                    atomicExch(&ws.tile_state[tile], kFlagAggregate | total);
                    int64_t j = (int64_t)tile - 1;
                    uint32_t spins = 0;
                    while (j >= 0) {
                        const unsigned long long st = *reinterpret_cast<volatile unsigned long long*>(&ws.tile_state[j]);
                        const unsigned long long flag = st & ~kValueMask;
                        if (flag == 0) {
                            if (++spins > kSpinLimit) {
                                atomicExch(ws.error, 1u);
                                s_abort = 1;
                                break;
                            }
                            continue;
                        }
                        prefix += st & kValueMask;
                        if (flag == kFlagPrefix) break;
                        --j;
                    }
                    atomicExch(&ws.tile_state[tile], kFlagPrefix | (prefix + total));
                }
                s_prefix = prefix;
                if (tile == num_tiles - 1) *d_count = base + prefix + total;
            }
        }
        __syncthreads();
        if (s_abort) break;
        const uint64_t tile_base = base + s_prefix;
#pragma unroll
        for (int k = 0; k < kItems; ++k) {
            if (flags & (1u << k)) {
                const uint64_t i = t0 + (uint64_t)k * kBlock + threadIdx.x;
                const uint64_t o = tile_base + s_cnt[k * kWarps + warp] + lane_rank[k];
                const uint32_t row = rows ? __ldcs(rows + i) : (uint32_t)i;
                __stcs(reinterpret_cast<unsigned long long*>(pairs + o), ((unsigned long long)pos[k] << 32) | row);
            }
        }
        __syncthreads();
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
        case GJ_INDEX_LEARNED:
            sd.src0 = reinterpret_cast<const uint64_t*>(idx->ln.root);
            sd.words0 = idx->smem_words;
            break;
        default:
            break;
    }
    return sd;
}

size_t stage_bytes(const stage_desc& sd) { return (size_t)(sd.words0 + sd.words1) * sizeof(uint64_t); }

template <class Kernel>
int grid_for(Kernel kernel, size_t smem, uint64_t work_items, int* grid) {
    device_info di;
    GJ_TRY(current_device_info(&di));
    if (smem > 48 * 1024) GJ_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
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
    int grid = 0;
    GJ_TRY(grid_for(k_lookup<Op>, smem, (m + kLookupItems - 1) / kLookupItems, &grid));
    k_lookup<Op><<<grid, kBlock, smem, s>>>(op, sd, probes, m, out);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

template <class Op>
int run_scatter(const Op& op, const stage_desc& sd, const uint64_t* keys, const uint32_t* rows, uint64_t m,
                uint32_t* out, cudaStream_t s) {
    const size_t smem = stage_bytes(sd);
    int grid = 0;
    GJ_TRY(grid_for(k_scatter_lookup<Op>, smem, (m + kLookupItems - 1) / kLookupItems, &grid));
    k_scatter_lookup<Op><<<grid, kBlock, smem, s>>>(op, sd, keys, rows, m, out);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

template <class Op>
int run_pairs(const Op& op, const stage_desc& sd, const uint64_t* probes, const uint32_t* rows, uint64_t m,
              uint32_t* pairs, const uint64_t* d_base, uint64_t* d_count, void* ws, size_t ws_bytes, cudaStream_t s) {
    const uint32_t num_tiles = (uint32_t)((m + kTile - 1) / kTile);
    workspace_carver wc(ws, ws_bytes);
    pairs_ws pw;
    pw.tile_state = wc.take<unsigned long long>(num_tiles ? num_tiles : 1);
    pw.tile_counter = wc.take<unsigned int>(2);
    pw.error = pw.tile_counter + 1;
    if (!pw.tile_state || !pw.tile_counter) {
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
    GJ_CUDA_TRY(cudaMemsetAsync(ws, 0, wc.used, s));
    const size_t smem = stage_bytes(sd);
    int grid = 0;
    GJ_TRY(grid_for(k_pairs<Op>, smem, (uint64_t)num_tiles * kBlock, &grid));
    k_pairs<Op><<<grid, kBlock, smem, s>>>(op, sd, probes, rows, m, reinterpret_cast<uint2*>(pairs), d_base, d_count,
                                           pw, num_tiles);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

// dispatch an action over the index kind
template <class Fn>
int with_op(const gj_index* idx, Fn&& fn) {
    switch (idx->type) {
        case GJ_INDEX_BINARY_SEARCH: return fn(op_bs{idx->bs});
        case GJ_INDEX_BTREE:
            return btree_dispatch(idx->bt.node_keys, [&](auto w) { return fn(op_btree<decltype(w)::value>{idx->bt}); });
        case GJ_INDEX_HARMONIA: return fn(op_harmonia{idx->hm});
        case GJ_INDEX_RADIX_SPLINE: return fn(op_rs{idx->rs});
        case GJ_INDEX_LEARNED: return fn(op_learned{idx->ln});
        case GJ_INDEX_NO_OP: return fn(op_noop{});
        default: set_error("unknown index type %d", idx->type); return GJ_ERR_INVALID_ARGUMENT;
    }
}

}  // namespace

size_t pairs_workspace_bytes(uint64_t m) {
    const uint64_t tiles = (m + kTile - 1) / kTile;
    return workspace_carver::need({(size_t)(tiles ? tiles : 1) * 8, 8});
}

int launch_lookup(const gj_index* idx, const uint64_t* d_probes, uint64_t m, uint32_t* d_out, cudaStream_t s) {
    if (m == 0) return GJ_OK;
    const stage_desc sd = make_stage(idx);
    return with_op(idx, [&](const auto& op) { return run_lookup(op, sd, d_probes, m, d_out, s); });
}

int launch_scatter_lookup(const gj_index* idx, const uint64_t* d_keys, const uint32_t* d_rows, uint64_t m,
                          uint32_t* d_out, cudaStream_t s) {
    if (m == 0) return GJ_OK;
    const stage_desc sd = make_stage(idx);
    return with_op(idx, [&](const auto& op) { return run_scatter(op, sd, d_keys, d_rows, m, d_out, s); });
}

int launch_pairs(const gj_index* idx, const uint64_t* d_probes, uint64_t m, const uint32_t* d_rows, uint32_t* d_pairs,
                 const uint64_t* d_base, uint64_t* d_count, void* ws, size_t ws_bytes, cudaStream_t s) {
    const stage_desc sd = make_stage(idx);
    return with_op(idx, [&](const auto& op) {
        return run_pairs(op, sd, d_probes, d_rows, m, d_pairs, d_base, d_count, ws, ws_bytes, s);
    });
}

int pairs_error_flag(void* ws, size_t ws_bytes, uint64_t m, unsigned int* flag, cudaStream_t s) {
    const uint32_t num_tiles = (uint32_t)((m + kTile - 1) / kTile);
    workspace_carver wc(ws, ws_bytes);
    wc.take<unsigned long long>(num_tiles ? num_tiles : 1);
    unsigned int* ctr = wc.take<unsigned int>(2);
    if (!ctr) return GJ_ERR_WORKSPACE;
    GJ_CUDA_TRY(cudaMemcpyAsync(flag, ctr + 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    return GJ_OK;
}

}  // namespace gj
