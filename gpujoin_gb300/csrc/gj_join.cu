// gj_join.cu -- star-join aggregate: filter the fact table on a date window,
// look the surviving foreign keys up in the dimension index, and sum
// price * (100 - discount) overall and over flagged dimension rows.
//
// Replaces ij_plain_kernel / ij_lookup_kernel + ij_join_kernel
// (src/tpch/tpch_14_ij.cu:34-85, :371-459) with the semantics of the CPU
// query (src/tpch/cpu_only.cpp:230-275): rows pass when lo <= date < hi (the
// GPU kernels of the reference test `date >= upper`, a bug not reproduced).
//
// Each block scans a tile of fact rows, compacts the rows that pass the date
// filter into shared memory (ballot + popc), and only then probes the index
// with the compacted rows, so warps stay full during the lookups (the role of
// ij_np_lane_refill_scan_lookup, src/tpch/tpch_14_ij.cu:466-566).  Sums are
// integer, so the result does not depend on the order of the atomics.
#include <cuda_runtime.h>

#include <cstdint>

#include "gj_internal.h"

namespace gj {
namespace {

constexpr int kJoinBlock = 256;
constexpr int kJoinItems = 16;
constexpr int kJoinTile = kJoinBlock * kJoinItems;

template <class Lookup>
__global__ void __launch_bounds__(kJoinBlock) k_star_join(const Lookup lookup, const uint64_t* __restrict__ dim_col,
                                                          const uint32_t* __restrict__ fk,
                                                          const uint32_t* __restrict__ date,
                                                          const int64_t* __restrict__ price,
                                                          const int64_t* __restrict__ disc, uint64_t nfact,
                                                          const uint8_t* __restrict__ flag, uint32_t lo, uint32_t hi,
                                                          unsigned long long* __restrict__ out) {
    __shared__ uint32_t s_rows[kJoinTile];
    __shared__ uint32_t s_warp[kJoinBlock / 32];
    __shared__ uint32_t s_count;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long num = 0, den = 0;
    const uint64_t tiles = (nfact + kJoinTile - 1) / kJoinTile;
    for (uint64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        const uint64_t base = t * kJoinTile;
        // 1. filter + compact (rows in tile order)
        uint32_t selected = 0;
        uint32_t local[kJoinItems];
#pragma unroll
        for (int k = 0; k < kJoinItems; ++k) {
            const uint64_t i = base + (uint64_t)k * kJoinBlock + threadIdx.x;
            bool pass = false;
            if (i < nfact) {
                const uint32_t d = __ldcs(date + i);
                pass = (d >= lo) && (d < hi);
            }
            local[k] = pass ? 1u : 0u;
            selected += local[k];
        }
        uint32_t incl = selected;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += v;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = lane < kJoinBlock / 32 ? s_warp[lane] : 0u;
            uint32_t wi = w;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, wi, d);
                if (lane >= (uint32_t)d) wi += v;
            }
            if (lane < kJoinBlock / 32) s_warp[lane] = wi - w;
            if (lane == kJoinBlock / 32 - 1) s_count = wi;
        }
        __syncthreads();
        uint32_t o = s_warp[warp] + incl - selected;
#pragma unroll
        for (int k = 0; k < kJoinItems; ++k)
            if (local[k]) s_rows[o++] = (uint32_t)(k * kJoinBlock + threadIdx.x);
        __syncthreads();
        // 2. probe the compacted rows
        const uint32_t cnt = s_count;
        for (uint32_t r = threadIdx.x; r < cnt; r += kJoinBlock) {
            const uint64_t i = base + s_rows[r];
            const uint64_t key = __ldg(fk + i);
            const uint32_t pos = lookup(key);
            if (pos != kInvalid && __ldg(reinterpret_cast<const unsigned long long*>(dim_col) + pos) == key) {
                const int64_t summand = __ldg(reinterpret_cast<const long long*>(price) + i) *
                                        (100 - __ldg(reinterpret_cast<const long long*>(disc) + i));
                den += (unsigned long long)summand;
                if (__ldg(flag + pos)) num += (unsigned long long)summand;
            }
        }
        __syncthreads();
    }
    // block reduction, one atomic per sum per block
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        num += __shfl_down_sync(0xffffffffu, num, d);
        den += __shfl_down_sync(0xffffffffu, den, d);
    }
    __shared__ unsigned long long s_num[kJoinBlock / 32], s_den[kJoinBlock / 32];
    if (lane == 0) {
        s_num[warp] = num;
        s_den[warp] = den;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a = 0, b = 0;
        for (int w = 0; w < kJoinBlock / 32; ++w) {
            a += s_num[w];
            b += s_den[w];
        }
        atomicAdd(&out[0], a);
        atomicAdd(&out[1], b);
    }
}

// The reference's pipelined order, ij_pbws (src/tpch/tpch_14_ij.cu:95-362):
// rows that pass the date filter are buffered in shared memory across the
// block's tiles until kSortBatch of them are waiting (or the rows run out);
// the batch is sorted by foreign key, probed in that order -- neighbouring
// lanes share index paths, as in the block-wise sorted probe order -- and
// aggregated.  A buffered row is (fk << 32 | row), so the sort orders by key
// (rows below 2^32).  The sums are integers and equal the unsorted kernel's.
constexpr int kSortItems = 4;
constexpr int kSortTile = kJoinBlock * kSortItems;  // rows filtered per step
constexpr int kSortBatch = 2048;                    // buffered rows that trigger a sort
constexpr int kSortCap = 4096;                      // batch + one tile, a power of two

// ascending bitonic sort of s[0, p) (p a power of two <= kSortCap) by the block
__device__ __forceinline__ void block_bitonic_sort(unsigned long long* s, uint32_t p) {
    for (uint32_t k = 2; k <= p; k <<= 1) {
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            for (uint32_t t = threadIdx.x; t < p / 2; t += kJoinBlock) {
                // the t-th pair (i, i ^ j) with bit j of i clear
                const uint32_t i = 2 * t - (t & (j - 1));
                const uint32_t l = i ^ j;
                const unsigned long long a = s[i], b = s[l];
                const bool up = (i & k) == 0;
                if ((a > b) == up) {
                    s[i] = b;
                    s[l] = a;
                }
            }
            __syncthreads();
        }
    }
}

template <class Lookup>
__global__ void __launch_bounds__(kJoinBlock) k_star_join_sorted(const Lookup lookup, const uint64_t* __restrict__ dim_col,
                                                                 const uint32_t* __restrict__ fk,
                                                                 const uint32_t* __restrict__ date,
                                                                 const int64_t* __restrict__ price,
                                                                 const int64_t* __restrict__ disc, uint64_t nfact,
                                                                 const uint8_t* __restrict__ flag, uint32_t lo,
                                                                 uint32_t hi, unsigned long long* __restrict__ out) {
    __shared__ unsigned long long s_buf[kSortCap];
    __shared__ uint32_t s_warp[kJoinBlock / 32];
    __shared__ uint32_t s_fill;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long num = 0, den = 0;
    const uint64_t tiles = (nfact + kSortTile - 1) / kSortTile;
    if (threadIdx.x == 0) s_fill = 0;
    __syncthreads();
    // the block's tiles: blockIdx.x, + gridDim.x, ...; one more round flushes
    for (uint64_t t = blockIdx.x;; t += gridDim.x) {
        const bool more = t < tiles;
        if (more) {
            // filter the tile and append the passing rows to the buffer
            const uint64_t base = t * kSortTile;
            uint32_t pass[kSortItems], selected = 0;
#pragma unroll
            for (int k = 0; k < kSortItems; ++k) {
                const uint64_t i = base + (uint64_t)k * kJoinBlock + threadIdx.x;
                bool ok = false;
                if (i < nfact) {
                    const uint32_t d = __ldcs(date + i);
                    ok = (d >= lo) && (d < hi);
                }
                pass[k] = ok ? 1u : 0u;
                selected += pass[k];
            }
            uint32_t incl = selected;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= (uint32_t)d) incl += v;
            }
            if (lane == 31) s_warp[warp] = incl;
            __syncthreads();
            if (warp == 0) {
                const uint32_t w = lane < kJoinBlock / 32 ? s_warp[lane] : 0u;
                uint32_t wi = w;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const uint32_t v = __shfl_up_sync(0xffffffffu, wi, d);
                    if (lane >= (uint32_t)d) wi += v;
                }
                if (lane < kJoinBlock / 32) s_warp[lane] = wi - w;
            }
            __syncthreads();
            uint32_t o = s_fill + s_warp[warp] + incl - selected;
#pragma unroll
            for (int k = 0; k < kSortItems; ++k) {
                if (!pass[k]) continue;
                const uint64_t i = base + (uint64_t)k * kJoinBlock + threadIdx.x;
                s_buf[o++] = ((unsigned long long)__ldg(fk + i) << 32) | (uint32_t)i;
            }
            __syncthreads();
            if (threadIdx.x == kJoinBlock - 1) s_fill = o;  // the last thread's end is the new fill
            __syncthreads();
        }
        const uint32_t fill = s_fill;
        if (fill >= (uint32_t)kSortBatch || (!more && fill > 0)) {
            // sort the batch by key (padded to a power of two with the largest value)
            uint32_t p = 1;
            while (p < fill) p <<= 1;
            for (uint32_t j = fill + threadIdx.x; j < p; j += kJoinBlock) s_buf[j] = ~0ull;
            __syncthreads();
            block_bitonic_sort(s_buf, p);
            for (uint32_t j = threadIdx.x; j < fill; j += kJoinBlock) {
                const unsigned long long e = s_buf[j];
                const uint64_t key = e >> 32, i = (uint32_t)e;
                const uint32_t pos = lookup(key);
                if (pos != kInvalid && __ldg(reinterpret_cast<const unsigned long long*>(dim_col) + pos) == key) {
                    const int64_t summand = __ldg(reinterpret_cast<const long long*>(price) + i) *
                                            (100 - __ldg(reinterpret_cast<const long long*>(disc) + i));
                    den += (unsigned long long)summand;
                    if (__ldg(flag + pos)) num += (unsigned long long)summand;
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) s_fill = 0;
            __syncthreads();
        }
        if (!more) break;
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
        num += __shfl_down_sync(0xffffffffu, num, d);
        den += __shfl_down_sync(0xffffffffu, den, d);
    }
    __shared__ unsigned long long s_num[kJoinBlock / 32], s_den[kJoinBlock / 32];
    if (lane == 0) {
        s_num[warp] = num;
        s_den[warp] = den;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a = 0, b = 0;
        for (int w = 0; w < kJoinBlock / 32; ++w) {
            a += s_num[w];
            b += s_den[w];
        }
        atomicAdd(&out[0], a);
        atomicAdd(&out[1], b);
    }
}
static_assert(kSortBatch + kSortTile <= kSortCap, "a batch plus one tile fits the buffer");

template <int W>
struct join_btree {
    btree_view v;
    __device__ __forceinline__ uint32_t operator()(uint64_t key) const { return btree_lookup<W>(v, nullptr, key); }
};
struct join_harmonia {
    harmonia_view v;
    __device__ __forceinline__ uint32_t operator()(uint64_t key) const { return harmonia_lookup(v, nullptr, key); }
};
struct join_bs {
    bs_view v;
    __device__ __forceinline__ uint32_t operator()(uint64_t key) const {
        bs_view u = v;
        u.fence_slots = 0;  // no shared cache in this kernel
        return bs_lookup(u, nullptr, key);
    }
};
struct join_rs {
    rs_view v;
    __device__ __forceinline__ uint32_t operator()(uint64_t key) const { return rs_lookup(v, key); }
};

template <class Lookup>
int run_star_join_sorted(const Lookup& l, const gj_index* idx, const uint32_t* fk, const uint32_t* date,
                         const int64_t* price, const int64_t* disc, uint64_t nfact, const uint8_t* flag, uint32_t lo,
                         uint32_t hi, int64_t* out, cudaStream_t s) {
    GJ_CUDA_TRY(cudaMemsetAsync(out, 0, 2 * sizeof(int64_t), s));
    if (nfact == 0) return GJ_OK;
    device_info di;
    GJ_TRY(current_device_info(&di));
    int per_sm = 0;
    GJ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_star_join_sorted<Lookup>, kJoinBlock, 0));
    uint64_t grid = (uint64_t)di.sm_count * (per_sm > 0 ? per_sm : 1);
    const uint64_t tiles = (nfact + kSortTile - 1) / kSortTile;
    if (grid > tiles) grid = tiles;
    k_star_join_sorted<Lookup><<<(unsigned)grid, kJoinBlock, 0, s>>>(l, idx->d_col, fk, date, price, disc, nfact, flag,
                                                                     lo, hi, reinterpret_cast<unsigned long long*>(out));
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

template <class Lookup>
int run_star_join(const Lookup& l, const gj_index* idx, const uint32_t* fk, const uint32_t* date, const int64_t* price,
                  const int64_t* disc, uint64_t nfact, const uint8_t* flag, uint32_t lo, uint32_t hi, int64_t* out,
                  cudaStream_t s, bool sorted = false) {
    if (sorted) return run_star_join_sorted(l, idx, fk, date, price, disc, nfact, flag, lo, hi, out, s);
    GJ_CUDA_TRY(cudaMemsetAsync(out, 0, 2 * sizeof(int64_t), s));
    if (nfact == 0) return GJ_OK;
    device_info di;
    GJ_TRY(current_device_info(&di));
    int per_sm = 0;
    GJ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_star_join<Lookup>, kJoinBlock, 0));
    uint64_t grid = (uint64_t)di.sm_count * (per_sm > 0 ? per_sm : 1);
    const uint64_t tiles = (nfact + kJoinTile - 1) / kJoinTile;
    if (grid > tiles) grid = tiles;
    k_star_join<Lookup><<<(unsigned)grid, kJoinBlock, 0, s>>>(l, idx->d_col, fk, date, price, disc, nfact, flag, lo, hi,
                                                             reinterpret_cast<unsigned long long*>(out));
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

}  // namespace
}  // namespace gj

using namespace gj;

namespace {
int star_join(const gj_index* dim_index, const uint32_t* d_fk, const uint32_t* d_date, const int64_t* d_price,
              const int64_t* d_discount, uint64_t nfact, const uint8_t* d_dim_flag, uint32_t lo, uint32_t hi,
              int64_t* d_out, void* stream, bool sorted) {
    GJ_CHECK_ARG(dim_index && d_out, "gj_star_join_sum: null argument");
    GJ_CHECK_ARG(nfact == 0 || (d_fk && d_date && d_price && d_discount && d_dim_flag), "gj_star_join_sum: null column");
    if (sorted && nfact > (uint64_t)UINT32_MAX) {
        set_error("gj_star_join_sum_sorted: fact rows must fit 32 bits");
        return GJ_ERR_TOO_LARGE;
    }
    cudaStream_t s = as_stream(stream);
    const gj_index* idx = dim_index;
    // this kernel stages nothing in shared memory: every level comes from global memory
    btree_view bt = idx->bt;
    bt.cached_levels = 0;
    harmonia_view hm = idx->hm;
    hm.cached_nodes = 0;
    hm.cached_levels = 0;
    switch (idx->type) {
        case GJ_INDEX_BTREE:
            return btree_dispatch(idx->bt.node_keys, [&](auto w) {
                return run_star_join(join_btree<decltype(w)::value>{bt}, idx, d_fk, d_date, d_price, d_discount,
                                     nfact, d_dim_flag, lo, hi, d_out, s, sorted);
            });
        case GJ_INDEX_HARMONIA:
            return run_star_join(join_harmonia{hm}, idx, d_fk, d_date, d_price, d_discount, nfact, d_dim_flag, lo, hi,
                                 d_out, s, sorted);
        case GJ_INDEX_BINARY_SEARCH:
            return run_star_join(join_bs{idx->bs}, idx, d_fk, d_date, d_price, d_discount, nfact, d_dim_flag, lo, hi,
                                 d_out, s, sorted);
        case GJ_INDEX_RADIX_SPLINE:
            return run_star_join(join_rs{idx->rs}, idx, d_fk, d_date, d_price, d_discount, nfact, d_dim_flag, lo, hi,
                                 d_out, s, sorted);
        default:
            set_error("gj_star_join_sum: the dimension index must be btree, harmonia, binary_search or radix_spline");
            return GJ_ERR_UNSUPPORTED;
    }
}
}  // namespace

extern "C" int gj_star_join_sum(const gj_index* dim_index, const uint32_t* d_fk, const uint32_t* d_date,
                                const int64_t* d_price, const int64_t* d_discount, uint64_t nfact,
                                const uint8_t* d_dim_flag, uint32_t lo, uint32_t hi, int64_t* d_out, void* stream) {
    return star_join(dim_index, d_fk, d_date, d_price, d_discount, nfact, d_dim_flag, lo, hi, d_out, stream, false);
}

extern "C" int gj_star_join_sum_sorted(const gj_index* dim_index, const uint32_t* d_fk, const uint32_t* d_date,
                                       const int64_t* d_price, const int64_t* d_discount, uint64_t nfact,
                                       const uint8_t* d_dim_flag, uint32_t lo, uint32_t hi, int64_t* d_out,
                                       void* stream) {
    return star_join(dim_index, d_fk, d_date, d_price, d_discount, nfact, d_dim_flag, lo, hi, d_out, stream, true);
}
