// gj_partition.cu -- range partitioning of the probe side.
//
// Replaces the fast-interconnects prefix-sum + chunked radix-partition
// kernels driven by run_on_stream (src/index_lookup_partitioning.cu:300-359).
// The reference
// partitions on key bits [max_bits - 11, max_bits) (src/index_lookup_new.cu:
// 63-67); here the partition function is a range split of the index's key
// range, partition(k) = min((k - min) >> shift, fanout - 1), so each partition
// maps onto one contiguous slice of the index and a window's lookups walk the
// index in order (the slices stay resident in the 126 MB L2).
//
// A partition pass (all on the caller's stream):
//   1. k_part_hist   per-block histograms of the keys
//   2. scan          exclusive offsets, partition-major (p, block)
//   3. k_part_scatter keys and row ids to their partition, in block order
// The windowed partitioned INLJ that drives it is in gj_partitioned.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "gj_internal.h"

namespace gj {
namespace {

constexpr int kPartBlock = 512;
constexpr uint32_t kMaxRadixBits = 12;
constexpr int kHistUnroll = 8;                                    // keys in flight per thread
// scatter geometry: block size and resident blocks per SM (its register cap)
#ifndef GJ_SCATTER_BLOCK
#define GJ_SCATTER_BLOCK 512
#endif
#ifndef GJ_SCATTER_PER_SM
#define GJ_SCATTER_PER_SM 3
#endif
constexpr int kScatterBlock = GJ_SCATTER_BLOCK;
constexpr int kScatterPerSM = GJ_SCATTER_PER_SM;
constexpr int kScatterItems = 8;                                  // keys per thread per tile
constexpr uint32_t kScatterTile = kScatterBlock * kScatterItems;

__device__ __forceinline__ uint32_t part_of(uint64_t key, uint64_t min_key, uint32_t shift, uint32_t fanout) {
    if (key <= min_key) return 0;
    const uint64_t p = (key - min_key) >> shift;
    return p >= fanout ? fanout - 1 : (uint32_t)p;
}

// sub-histograms per block: warps spread their shared-memory atomics over
// several copies when the fanout is small (fewer same-address conflicts)
__host__ __device__ __forceinline__ uint32_t hist_copies(uint32_t fanout) {
    uint32_t c = 16;  // one per warp of kPartBlock
    while (c > 1 && (size_t)c * fanout * sizeof(uint32_t) > 32768) c >>= 1;
    return c;
}

// hist[p * G + b] = number of keys of block b's chunk in partition p (kB
// threads a block: 512, or 1024 when the scatter runs one block per SM)
template <int kB>
__global__ void __launch_bounds__(kB) k_part_hist(const uint64_t* __restrict__ keys, uint64_t m, uint64_t chunk,
                                                  uint64_t min_key, uint32_t shift, uint32_t fanout,
                                                  uint64_t* __restrict__ hist) {
    extern __shared__ uint32_t s_hist[];
    const uint32_t copies = hist_copies(fanout);
    for (uint32_t p = threadIdx.x; p < fanout * copies; p += blockDim.x) s_hist[p] = 0;
    __syncthreads();
    uint32_t* mine = s_hist + ((threadIdx.x >> 5) & (copies - 1)) * fanout;
    const uint64_t b0 = blockIdx.x * chunk, b1 = min(m, b0 + chunk);
    const unsigned long long* k64 = reinterpret_cast<const unsigned long long*>(keys);
    for (uint64_t i = b0 + threadIdx.x; i < b1; i += (uint64_t)kB * kHistUnroll) {
        uint64_t k[kHistUnroll];
#pragma unroll
        for (int u = 0; u < kHistUnroll; ++u) {
            const uint64_t j = i + (uint64_t)u * kB;
            k[u] = j < b1 ? __ldcs(k64 + j) : 0ull;
        }
#pragma unroll
        for (int u = 0; u < kHistUnroll; ++u)
            if (i + (uint64_t)u * kB < b1) atomicAdd(&mine[part_of(k[u], min_key, shift, fanout)], 1u);
    }
    __syncthreads();
    for (uint32_t p = threadIdx.x; p < fanout; p += blockDim.x) {
        uint32_t c = 0;
        for (uint32_t q = 0; q < copies; ++q) c += s_hist[q * fanout + p];
        hist[(uint64_t)p * gridDim.x + blockIdx.x] = c;
    }
}

// offsets[p] = start of partition p (inclusive scan of hist, read at the
// previous partition's last block); offsets[fanout] = m
__global__ void k_part_offsets(const uint64_t* __restrict__ incl, uint32_t fanout, uint32_t nblocks, uint64_t m,
                               uint64_t* __restrict__ offsets) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p <= fanout; p += gridDim.x * blockDim.x)
        offsets[p] = p == 0 ? 0 : (p == fanout ? m : incl[(uint64_t)p * nblocks - 1]);
}

// out[p] = sum of in[0..p) over count entries, by the whole block of kB threads
template <int kB>
__device__ __forceinline__ void block_exclusive_scan(const uint32_t* in, uint32_t* out, uint32_t count) {
    __shared__ uint32_t s_warp[kB / 32];
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t per = (count + kB - 1) / kB;
    const uint32_t begin = threadIdx.x * per;
    uint32_t sum = 0;
    for (uint32_t q = 0; q < per; ++q)
        if (begin + q < count) sum += in[begin + q];
    uint32_t incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= (uint32_t)d) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        constexpr int kWarps = kB / 32;
        const uint32_t v = lane < kWarps ? s_warp[lane] : 0u;
        uint32_t w = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= (uint32_t)d) w += t;
        }
        if (lane < kWarps) s_warp[lane] = w - v;
    }
    __syncthreads();
    uint32_t run = s_warp[warp] + incl - sum;
    for (uint32_t q = 0; q < per; ++q)
        if (begin + q < count) {
            out[begin + q] = run;
            run += in[begin + q];
        }
}

// Scatter block b's chunk.  The flat (partition, block) order of the scanned
// histogram makes the start of cell c the inclusive sum of cell c - 1, so the
// keys are read once.  Each tile of kScatterTile keys is first grouped by
// partition in shared memory (a counting sort whose ranks come from
// shared-memory atomics), then every partition's run of the tile is written
// with consecutive threads on consecutive addresses: whole sectors instead of
// one scattered 8-byte store per key.  The order inside a partition follows
// the block and tile order; inside a tile it is not fixed.
// kScatterPerSM resident blocks (the register cap; about 52 KB of shared
// memory per 512-thread block for fanouts up to 2^8)
__global__ void __launch_bounds__(kScatterBlock, kScatterPerSM) k_part_scatter(const uint64_t* __restrict__ keys, uint64_t m,
                                                             uint64_t chunk, uint64_t min_key, uint32_t shift,
                                                             uint32_t fanout, const uint64_t* __restrict__ incl,
                                                             uint64_t row_base, uint64_t* __restrict__ out_keys,
                                                             uint32_t* __restrict__ out_rows) {
    extern __shared__ unsigned long long s_mem[];
    uint64_t* s_keys = reinterpret_cast<uint64_t*>(s_mem);                       // kScatterTile
    unsigned long long* s_dst = s_mem + kScatterTile;                            // fanout: next output slot
    uint32_t* s_rows = reinterpret_cast<uint32_t*>(s_dst + fanout);              // kScatterTile
    uint32_t* s_cnt = s_rows + kScatterTile;                                     // fanout
    uint32_t* s_start = s_cnt + fanout;                                          // fanout
    unsigned long long* s_delta = reinterpret_cast<unsigned long long*>(s_start + fanout);  // fanout
    for (uint32_t p = threadIdx.x; p < fanout; p += blockDim.x) {
        const uint64_t cell = (uint64_t)p * gridDim.x + blockIdx.x;
        s_dst[p] = cell == 0 ? 0ull : incl[cell - 1];
    }
    const unsigned long long* k64 = reinterpret_cast<const unsigned long long*>(keys);
    const uint64_t b0 = blockIdx.x * chunk, b1 = min(m, b0 + chunk);
    static_assert(kScatterTile <= (1u << 13) && (1u << kMaxRadixBits) <= (1u << 19), "slot packing");
    for (uint64_t t0 = b0; t0 < b1; t0 += kScatterTile) {
        const uint32_t tn = b1 - t0 < kScatterTile ? (uint32_t)(b1 - t0) : kScatterTile;
        for (uint32_t p = threadIdx.x; p < fanout; p += blockDim.x) s_cnt[p] = 0;
        __syncthreads();
        uint64_t key[kScatterItems];
        uint32_t slot[kScatterItems];  // partition << 13 | rank inside the tile's partition run
#pragma unroll
        for (int k = 0; k < kScatterItems; ++k) {
            const uint32_t j = k * kScatterBlock + threadIdx.x;
            key[k] = j < tn ? __ldcs(k64 + t0 + j) : 0ull;
        }
#pragma unroll
        for (int k = 0; k < kScatterItems; ++k) {
            const uint32_t j = k * kScatterBlock + threadIdx.x;
            const uint32_t p = part_of(key[k], min_key, shift, fanout);
            slot[k] = j < tn ? (p << 13) | atomicAdd(&s_cnt[p], 1u) : 0u;
        }
        __syncthreads();
        block_exclusive_scan<kScatterBlock>(s_cnt, s_start, fanout);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kScatterItems; ++k) {
            const uint32_t j = k * kScatterBlock + threadIdx.x;
            if (j < tn) {
                const uint32_t q = s_start[slot[k] >> 13] + (slot[k] & ((1u << 13) - 1));
                s_keys[q] = key[k];
                s_rows[q] = (uint32_t)(row_base + t0 + j);
            }
        }
        // output index of the tile's j-th sorted key = s_delta[p] + j
        for (uint32_t p = threadIdx.x; p < fanout; p += blockDim.x) s_delta[p] = s_dst[p] - s_start[p];
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < tn; j += kScatterBlock) {
            const uint64_t k = s_keys[j];
            const uint64_t d = s_delta[part_of(k, min_key, shift, fanout)] + j;
            __stcg(reinterpret_cast<unsigned long long*>(out_keys) + d, (unsigned long long)k);
            __stcg(out_rows + d, s_rows[j]);
        }
        __syncthreads();
        for (uint32_t p = threadIdx.x; p < fanout; p += blockDim.x) s_dst[p] += s_cnt[p];
        __syncthreads();
    }
}

size_t scatter_smem_bytes(uint32_t fanout) {
    return (size_t)kScatterTile * (sizeof(uint64_t) + sizeof(uint32_t)) + (size_t)fanout * (8 + 4 + 4 + 8);
}

// The scatter for fanouts of 2^8 and more: the same counting sort per tile,
// with tiles large enough that a partition's run in a tile covers whole
// sectors (8192 keys: 32 a partition at 2^8, 8 at 2^10, 2 at 2^12), one
// 1024-thread block per SM, and the next tile's keys loaded into registers
// while the current tile is sorted and written (measured at fanout 2^8:
// 11.33 against 12.46 ms for the partitioned step with the 4K-tile kernel).  A key's place in the tile
// is kept as a 16-bit offset (its row is row_base + tile start + offset).
// fanout from which the wide scatter runs; GJ_WIDE_RADIX_BITS overrides it
// in tuning builds
#ifndef GJ_WIDE_RADIX_BITS
#define GJ_WIDE_RADIX_BITS 8
#endif
constexpr uint32_t kWideRadixBits = GJ_WIDE_RADIX_BITS;
// the sorted tile keeps each key's partition beside its offset (one 32-bit
// word), so the write pass reads it instead of recomputing it from the key
// (1); GJ_SCATTER_META=0 recomputes it
#ifndef GJ_SCATTER_META
#define GJ_SCATTER_META 1
#endif
// block size, resident blocks per SM and the register prefetch of the next
// tile (one 1024-thread block with the prefetch measured fastest: 10.63 ms
// per partitioned step of 2^29 probes, against 11.71 for two 1024-thread
// blocks without it and 11.18 / 12.47 for two 768-thread blocks without /
// with it); GJ_WIDE_BLOCK / GJ_WIDE_PER_SM / GJ_WIDE_PREFETCH override them
// in tuning builds
#ifndef GJ_WIDE_BLOCK
#define GJ_WIDE_BLOCK 1024
#endif
#ifndef GJ_WIDE_PER_SM
#define GJ_WIDE_PER_SM 1
#endif
#ifndef GJ_WIDE_PREFETCH
#define GJ_WIDE_PREFETCH 1
#endif
constexpr int kWideBlock = GJ_WIDE_BLOCK;
constexpr int kWidePerSM = GJ_WIDE_PER_SM;
constexpr int kWideItems = 8;
constexpr uint32_t kWideTile = kWideBlock * kWideItems;

__global__ void __launch_bounds__(kWideBlock, kWidePerSM) k_part_scatter_wide(const uint64_t* __restrict__ keys, uint64_t m,
                                                                     uint64_t chunk, uint64_t min_key, uint32_t shift,
                                                                     uint32_t fanout, const uint64_t* __restrict__ incl,
                                                                     uint64_t row_base, uint64_t* __restrict__ out_keys,
                                                                     uint32_t* __restrict__ out_rows) {
    extern __shared__ unsigned long long s_mem[];
    uint64_t* s_keys = reinterpret_cast<uint64_t*>(s_mem);             // kWideTile
    unsigned long long* s_dst = s_mem + kWideTile;                     // fanout: next output slot
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_dst + fanout);     // fanout
    uint32_t* s_start = s_cnt + fanout;                                // fanout
    unsigned long long* s_delta = reinterpret_cast<unsigned long long*>(s_start + fanout);  // fanout
#if GJ_SCATTER_META
    uint32_t* s_meta = reinterpret_cast<uint32_t*>(s_delta + fanout);  // kWideTile: partition << 16 | offset
#else
    uint16_t* s_off = reinterpret_cast<uint16_t*>(s_delta + fanout);   // kWideTile
#endif
    for (uint32_t p = threadIdx.x; p < fanout; p += kWideBlock) {
        const uint64_t cell = (uint64_t)p * gridDim.x + blockIdx.x;
        s_dst[p] = cell == 0 ? 0ull : incl[cell - 1];
        s_cnt[p] = 0;
    }
    const unsigned long long* k64 = reinterpret_cast<const unsigned long long*>(keys);
    const uint64_t b0 = blockIdx.x * chunk, b1 = min(m, b0 + chunk);
    static_assert(kWideTile <= (1u << 13) && (1u << kMaxRadixBits) <= (1u << 19), "slot packing");
    static_assert(kWideTile <= (1u << 16) && (1u << kMaxRadixBits) <= (1u << 16), "16-bit tile offsets and partitions");
#if GJ_WIDE_PREFETCH
    uint64_t next[kWideItems];
#pragma unroll
    for (int k = 0; k < kWideItems; ++k) {
        const uint64_t i = b0 + (uint64_t)k * kWideBlock + threadIdx.x;
        next[k] = i < b1 ? __ldcs(k64 + i) : 0ull;
    }
#endif
    __syncthreads();
    for (uint64_t t0 = b0; t0 < b1; t0 += kWideTile) {
        const uint32_t tn = b1 - t0 < kWideTile ? (uint32_t)(b1 - t0) : kWideTile;
        uint64_t key[kWideItems];
#if GJ_WIDE_PREFETCH
#pragma unroll
        for (int k = 0; k < kWideItems; ++k) key[k] = next[k];
        const uint64_t t1 = t0 + kWideTile;
#pragma unroll
        for (int k = 0; k < kWideItems; ++k) {
            const uint64_t i = t1 + (uint64_t)k * kWideBlock + threadIdx.x;
            next[k] = i < b1 ? __ldcs(k64 + i) : 0ull;
        }
#else
#pragma unroll
        for (int k = 0; k < kWideItems; ++k) {
            const uint64_t i = t0 + (uint64_t)k * kWideBlock + threadIdx.x;
            key[k] = i < b1 ? __ldcs(k64 + i) : 0ull;
        }
#endif
        uint32_t slot[kWideItems];  // partition << 13 | rank inside the tile's partition run
#pragma unroll
        for (int k = 0; k < kWideItems; ++k) {
            const uint32_t j = k * kWideBlock + threadIdx.x;
            const uint32_t p = part_of(key[k], min_key, shift, fanout);
            slot[k] = j < tn ? (p << 13) | atomicAdd(&s_cnt[p], 1u) : 0u;
        }
        __syncthreads();
        block_exclusive_scan<kWideBlock>(s_cnt, s_start, fanout);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kWideItems; ++k) {
            const uint32_t j = k * kWideBlock + threadIdx.x;
            if (j < tn) {
                const uint32_t q = s_start[slot[k] >> 13] + (slot[k] & ((1u << 13) - 1));
                s_keys[q] = key[k];
#if GJ_SCATTER_META
                s_meta[q] = ((slot[k] >> 13) << 16) | j;
#else
                s_off[q] = (uint16_t)j;
#endif
            }
        }
        // output index of the tile's j-th sorted key = s_delta[p] + j
        for (uint32_t p = threadIdx.x; p < fanout; p += kWideBlock) s_delta[p] = s_dst[p] - s_start[p];
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < tn; j += kWideBlock) {
            const uint64_t k = s_keys[j];
#if GJ_SCATTER_META
            // the partition and the tile offset were stored with the key
            const uint32_t meta = s_meta[j];
            const uint64_t d = s_delta[meta >> 16] + j;
            __stcg(reinterpret_cast<unsigned long long*>(out_keys) + d, (unsigned long long)k);
            __stcg(out_rows + d, (uint32_t)(row_base + t0 + (meta & 0xFFFFu)));
#else
            const uint64_t d = s_delta[part_of(k, min_key, shift, fanout)] + j;
            __stcg(reinterpret_cast<unsigned long long*>(out_keys) + d, (unsigned long long)k);
            __stcg(out_rows + d, (uint32_t)(row_base + t0 + s_off[j]));
#endif
        }
        __syncthreads();
        for (uint32_t p = threadIdx.x; p < fanout; p += kWideBlock) {
            s_dst[p] += s_cnt[p];
            s_cnt[p] = 0;
        }
        __syncthreads();
    }
}

size_t scatter_wide_smem_bytes(uint32_t fanout) {
    return (size_t)kWideTile * (sizeof(uint64_t) + (GJ_SCATTER_META ? sizeof(uint32_t) : sizeof(uint16_t))) +
           (size_t)fanout * (8 + 4 + 4 + 8);
}

struct partition_plan {
    uint32_t fanout, nblocks;
    uint64_t chunk;
    bool wide;
};

partition_plan plan_partition(uint64_t m, uint32_t radix_bits, int sm_count) {
    partition_plan pl;
    pl.fanout = 1u << radix_bits;
    pl.wide = radix_bits >= kWideRadixBits;
    // the scatter kernel's resident blocks
    uint64_t nb = (uint64_t)sm_count * (pl.wide ? kWidePerSM : kScatterPerSM);
    const uint64_t min_chunk = 4096;
    if (nb * min_chunk > m) nb = std::max<uint64_t>(1, (m + min_chunk - 1) / min_chunk);
    pl.chunk = (m + nb - 1) / nb;
    pl.nblocks = (uint32_t)((m + pl.chunk - 1) / pl.chunk);
    if (pl.nblocks == 0) pl.nblocks = 1;
    return pl;
}

}  // namespace

size_t partition_ws_bytes(uint64_t m, uint32_t radix_bits, int sm_count) {
    const partition_plan pl = plan_partition(m ? m : 1, radix_bits, sm_count);
    const uint64_t cells = (uint64_t)pl.fanout * pl.nblocks;
    return workspace_carver::need({cells * sizeof(uint64_t), scan_workspace_bytes(cells)});
}

int range_partition_impl(const uint64_t* d_keys, uint64_t m, uint64_t min_key, uint32_t shift, uint32_t radix_bits,
                         uint64_t row_base, uint64_t* d_out_keys, uint32_t* d_out_rows, uint64_t* d_offsets, void* ws,
                         size_t ws_bytes, cudaStream_t s) {
    device_info di;
    GJ_TRY(current_device_info(&di));
    const partition_plan pl = plan_partition(m ? m : 1, radix_bits, di.sm_count);
    const uint64_t cells = (uint64_t)pl.fanout * pl.nblocks;
    workspace_carver wc(ws, ws_bytes);
    uint64_t* hist = wc.take<uint64_t>(cells);
    void* scan_ws = wc.take<char>(scan_workspace_bytes(cells));
    if (!hist || !scan_ws) {
        set_error("range partition: workspace of %zu bytes is smaller than the %zu required", ws_bytes,
                  partition_ws_bytes(m, radix_bits, di.sm_count));
        return GJ_ERR_WORKSPACE;
    }
    if (m == 0) {
        if (d_offsets) GJ_CUDA_TRY(cudaMemsetAsync(d_offsets, 0, ((size_t)pl.fanout + 1) * sizeof(uint64_t), s));
        return GJ_OK;
    }
    const size_t smem_hist = (size_t)pl.fanout * hist_copies(pl.fanout) * sizeof(uint32_t);
    const size_t smem_scatter = pl.wide ? scatter_wide_smem_bytes(pl.fanout) : scatter_smem_bytes(pl.fanout);
    if (smem_scatter > 48 * 1024) {
        if (pl.wide)
            GJ_CUDA_TRY(cudaFuncSetAttribute(k_part_scatter_wide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem_scatter));
        else
            GJ_CUDA_TRY(cudaFuncSetAttribute(k_part_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem_scatter));
    }
    if (pl.wide)
        k_part_hist<kWideBlock><<<pl.nblocks, kWideBlock, smem_hist, s>>>(d_keys, m, pl.chunk, min_key, shift,
                                                                          pl.fanout, hist);
    else
        k_part_hist<kPartBlock><<<pl.nblocks, kPartBlock, smem_hist, s>>>(d_keys, m, pl.chunk, min_key, shift,
                                                                          pl.fanout, hist);
    GJ_CUDA_TRY(cudaGetLastError());
    GJ_TRY(inclusive_scan_sum(hist, cells, scan_ws, scan_workspace_bytes(cells), s));
    if (d_offsets) {
        k_part_offsets<<<(pl.fanout + 256) / 256, 256, 0, s>>>(hist, pl.fanout, pl.nblocks, m, d_offsets);
        GJ_CUDA_TRY(cudaGetLastError());
    }
    if (pl.wide)
        k_part_scatter_wide<<<pl.nblocks, kWideBlock, smem_scatter, s>>>(d_keys, m, pl.chunk, min_key, shift, pl.fanout,
                                                                         hist, row_base, d_out_keys, d_out_rows);
    else
        k_part_scatter<<<pl.nblocks, kScatterBlock, smem_scatter, s>>>(d_keys, m, pl.chunk, min_key, shift, pl.fanout,
                                                                    hist, row_base, d_out_keys, d_out_rows);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

// key range used by the partitioned INLJ for an index (recorded at build)
void index_key_range(const gj_index* idx, uint64_t* min_key, uint64_t* max_key) {
    *min_key = idx->min_key;
    *max_key = idx->max_key;
}

uint32_t default_radix_bits(uint64_t n) {
    // about 2^20 index keys (8 MB of column, 4 MB of directory) per partition,
    // fanout within [2^5, 2^12]: a partition's slices stay in L2 while it is
    // probed, and the scatter's runs stay long (measured best: 2^5-2^6 at
    // 2^26 keys, 2^7-2^8 at 2^28)
    uint32_t b = 5;
    while (b < kMaxRadixBits && (n >> b) > (1ull << 20)) ++b;
    return b;
}

uint32_t shift_for(uint64_t min_key, uint64_t max_key, uint32_t radix_bits) {
    const uint64_t range = max_key - min_key;
    const unsigned used = range ? 64u - (unsigned)__builtin_clzll(range) : 0u;
    return used > radix_bits ? used - radix_bits : 0u;
}

}  // namespace gj

using namespace gj;

extern "C" {

int gj_partition_workspace_size(uint64_t m, uint32_t radix_bits, size_t* bytes) {
    GJ_CHECK_ARG(bytes, "gj_partition_workspace_size: null argument");
    GJ_CHECK_ARG(radix_bits >= 1 && radix_bits <= kMaxRadixBits, "gj_partition_workspace_size: radix_bits not in [1, 12]");
    device_info di;
    GJ_TRY(current_device_info(&di));
    *bytes = partition_ws_bytes(m, radix_bits, di.sm_count);
    return GJ_OK;
}

int gj_range_partition(const uint64_t* d_keys, uint64_t m, uint64_t min_key, uint32_t shift, uint32_t radix_bits,
                       uint64_t* d_out_keys, uint32_t* d_out_rows, uint64_t* d_offsets, void* d_workspace,
                       size_t workspace_bytes, void* stream) {
    GJ_CHECK_ARG(radix_bits >= 1 && radix_bits <= kMaxRadixBits, "gj_range_partition: radix_bits not in [1, 12]");
    GJ_CHECK_ARG(m == 0 || (d_keys && d_out_keys && d_out_rows), "gj_range_partition: null buffer");
    GJ_CHECK_ARG(shift < 64, "gj_range_partition: shift must be < 64");
    if (m > (uint64_t)UINT32_MAX) {
        set_error("gj_range_partition: row ids must fit 32 bits");
        return GJ_ERR_TOO_LARGE;
    }
    return range_partition_impl(d_keys, m, min_key, shift, radix_bits, 0, d_out_keys, d_out_rows, d_offsets,
                                d_workspace, workspace_bytes, as_stream(stream));
}

int gj_partitioned_lookup(const gj_index* index, const uint64_t* d_part_keys, const uint32_t* d_part_rows, uint64_t m,
                          uint32_t* d_positions, void* stream) {
    GJ_CHECK_ARG(index, "gj_partitioned_lookup: null index");
    GJ_CHECK_ARG(m == 0 || (d_part_keys && d_part_rows && d_positions), "gj_partitioned_lookup: null buffer");
    return launch_scatter_lookup(index, d_part_keys, d_part_rows, m, d_positions, as_stream(stream));
}

}  // extern "C"
