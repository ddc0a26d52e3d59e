// gj_batch.cu -- batched lookup stream: many probe batches of uneven size
// against several indexes.  Not in the reference (its driver runs one index
// and one probe column per process, src/index_lookup_new.cu:375-434).
//
// mode 0: one persistent kernel.  All batches are cut into tiles; blocks
//         claim tiles in order from an atomic counter (largest-first order is
//         the caller's choice of batch order), so small batches never wait
//         behind a kernel boundary and no SM idles at batch tails.
// mode 1: one lookup launch per batch -- the baseline the persistent kernel
//         is measured against.
// Both modes can record per-batch completion times (device globaltimer) for
// latency percentiles.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "gj_internal.h"

namespace gj {
namespace {

constexpr int kBatchBlock = 256;
constexpr int kBatchItems = 8;
constexpr uint64_t kBatchTile = (uint64_t)kBatchBlock * kBatchItems;

struct any_view {
    int32_t type;
    uint32_t pad;
    union {
        bs_view bs;
        btree_view bt;
        harmonia_view hm;
        rs_view rs;
        learned_view ln;
    } u;
};

struct batch_desc {
    uint64_t offset;      // first probe of the batch
    uint64_t size;        // probes in the batch
    uint64_t tile_begin;  // first global tile of the batch
    uint32_t index;       // view of the batch
    uint32_t pad;
};

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t any_lookup(const any_view& v, uint64_t key) {
    switch (v.type) {
        case GJ_INDEX_BINARY_SEARCH: {
            bs_view b = v.u.bs;
            b.fence_slots = 0;
            return bs_lookup(b, nullptr, key);
        }
        case GJ_INDEX_BTREE:
            switch (v.u.bt.node_keys) {
                case 4: return btree_lookup<4>(v.u.bt, nullptr, key);
                case 8: return btree_lookup<8>(v.u.bt, nullptr, key);
                case 16: return btree_lookup<16>(v.u.bt, nullptr, key);
                case 32: return btree_lookup<32>(v.u.bt, nullptr, key);
                default: return btree_lookup<64>(v.u.bt, nullptr, key);
            }
        case GJ_INDEX_HARMONIA: return harmonia_lookup(v.u.hm, nullptr, key);
        case GJ_INDEX_RADIX_SPLINE: return rs_lookup(v.u.rs, key);
        case GJ_INDEX_LEARNED: return learned_lookup(v.u.ln, v.u.ln.root, key);
        default: return kInvalid;
    }
}

__global__ void __launch_bounds__(kBatchBlock) k_batch(const any_view* __restrict__ views,
                                                       const batch_desc* __restrict__ batches, uint32_t nb,
                                                       uint64_t total_tiles, const uint64_t* __restrict__ probes,
                                                       uint32_t* __restrict__ out, unsigned int* tile_counter,
                                                       unsigned long long* remaining, uint64_t* done_ns) {
    __shared__ uint32_t s_tile;
    __shared__ any_view s_view;
    __shared__ uint32_t s_batch;
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t t = atomicAdd(tile_counter, 1u);
            s_tile = t;
            if (t < total_tiles) {
                // batch owning tile t: last b with tile_begin <= t
                uint32_t lo = 0, hi = nb;
                while (hi - lo > 1) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (batches[mid].tile_begin <= t) lo = mid; else hi = mid;
                }
                s_batch = lo;
            }
        }
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= total_tiles) break;
        const uint32_t b = s_batch;
        if (threadIdx.x == 0) s_view = views[batches[b].index];
        __syncthreads();
        const batch_desc bd = batches[b];
        const uint64_t first = (tile - bd.tile_begin) * kBatchTile;
        const uint64_t last = min(bd.size, first + kBatchTile);
        for (uint64_t j = first + threadIdx.x; j < last; j += kBatchBlock) {
            const uint64_t i = bd.offset + j;
            const uint64_t key = __ldcs(reinterpret_cast<const unsigned long long*>(probes + i));
            __stcs(out + i, any_lookup(s_view, key));
        }
        __syncthreads();
        if (threadIdx.x == 0 && done_ns) {
            __threadfence();
            const unsigned long long done = last - first;
            const unsigned long long left = atomicAdd(&remaining[b], 0ull - done) - done;
            if (left == 0) done_ns[b] = globaltimer_ns();
        }
    }
}

__global__ void k_stamp(uint64_t* done_ns) { *done_ns = globaltimer_ns(); }

__global__ void k_fill_remaining(const batch_desc* __restrict__ batches, uint32_t nb, unsigned long long* remaining) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
        remaining[b] = batches[b].size;
}

}  // namespace
}  // namespace gj

using namespace gj;

extern "C" {

int gj_batch_workspace_size(uint32_t num_indexes, uint32_t num_batches, size_t* bytes) {
    GJ_CHECK_ARG(bytes, "gj_batch_workspace_size: null argument");
    *bytes = workspace_carver::need({(size_t)num_indexes * sizeof(any_view), (size_t)num_batches * sizeof(batch_desc),
                                     (size_t)num_batches * sizeof(unsigned long long), 64});
    return GJ_OK;
}

int gj_batch_lookup(gj_index* const* indexes, uint32_t num_indexes, const uint32_t* h_batch_index,
                    const uint64_t* h_probe_offset, const uint64_t* h_batch_size, uint32_t num_batches,
                    const uint64_t* d_probes, uint32_t* d_positions, uint32_t mode, uint64_t* d_batch_done_ns,
                    void* d_workspace, size_t workspace_bytes, void* stream) {
    GJ_CHECK_ARG(indexes && num_indexes > 0, "gj_batch_lookup: no indexes");
    GJ_CHECK_ARG(num_batches == 0 || (h_batch_index && h_probe_offset && h_batch_size), "gj_batch_lookup: null batch arrays");
    GJ_CHECK_ARG(mode <= 1, "gj_batch_lookup: mode must be 0 or 1");
    cudaStream_t s = as_stream(stream);
    for (uint32_t i = 0; i < num_indexes; ++i) GJ_CHECK_ARG(indexes[i], "gj_batch_lookup: null index");
    for (uint32_t b = 0; b < num_batches; ++b)
        GJ_CHECK_ARG(h_batch_index[b] < num_indexes, "gj_batch_lookup: batch refers to a missing index");
    if (num_batches == 0) return GJ_OK;
    GJ_CHECK_ARG(d_probes && d_positions, "gj_batch_lookup: null probe or output buffer");

    if (mode == 1) {
        for (uint32_t b = 0; b < num_batches; ++b) {
            GJ_TRY(launch_lookup(indexes[h_batch_index[b]], d_probes + h_probe_offset[b], h_batch_size[b],
                                 d_positions + h_probe_offset[b], s));
            if (d_batch_done_ns) k_stamp<<<1, 1, 0, s>>>(d_batch_done_ns + b);
        }
        GJ_CUDA_TRY(cudaGetLastError());
        return GJ_OK;
    }

    workspace_carver wc(d_workspace, workspace_bytes);
    any_view* d_views = wc.take<any_view>(num_indexes);
    batch_desc* d_batches = wc.take<batch_desc>(num_batches);
    unsigned long long* d_remaining = wc.take<unsigned long long>(num_batches);
    unsigned int* d_counter = wc.take<unsigned int>(16);
    if (!d_views || !d_batches || !d_remaining || !d_counter) {
        set_error("gj_batch_lookup: workspace too small");
        return GJ_ERR_WORKSPACE;
    }
    // host staging; pageable uploads return once the driver holds a copy
    static thread_local std::vector<any_view> views;
    static thread_local std::vector<batch_desc> descs;
    views.assign(num_indexes, any_view{});
    for (uint32_t i = 0; i < num_indexes; ++i) {
        const gj_index* ix = indexes[i];
        any_view& v = views[i];
        std::memset(&v, 0, sizeof(v));
        v.type = ix->type;
        switch (ix->type) {
            case GJ_INDEX_BINARY_SEARCH: v.u.bs = ix->bs; break;
            case GJ_INDEX_BTREE: v.u.bt = ix->bt; v.u.bt.cached_levels = 0; break;
            case GJ_INDEX_HARMONIA: v.u.hm = ix->hm; v.u.hm.cached_nodes = 0; v.u.hm.cached_levels = 0; break;
            case GJ_INDEX_RADIX_SPLINE: v.u.rs = ix->rs; break;
            case GJ_INDEX_LEARNED: v.u.ln = ix->ln; break;
            default: break;
        }
    }
    descs.assign(num_batches, batch_desc{});
    uint64_t tiles = 0;
    for (uint32_t b = 0; b < num_batches; ++b) {
        descs[b].offset = h_probe_offset[b];
        descs[b].size = h_batch_size[b];
        descs[b].tile_begin = tiles;
        descs[b].index = h_batch_index[b];
        tiles += (h_batch_size[b] + kBatchTile - 1) / kBatchTile;
    }
    if (tiles > (uint64_t)UINT32_MAX) {
        set_error("gj_batch_lookup: too many tiles");
        return GJ_ERR_TOO_LARGE;
    }
    GJ_CUDA_TRY(cudaMemcpyAsync(d_views, views.data(), num_indexes * sizeof(any_view), cudaMemcpyHostToDevice, s));
    GJ_CUDA_TRY(cudaMemcpyAsync(d_batches, descs.data(), num_batches * sizeof(batch_desc), cudaMemcpyHostToDevice, s));
    GJ_CUDA_TRY(cudaMemsetAsync(d_counter, 0, 16 * sizeof(unsigned int), s));
    if (d_batch_done_ns) {
        k_fill_remaining<<<(num_batches + 255) / 256, 256, 0, s>>>(d_batches, num_batches, d_remaining);
        GJ_CUDA_TRY(cudaMemsetAsync(d_batch_done_ns, 0, num_batches * sizeof(uint64_t), s));
    }
    device_info di;
    GJ_TRY(current_device_info(&di));
    int per_sm = 0;
    GJ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, kBatchBlock, 0));
    uint64_t grid = (uint64_t)di.sm_count * (per_sm > 0 ? per_sm : 1);
    if (grid > tiles) grid = tiles ? tiles : 1;
    k_batch<<<(unsigned)grid, kBatchBlock, 0, s>>>(d_views, d_batches, num_batches, tiles, d_probes, d_positions,
                                                   d_counter, d_remaining, d_batch_done_ns);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

}  // extern "C"
