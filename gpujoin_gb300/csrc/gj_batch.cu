// gj_batch.cu -- batched lookup stream: many probe batches of uneven size
// against several indexes.  Not in the reference (its driver runs one index
// and one probe column per process, src/index_lookup_new.cu:375-434).
//
// A plan (gj_batch_plan) holds the batch descriptors, the index views and a
// tile -> batch map in device memory, uploaded once when the plan is made.
// Running a plan only enqueues device work on the caller's stream -- a memset
// and kernels, no host synchronisation and no allocation -- so it can be
// captured in a CUDA graph; the plan captures and replays one itself
// (gj_batch_plan_run_graph).
//
// mode 0: one persistent kernel.  All batches are cut into tiles of
//         kBatchBlock * tile_items probes; blocks claim tiles in order from an
//         atomic counter, so small batches never wait behind a kernel
//         boundary and no SM idles at batch tails.
// mode 1: one lookup launch per batch -- the baseline the persistent kernel
//         is measured against.
// Both modes can record per-batch completion times (device globaltimer) for
// latency percentiles.  The tile shape is the plan's autotuned parameter.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <new>
#include <type_traits>
#include <vector>

#include "gj_internal.h"

namespace gj {
namespace {

constexpr int kBatchBlock = 256;

struct any_view {
    int32_t type;
    uint32_t pad;
    union {
        bs_view bs;
        btree_view bt;
        harmonia_view hm;
        rs_view rs;
        learned_view ln;
        hash_view hs;
    } u;
};
static_assert(sizeof(any_view) % 4 == 0, "views are staged as 32-bit words");

struct batch_desc {
    uint64_t offset;      // first probe of the batch
    uint64_t size;        // probes in the batch
    uint64_t tile_begin;  // first tile of the batch
    uint32_t index;       // view of the batch
    uint32_t pad;
};

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t any_lookup(const any_view& v, const float* root, uint64_t key) {
    switch (v.type) {
        case GJ_INDEX_BINARY_SEARCH: return bs_lookup(v.u.bs, nullptr, key);
        case GJ_INDEX_BTREE:
            switch (v.u.bt.node_keys) {
                case 4: return btree_lookup<4>(v.u.bt, nullptr, key);
                case 7: return btree_lookup<7>(v.u.bt, nullptr, key);
                case 8: return btree_lookup<8>(v.u.bt, nullptr, key);
                case 15: return btree_lookup<15>(v.u.bt, nullptr, key);
                case 16: return btree_lookup<16>(v.u.bt, nullptr, key);
                case 32: return btree_lookup<32>(v.u.bt, nullptr, key);
                default: return btree_lookup<64>(v.u.bt, nullptr, key);
            }
        case GJ_INDEX_HARMONIA: return harmonia_lookup(v.u.hm, nullptr, key);
        case GJ_INDEX_RADIX_SPLINE: return rs_lookup(v.u.rs, key);
        case GJ_INDEX_LEARNED: return learned_lookup(v.u.ln, root, key);
        case GJ_INDEX_HASH: return hash_lookup(v.u.hs, key);
        default: return kInvalid;
    }
}

// The block stages the view of its tile's index (and a learned index's root
// parameters) in shared memory; consecutive tiles of one batch reuse them.
template <int kItems>
__global__ void __launch_bounds__(kBatchBlock) k_batch(const any_view* __restrict__ views,
                                                       const batch_desc* __restrict__ batches,
                                                       const uint32_t* __restrict__ tile_batch, uint32_t total_tiles,
                                                       const uint64_t* __restrict__ probes,
                                                       uint32_t* __restrict__ out, unsigned int* tile_counter,
                                                       unsigned long long* remaining, uint64_t* done_ns) {
    constexpr uint64_t kTile = (uint64_t)kBatchBlock * kItems;
    __shared__ uint32_t s_tile, s_batch;
    __shared__ __align__(16) any_view s_view;
    __shared__ __align__(8) float s_root[kMlpParams];
    uint32_t staged = 0xFFFFFFFFu;  // index whose view is in shared memory
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t t = atomicAdd(tile_counter, 1u);
            s_tile = t;
            if (t < total_tiles) s_batch = tile_batch[t];
        }
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= total_tiles) break;
        const batch_desc bd = batches[s_batch];
        if (bd.index != staged) {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(views + bd.index);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&s_view);
            for (uint32_t w = threadIdx.x; w < sizeof(any_view) / 4; w += kBatchBlock) dst[w] = src[w];
            __syncthreads();
            if (s_view.type == GJ_INDEX_LEARNED) {
                const uint32_t np = s_view.u.ln.root_kind == GJ_LEARNED_ROOT_MLP ? (uint32_t)kMlpParams : 2u;
                for (uint32_t w = threadIdx.x; w < np; w += kBatchBlock) s_root[w] = s_view.u.ln.root[w];
            }
            __syncthreads();
            staged = bd.index;
        }
        const uint64_t first = (tile - bd.tile_begin) * kTile;
        const uint64_t last = min(bd.size, first + kTile);
        uint64_t j = first + threadIdx.x;
        uint64_t next = j < last ? __ldcs(reinterpret_cast<const unsigned long long*>(probes + bd.offset + j)) : 0ull;
#pragma unroll 1
        for (; j < last; j += kBatchBlock) {
            const uint64_t key = next;
            if (j + kBatchBlock < last)
                next = __ldcs(reinterpret_cast<const unsigned long long*>(probes + bd.offset + j + kBatchBlock));
            __stcs(out + bd.offset + j, any_lookup(s_view, s_root, key));
        }
        __syncthreads();
        if (threadIdx.x == 0 && done_ns) {
            __threadfence();
            const unsigned long long done = last - first;
            const unsigned long long left = atomicAdd(&remaining[s_batch], 0ull - done) - done;
            if (left == 0) done_ns[s_batch] = globaltimer_ns();
        }
    }
}

__global__ void k_stamp(uint64_t* done_ns) { *done_ns = globaltimer_ns(); }

__global__ void k_fill_remaining(const batch_desc* __restrict__ batches, uint32_t nb, unsigned long long* remaining) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x)
        remaining[b] = batches[b].size;
}

// tile_batch[t] = batch owning tile t (batches own consecutive tile ranges)
__global__ void k_fill_tile_map(const batch_desc* __restrict__ batches, uint32_t nb, uint64_t tile_probes,
                                uint32_t* __restrict__ tile_batch) {
    for (uint32_t b = blockIdx.x; b < nb; b += gridDim.x) {
        const uint64_t t0 = batches[b].tile_begin;
        const uint64_t nt = (batches[b].size + tile_probes - 1) / tile_probes;
        for (uint64_t t = threadIdx.x; t < nt; t += blockDim.x) tile_batch[t0 + t] = b;
    }
}

constexpr uint32_t kTileItems[] = {2, 4, 8, 16};

template <class Fn>
int with_items(uint32_t items, Fn&& fn) {
    switch (items) {
        case 2: return fn(std::integral_constant<int, 2>{});
        case 4: return fn(std::integral_constant<int, 4>{});
        case 8: return fn(std::integral_constant<int, 8>{});
        case 16: return fn(std::integral_constant<int, 16>{});
        default: set_error("batch plan: tile items must be 2, 4, 8 or 16"); return GJ_ERR_INVALID_ARGUMENT;
    }
}

}  // namespace
}  // namespace gj

using namespace gj;

struct gj_batch_plan {
    int device = 0;
    std::vector<gj_index*> indexes;
    std::vector<uint32_t> batch_index;
    std::vector<uint64_t> offset, size;
    uint32_t num_batches = 0;
    uint32_t tile_items = 8;
    uint64_t tiles = 0;
    any_view* d_views = nullptr;
    batch_desc* d_batches = nullptr;
    uint32_t* d_tile_batch = nullptr;
    unsigned long long* d_remaining = nullptr;
    unsigned int* d_counter = nullptr;
    size_t tile_map_capacity = 0;
    int grid = 1;
    // graph cache: the last captured run
    cudaGraphExec_t exec = nullptr;
    cudaStream_t capture_stream = nullptr;
    const void* g_probes = nullptr;
    const void* g_positions = nullptr;
    const void* g_done = nullptr;
    uint32_t g_mode = 0xFFFFFFFFu;
    uint32_t g_items = 0;

    ~gj_batch_plan() {
        if (exec) cudaGraphExecDestroy(exec);
        if (capture_stream) cudaStreamDestroy(capture_stream);
        cudaFree(d_views);
        cudaFree(d_batches);
        cudaFree(d_tile_batch);
        cudaFree(d_remaining);
        cudaFree(d_counter);
    }
};

namespace {

template <class T>
int plan_alloc(T** p, size_t count) {
    GJ_CUDA_TRY(cudaMalloc(reinterpret_cast<void**>(p), (count ? count : 1) * sizeof(T)));
    return GJ_OK;
}

// descriptors and tile map for the plan's tile shape (synchronous upload)
int plan_layout(gj_batch_plan* pl, uint32_t items, cudaStream_t s) {
    const uint64_t tile_probes = (uint64_t)kBatchBlock * items;
    std::vector<batch_desc> descs(pl->num_batches);
    uint64_t tiles = 0;
    for (uint32_t b = 0; b < pl->num_batches; ++b) {
        descs[b].offset = pl->offset[b];
        descs[b].size = pl->size[b];
        descs[b].tile_begin = tiles;
        descs[b].index = pl->batch_index[b];
        descs[b].pad = 0;
        tiles += (pl->size[b] + tile_probes - 1) / tile_probes;
    }
    if (tiles > (uint64_t)UINT32_MAX) {
        set_error("batch plan: too many tiles");
        return GJ_ERR_TOO_LARGE;
    }
    if (tiles > pl->tile_map_capacity) {
        cudaFree(pl->d_tile_batch);
        pl->d_tile_batch = nullptr;
        GJ_TRY(plan_alloc(&pl->d_tile_batch, tiles));
        pl->tile_map_capacity = tiles;
    }
    GJ_CUDA_TRY(cudaMemcpyAsync(pl->d_batches, descs.data(), descs.size() * sizeof(batch_desc), cudaMemcpyHostToDevice,
                                s));
    if (pl->num_batches) {
        k_fill_tile_map<<<pl->num_batches < 4096 ? pl->num_batches : 4096, 256, 0, s>>>(pl->d_batches, pl->num_batches,
                                                                                      tile_probes, pl->d_tile_batch);
        GJ_CUDA_TRY(cudaGetLastError());
    }
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    pl->tiles = tiles;
    pl->tile_items = items;
    return with_items(items, [&](auto it) {
        constexpr int I = decltype(it)::value;
        device_info di;
        GJ_TRY(current_device_info(&di));
        int per_sm = 0;
        GJ_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<I>, kBatchBlock, 0));
        uint64_t grid = (uint64_t)di.sm_count * (per_sm > 0 ? per_sm : 1);
        if (grid > tiles) grid = tiles ? tiles : 1;
        pl->grid = (int)grid;
        return GJ_OK;
    });
}

int plan_run(gj_batch_plan* pl, const uint64_t* d_probes, uint32_t* d_positions, uint32_t mode, uint64_t* d_done,
             cudaStream_t s) {
    if (pl->num_batches == 0) return GJ_OK;
    if (d_done) {
        k_stamp<<<1, 1, 0, s>>>(d_done + pl->num_batches);  // start of the run
        GJ_CUDA_TRY(cudaGetLastError());
    }
    if (mode == 1) {
        for (uint32_t b = 0; b < pl->num_batches; ++b) {
            GJ_TRY(launch_lookup(pl->indexes[pl->batch_index[b]], d_probes + pl->offset[b], pl->size[b],
                                 d_positions + pl->offset[b], s));
            if (d_done) k_stamp<<<1, 1, 0, s>>>(d_done + b);
        }
        GJ_CUDA_TRY(cudaGetLastError());
        return GJ_OK;
    }
    GJ_CUDA_TRY(cudaMemsetAsync(pl->d_counter, 0, sizeof(unsigned int), s));
    if (d_done) {
        k_fill_remaining<<<(pl->num_batches + 255) / 256, 256, 0, s>>>(pl->d_batches, pl->num_batches,
                                                                     pl->d_remaining);
        GJ_CUDA_TRY(cudaMemsetAsync(d_done, 0, pl->num_batches * sizeof(uint64_t), s));
    }
    return with_items(pl->tile_items, [&](auto it) {
        constexpr int I = decltype(it)::value;
        k_batch<I><<<pl->grid, kBatchBlock, 0, s>>>(pl->d_views, pl->d_batches, pl->d_tile_batch,
                                                   (uint32_t)pl->tiles, d_probes, d_positions, pl->d_counter,
                                                   pl->d_remaining, d_done);
        GJ_CUDA_TRY(cudaGetLastError());
        return GJ_OK;
    });
}

}  // namespace

extern "C" {

int gj_batch_plan_create(gj_index* const* indexes, uint32_t num_indexes, const uint32_t* h_batch_index,
                         const uint64_t* h_probe_offset, const uint64_t* h_batch_size, uint32_t num_batches,
                         uint32_t tile_items, void* stream, gj_batch_plan** plan) {
    GJ_CHECK_ARG(plan, "gj_batch_plan_create: null plan");
    *plan = nullptr;
    GJ_CHECK_ARG(indexes && num_indexes > 0, "gj_batch_plan_create: no indexes");
    GJ_CHECK_ARG(num_batches == 0 || (h_batch_index && h_probe_offset && h_batch_size),
                 "gj_batch_plan_create: null batch arrays");
    for (uint32_t i = 0; i < num_indexes; ++i) GJ_CHECK_ARG(indexes[i], "gj_batch_plan_create: null index");
    for (uint32_t b = 0; b < num_batches; ++b)
        GJ_CHECK_ARG(h_batch_index[b] < num_indexes, "gj_batch_plan_create: batch refers to a missing index");
    if (tile_items == 0) tile_items = 8;
    bool ok_items = false;
    for (uint32_t c : kTileItems) ok_items |= c == tile_items;
    GJ_CHECK_ARG(ok_items, "gj_batch_plan_create: tile_items must be 2, 4, 8 or 16");
    cudaStream_t s = as_stream(stream);
    gj_batch_plan* pl = new (std::nothrow) gj_batch_plan();
    if (!pl) {
        set_error("gj_batch_plan_create: out of host memory");
        return GJ_ERR_OUT_OF_MEMORY;
    }
    auto fail = [&](int rc) {
        delete pl;
        return rc;
    };
    cudaGetDevice(&pl->device);
    pl->indexes.assign(indexes, indexes + num_indexes);
    pl->num_batches = num_batches;
    pl->batch_index.assign(h_batch_index, h_batch_index + num_batches);
    pl->offset.assign(h_probe_offset, h_probe_offset + num_batches);
    pl->size.assign(h_batch_size, h_batch_size + num_batches);
    int rc = plan_alloc(&pl->d_views, num_indexes);
    if (rc == GJ_OK) rc = plan_alloc(&pl->d_batches, num_batches);
    if (rc == GJ_OK) rc = plan_alloc(&pl->d_remaining, num_batches);
    if (rc == GJ_OK) rc = plan_alloc(&pl->d_counter, 4);
    if (rc != GJ_OK) return fail(rc);
    std::vector<any_view> views(num_indexes);
    for (uint32_t i = 0; i < num_indexes; ++i) {
        const gj_index* ix = indexes[i];
        any_view& v = views[i];
        std::memset(&v, 0, sizeof(v));
        v.type = ix->type;
        switch (ix->type) {
            case GJ_INDEX_BINARY_SEARCH: v.u.bs = ix->bs; v.u.bs.fence_slots = 0; break;
            case GJ_INDEX_BTREE: v.u.bt = ix->bt; v.u.bt.cached_levels = 0; break;
            case GJ_INDEX_HARMONIA: v.u.hm = ix->hm; v.u.hm.cached_nodes = 0; v.u.hm.cached_levels = 0; break;
            case GJ_INDEX_RADIX_SPLINE: v.u.rs = ix->rs; break;
            case GJ_INDEX_LEARNED: v.u.ln = ix->ln; break;
            case GJ_INDEX_HASH: v.u.hs = ix->hs; break;
            default: break;
        }
    }
    if (cudaMemcpyAsync(pl->d_views, views.data(), views.size() * sizeof(any_view), cudaMemcpyHostToDevice, s) !=
        cudaSuccess) {
        set_error("gj_batch_plan_create: view upload failed");
        return fail(GJ_ERR_CUDA);
    }
    rc = plan_layout(pl, tile_items, s);
    if (rc != GJ_OK) return fail(rc);
    *plan = pl;
    return GJ_OK;
}

int gj_batch_plan_free(gj_batch_plan* plan) {
    delete plan;
    return GJ_OK;
}

int gj_batch_plan_tile_items(const gj_batch_plan* plan, uint32_t* tile_items) {
    GJ_CHECK_ARG(plan && tile_items, "gj_batch_plan_tile_items: null argument");
    *tile_items = plan->tile_items;
    return GJ_OK;
}

int gj_batch_plan_run(gj_batch_plan* plan, const uint64_t* d_probes, uint32_t* d_positions, uint32_t mode,
                      uint64_t* d_batch_done_ns, void* stream) {
    GJ_CHECK_ARG(plan, "gj_batch_plan_run: null plan");
    GJ_CHECK_ARG(mode <= 1, "gj_batch_plan_run: mode must be 0 or 1");
    GJ_CHECK_ARG(plan->num_batches == 0 || (d_probes && d_positions), "gj_batch_plan_run: null buffer");
    return plan_run(plan, d_probes, d_positions, mode, d_batch_done_ns, as_stream(stream));
}

int gj_batch_plan_run_graph(gj_batch_plan* plan, const uint64_t* d_probes, uint32_t* d_positions, uint32_t mode,
                            uint64_t* d_batch_done_ns, void* stream) {
    GJ_CHECK_ARG(plan, "gj_batch_plan_run_graph: null plan");
    GJ_CHECK_ARG(mode <= 1, "gj_batch_plan_run_graph: mode must be 0 or 1");
    GJ_CHECK_ARG(plan->num_batches == 0 || (d_probes && d_positions), "gj_batch_plan_run_graph: null buffer");
    cudaStream_t s = as_stream(stream);
    gj_batch_plan* pl = plan;
    const bool same = pl->exec && pl->g_probes == d_probes && pl->g_positions == d_positions &&
                      pl->g_done == d_batch_done_ns && pl->g_mode == mode && pl->g_items == pl->tile_items;
    if (!same) {
        if (pl->exec) {
            cudaGraphExecDestroy(pl->exec);
            pl->exec = nullptr;
        }
        if (!pl->capture_stream) GJ_CUDA_TRY(cudaStreamCreateWithFlags(&pl->capture_stream, cudaStreamNonBlocking));
        // capture on the plan's own stream: the run enqueues device work only
        GJ_CUDA_TRY(cudaStreamBeginCapture(pl->capture_stream, cudaStreamCaptureModeRelaxed));
        const int rc = plan_run(pl, d_probes, d_positions, mode, d_batch_done_ns, pl->capture_stream);
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(pl->capture_stream, &graph);
        if (rc != GJ_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (e != cudaSuccess) {
            set_error("gj_batch_plan_run_graph: capture failed: %s", cudaGetErrorString(e));
            return GJ_ERR_CUDA;
        }
        const cudaError_t ie = cudaGraphInstantiate(&pl->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            pl->exec = nullptr;
            set_error("gj_batch_plan_run_graph: instantiate failed: %s", cudaGetErrorString(ie));
            return GJ_ERR_CUDA;
        }
        pl->g_probes = d_probes;
        pl->g_positions = d_positions;
        pl->g_done = d_batch_done_ns;
        pl->g_mode = mode;
        pl->g_items = pl->tile_items;
    }
    GJ_CUDA_TRY(cudaGraphLaunch(pl->exec, s));
    return GJ_OK;
}

int gj_batch_plan_autotune(gj_batch_plan* plan, const uint64_t* d_probes, uint32_t* d_positions, void* stream,
                           uint32_t* tile_items, float* best_ms) {
    GJ_CHECK_ARG(plan, "gj_batch_plan_autotune: null plan");
    GJ_CHECK_ARG(plan->num_batches == 0 || (d_probes && d_positions), "gj_batch_plan_autotune: null buffer");
    cudaStream_t s = as_stream(stream);
    cudaEvent_t a = nullptr, b = nullptr;
    GJ_CUDA_TRY(cudaEventCreate(&a));
    GJ_CUDA_TRY(cudaEventCreate(&b));
    uint32_t best = plan->tile_items;
    float best_t = -1.f;
    int rc = GJ_OK;
    for (uint32_t items : kTileItems) {
        rc = plan_layout(plan, items, s);
        if (rc != GJ_OK) break;
        rc = plan_run(plan, d_probes, d_positions, 0, nullptr, s);  // warm
        if (rc != GJ_OK) break;
        cudaEventRecord(a, s);
        for (int r = 0; r < 3 && rc == GJ_OK; ++r) rc = plan_run(plan, d_probes, d_positions, 0, nullptr, s);
        cudaEventRecord(b, s);
        if (rc != GJ_OK || cudaEventSynchronize(b) != cudaSuccess) {
            if (rc == GJ_OK) {
                set_error("gj_batch_plan_autotune: timing failed");
                rc = GJ_ERR_CUDA;
            }
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (best_t < 0.f || ms < best_t) {
            best_t = ms;
            best = items;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc != GJ_OK) return rc;
    GJ_TRY(plan_layout(plan, best, s));
    if (tile_items) *tile_items = best;
    if (best_ms) *best_ms = best_t / 3.f;
    return GJ_OK;
}

}  // extern "C"
