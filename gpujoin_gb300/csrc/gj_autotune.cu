// gj_autotune.cu -- autotuners for the knobs of the probe path: partition
// fanout and window size of the partitioned INLJ, node and leaf width of the
// B+tree.  (The batched stream's tile shape is tuned by
// gj_batch_plan_autotune.)  Not in the reference, whose experiment_config
// takes these as command-line options (src/index_lookup_config.hpp:18-37).
//
// Every candidate is timed on the caller's data with CUDA events on the
// caller's stream (one warm-up run, then the best of `reps` timed runs) and
// the fastest is returned.  The tuners allocate their scratch and
// synchronise: they belong to set-up, not to the probe path.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "gj_internal.h"

using namespace gj;

namespace {

struct device_buffer {
    void* p = nullptr;
    ~device_buffer() { cudaFree(p); }
    int alloc(size_t bytes) {
        cudaFree(p);
        p = nullptr;
        const cudaError_t e = cudaMalloc(&p, bytes ? bytes : 1);
        if (e != cudaSuccess) {
            set_error("autotune: cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
            return GJ_ERR_OUT_OF_MEMORY;
        }
        return GJ_OK;
    }
};

struct event_pair {
    cudaEvent_t a = nullptr, b = nullptr;
    ~event_pair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    int init() {
        GJ_CUDA_TRY(cudaEventCreate(&a));
        GJ_CUDA_TRY(cudaEventCreate(&b));
        return GJ_OK;
    }
};

// best time (ms) of `reps` runs of fn after one warm-up
template <class Fn>
int time_best(Fn&& fn, cudaStream_t s, int reps, event_pair& ev, float* ms) {
    GJ_TRY(fn());
    float best = -1.f;
    for (int r = 0; r < reps; ++r) {
        GJ_CUDA_TRY(cudaEventRecord(ev.a, s));
        GJ_TRY(fn());
        GJ_CUDA_TRY(cudaEventRecord(ev.b, s));
        GJ_CUDA_TRY(cudaEventSynchronize(ev.b));
        float t = 0.f;
        GJ_CUDA_TRY(cudaEventElapsedTime(&t, ev.a, ev.b));
        if (best < 0.f || t < best) best = t;
    }
    *ms = best;
    return GJ_OK;
}

}  // namespace

extern "C" {

int gj_autotune_partitioned(const gj_index* index, const uint64_t* d_probes, uint64_t m, void* stream,
                            uint32_t* radix_bits, uint64_t* window_size, float* best_ms) {
    GJ_CHECK_ARG(index && radix_bits && window_size, "gj_autotune_partitioned: null argument");
    GJ_CHECK_ARG(m > 0 && d_probes, "gj_autotune_partitioned: no probes");
    cudaStream_t s = as_stream(stream);
    // candidates: fanout 2^5 .. 2^12 (the best partitions hold about 2^21
    // keys: measured 2^5 at 2^26 keys, 2^7-2^8 at 2^28); window = all
    // probes, a quarter, a sixteenth
    std::vector<uint64_t> windows = {m};
    if (m >= (4u << 20)) windows.push_back(m / 4);
    if (m >= (16u << 20)) windows.push_back(m / 16);
    size_t ws_max = 0;
    for (uint32_t bits = 5; bits <= 12; ++bits)
        for (uint64_t w : windows) {
            size_t need = 0;
            GJ_TRY(gj_partitioned_inlj_workspace_size(index, w, bits, &need));
            if (need > ws_max) ws_max = need;
        }
    device_buffer ws, pairs, count;
    GJ_TRY(ws.alloc(ws_max));
    GJ_TRY(pairs.alloc(2 * m * sizeof(uint32_t)));
    GJ_TRY(count.alloc(sizeof(uint64_t)));
    event_pair ev;
    GJ_TRY(ev.init());
    float best = -1.f;
    for (uint32_t bits = 5; bits <= 12; ++bits)
        for (uint64_t w : windows) {
            float t = 0.f;
            GJ_TRY(time_best(
                [&] {
                    return gj_partitioned_inlj(index, d_probes, m, w, bits, nullptr, static_cast<uint32_t*>(pairs.p),
                                               static_cast<uint64_t*>(count.p), ws.p, ws_max, stream);
                },
                s, 2, ev, &t));
            if (best < 0.f || t < best) {
                best = t;
                *radix_bits = bits;
                *window_size = w;
            }
        }
    if (best_ms) *best_ms = best;
    return GJ_OK;
}

int gj_autotune_partitioned_btree(const uint64_t* d_keys, uint64_t n, const uint64_t* d_probes, uint64_t m,
                                  void* stream, uint32_t* node_keys, uint32_t* leaf_keys, uint32_t* radix_bits,
                                  uint64_t* window_size, float* best_ms) {
    GJ_CHECK_ARG(node_keys && leaf_keys && radix_bits && window_size, "gj_autotune_partitioned_btree: null argument");
    GJ_CHECK_ARG(n > 0 && d_keys && m > 0 && d_probes, "gj_autotune_partitioned_btree: empty input");
    // Partitioned probes search the column slice of their partition through
    // the partition directory, not the tree's inner levels, so the node
    // format does not change their time: the default format is built and
    // the fanout and window are tuned for it.
    const uint32_t formats[][2] = {{kBtreeCompressed16, 4}};
    float best = -1.f;
    for (const auto& f : formats) {
        gj_index_params p;
        gj_index_params_default(&p);
        p.btree_node_keys = f[0];
        p.btree_leaf_keys = f[1];
        gj_index* ix = nullptr;
        GJ_TRY(gj_index_build(GJ_INDEX_BTREE, d_keys, nullptr, n, &p, stream, &ix));
        uint32_t bits = 0;
        uint64_t window = 0;
        float t = 0.f;
        const int rc = gj_autotune_partitioned(ix, d_probes, m, stream, &bits, &window, &t);
        gj_index_free(ix);
        GJ_TRY(rc);
        if (best < 0.f || t < best) {
            best = t;
            *node_keys = f[0];
            *leaf_keys = f[1];
            *radix_bits = bits;
            *window_size = window;
        }
    }
    if (best_ms) *best_ms = best;
    return GJ_OK;
}

int gj_autotune_ordering(const gj_index* index, const uint64_t* d_probes, uint64_t m, void* stream,
                         uint32_t* ordering, float* best_ms) {
    GJ_CHECK_ARG(index && ordering, "gj_autotune_ordering: null argument");
    GJ_CHECK_ARG(m > 0 && d_probes, "gj_autotune_ordering: no probes");
    cudaStream_t s = as_stream(stream);
    size_t ws_bytes = 0;
    GJ_TRY(gj_inlj_pairs_workspace_size(m, &ws_bytes));
    device_buffer ws, pairs, count;
    GJ_TRY(ws.alloc(ws_bytes));
    GJ_TRY(pairs.alloc(2 * m * sizeof(uint32_t)));
    GJ_TRY(count.alloc(sizeof(uint64_t)));
    event_pair ev;
    GJ_TRY(ev.init());
    float t_probe = 0.f, t_sorted = 0.f;
    GJ_TRY(time_best(
        [&] {
            return gj_inlj_pairs(index, d_probes, m, static_cast<uint32_t*>(pairs.p), static_cast<uint64_t*>(count.p),
                                 ws.p, ws_bytes, stream);
        },
        s, 2, ev, &t_probe));
    GJ_TRY(time_best(
        [&] {
            return gj_inlj_pairs_sorted(index, d_probes, m, static_cast<uint32_t*>(pairs.p),
                                        static_cast<uint64_t*>(count.p), ws.p, ws_bytes, stream);
        },
        s, 2, ev, &t_sorted));
    *ordering = t_sorted < t_probe ? GJ_ORDER_SORTED_TILES : GJ_ORDER_PROBE;
    float best = t_sorted < t_probe ? t_sorted : t_probe;
    // the partitioned INLJ in one window at the default fanout, timed as the
    // index stands (an index without its kept directory builds it per call)
    size_t pws_bytes = 0;
    GJ_TRY(gj_partitioned_inlj_workspace_size(index, m, 0, &pws_bytes));
    device_buffer pws;
    GJ_TRY(pws.alloc(pws_bytes));
    float t_part = 0.f;
    GJ_TRY(time_best(
        [&] {
            return gj_partitioned_inlj(index, d_probes, m, m, 0, nullptr, static_cast<uint32_t*>(pairs.p),
                                       static_cast<uint64_t*>(count.p), pws.p, pws_bytes, stream);
        },
        s, 2, ev, &t_part));
    if (t_part < best) {
        *ordering = GJ_ORDER_PARTITIONED;
        best = t_part;
    }
    if (best_ms) *best_ms = best;
    return GJ_OK;
}

int gj_autotune_btree(const uint64_t* d_keys, uint64_t n, const uint64_t* d_probes, uint64_t m, void* stream,
                      uint32_t* node_keys, uint32_t* leaf_keys, float* best_ms) {
    GJ_CHECK_ARG(node_keys && leaf_keys, "gj_autotune_btree: null argument");
    GJ_CHECK_ARG(n > 0 && d_keys && m > 0 && d_probes, "gj_autotune_btree: empty input");
    cudaStream_t s = as_stream(stream);
    device_buffer pos;
    GJ_TRY(pos.alloc(m * sizeof(uint32_t)));
    event_pair ev;
    GJ_TRY(ev.init());
    const uint32_t widths[] = {4, 7, 8, 15, 16};
    const uint32_t leaves[] = {4, 8, 16, 32};
    float best = -1.f;
    for (uint32_t w : widths)
        for (uint32_t l : leaves) {
            gj_index_params p;
            gj_index_params_default(&p);
            p.btree_node_keys = w;
            p.btree_leaf_keys = l;
            gj_index* ix = nullptr;
            GJ_TRY(gj_index_build(GJ_INDEX_BTREE, d_keys, nullptr, n, &p, stream, &ix));
            float t = 0.f;
            const int rc = time_best(
                [&] { return gj_index_lookup(ix, d_probes, m, static_cast<uint32_t*>(pos.p), stream); }, s, 2, ev,
                &t);
            gj_index_free(ix);
            GJ_TRY(rc);
            if (best < 0.f || t < best) {
                best = t;
                *node_keys = w;
                *leaf_keys = l;
            }
        }
    if (best_ms) *best_ms = best;
    return GJ_OK;
}

}  // extern "C"
