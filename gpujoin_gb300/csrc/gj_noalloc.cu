// gj_noalloc.cu -- join-pair materialisation that allocates nothing.
//
// Some callers cannot allocate device memory at the time they probe: code
// that runs inside a memory pool or arena it does not own, an embedding
// engine whose allocator is frozen after start-up, or a caller that must not
// call cudaMalloc/cudaFree on its probe path because they synchronise the
// device.  gj_inlj_pairs() needs a scratch workspace (the tile-state array
// of its single-pass compaction) that such callers cannot provide; this
// entry point runs the same kernel with its scratch in a fixed array that is
// part of the library image instead.
//
// The array lives in device memory of every GPU that loads the library until
// the process exits (GJ_NOALLOC_SCRATCH_BYTES per device).  Its device address
// is looked up once per device, on the first call made with that device
// current; make that first call before capturing a stream.  All calls share
// the array: two calls whose kernels overlap on the GPU (different streams,
// or different host threads) corrupt each other's results, so serialise them.
// The array keeps the previous call's contents; each call clears the part it
// uses before its kernel starts.
#include <cuda_runtime.h>

#include <mutex>

#include "gj_internal.h"

// scratch of the compaction: one 8-byte tile state per 2048-probe tile
// (1024 with 4 probes per thread) plus two counters, for up to
// GJ_NOALLOC_MAX_PROBES probes
#define GJ_NOALLOC_SCRATCH_BYTES (2u * 1024u * 1024u + 4096u)

static __device__ __align__(256) unsigned char g_noalloc_scratch[GJ_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[64] = {};  // device address of g_noalloc_scratch, per device ordinal

int noalloc_scratch(void** out) {
    int dev = 0;
    GJ_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        gj::set_error("gj_inlj_pairs_noalloc: device ordinal %d out of range", dev);
        return GJ_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            gj::set_error("gj_inlj_pairs_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return GJ_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return GJ_OK;
}
}  // namespace

extern "C" int gj_inlj_pairs_noalloc(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                                     uint64_t* d_count, void* stream) {
    GJ_CHECK_ARG(index && d_count, "gj_inlj_pairs_noalloc: null argument");
    GJ_CHECK_ARG(m == 0 || (d_probes && d_pairs), "gj_inlj_pairs_noalloc: null buffer");
    if (m > GJ_NOALLOC_MAX_PROBES) {
        gj::set_error("gj_inlj_pairs_noalloc: %llu probes exceed the limit of %llu per call (fixed scratch of %u bytes)",
                      (unsigned long long)m, (unsigned long long)GJ_NOALLOC_MAX_PROBES, GJ_NOALLOC_SCRATCH_BYTES);
        return GJ_ERR_TOO_LARGE;
    }
    const size_t need = gj::pairs_workspace_bytes(m);
    if (need > GJ_NOALLOC_SCRATCH_BYTES) {
        gj::set_error("gj_inlj_pairs_noalloc: %zu scratch bytes needed, %u available", need, GJ_NOALLOC_SCRATCH_BYTES);
        return GJ_ERR_TOO_LARGE;
    }
    void* scratch = nullptr;
    GJ_TRY(noalloc_scratch(&scratch));
    return gj::launch_pairs(index, d_probes, m, nullptr, d_pairs, nullptr, d_count, scratch, GJ_NOALLOC_SCRATCH_BYTES,
                            d_pairs ? d_pairs + m : nullptr, gj::as_stream(stream));
}
