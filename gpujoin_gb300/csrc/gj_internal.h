// gj_internal.h -- shared host-side definitions of the gpujoin GB300 library.
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <type_traits>
#include <vector>

#include "gpujoin.h"
#include "gpujoin/device.cuh"

namespace gj {

// thread-local last error (gj_last_error_string)
void set_error(const char* fmt, ...);
const char* last_error();

#define GJ_CUDA_TRY(call)                                                                   \
    do {                                                                                    \
        cudaError_t gj_e_ = (call);                                                         \
        if (gj_e_ != cudaSuccess) {                                                         \
            ::gj::set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(gj_e_),      \
                            __FILE__, __LINE__);                                            \
            return gj_e_ == cudaErrorMemoryAllocation ? GJ_ERR_OUT_OF_MEMORY : GJ_ERR_CUDA; \
        }                                                                                   \
    } while (0)

#define GJ_CHECK_ARG(cond, msg)                  \
    do {                                         \
        if (!(cond)) {                           \
            ::gj::set_error("%s", msg);          \
            return GJ_ERR_INVALID_ARGUMENT;      \
        }                                        \
    } while (0)

#define GJ_TRY(expr)                  \
    do {                              \
        int gj_rc_ = (expr);          \
        if (gj_rc_ != GJ_OK) return gj_rc_; \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// per-device properties, cached
struct device_info {
    int device = -1;
    int sm_count = 0;
    size_t smem_optin = 0;
    size_t l2_bytes = 0;
};
int current_device_info(device_info* out);

// aligned carve-out of a caller workspace
struct workspace_carver {
    char* base;
    size_t size;
    size_t used = 0;
    workspace_carver(void* b, size_t s) : base(static_cast<char*>(b)), size(s) {}
    template <class T>
    T* take(size_t count) {
        size_t off = (used + 255) & ~size_t(255);
        size_t bytes = count * sizeof(T);
        if (base == nullptr || off + bytes > size) return nullptr;
        used = off + bytes;
        return reinterpret_cast<T*>(base + off);
    }
    static size_t need(std::initializer_list<size_t> parts) {
        size_t t = 0;
        for (size_t p : parts) t = ((t + 255) & ~size_t(255)) + p;
        return t + 256;
    }
};

// host-side builders (gj_host_build.cpp)
struct harmonia_arrays {
    std::vector<uint64_t> keys;      // inner key array, 32 per inner node
    std::vector<uint64_t> children;  // per node
    std::vector<uint64_t> level_nodes;  // nodes per level, root first
    uint32_t depth = 0;
};
// returns GJ_OK or an error code (n % 32 != 0, depth limit)
int build_harmonia_arrays(const uint64_t* col, uint64_t n, harmonia_arrays* out);

struct radix_spline_arrays {
    std::vector<uint32_t> table;
    std::vector<uint64_t> sx;
    std::vector<double> sy;
    uint64_t min_key = 0, max_key = 0;
    uint32_t shift = 0;
};
int build_radix_spline(const uint64_t* col, uint64_t n, uint32_t radix_bits, uint32_t max_error,
                       radix_spline_arrays* out);

}  // namespace gj

// the index object behind the opaque handle
struct gj_index {
    int type = GJ_INDEX_NO_OP;
    uint64_t n = 0;
    int device = 0;
    const uint64_t* d_col = nullptr;
    uint64_t min_key = 0, max_key = 0;  // d_col[0], d_col[n - 1] (0 when empty)
    uint64_t bytes = 0;  // memory_consumption
    uint64_t host_bytes = 0;  // of which in pinned host memory
    gj_index_params params{};
    std::vector<void*> allocations;       // owned device memory
    std::vector<void*> host_allocations;  // owned pinned host memory (index_memory = host)

    gj::bs_view bs{};
    gj::btree_view bt{};
    gj::harmonia_view hm{};
    gj::rs_view rs{};
    gj::learned_view ln{};
    gj::hash_view hs{};
    gj::learned_root_params ln_root{};  // host copy of the root parameters (kernel arguments)
    uint64_t learned_max_error = 0;
    double learned_mean_window = 0.0;
    double learned_init_loss = 0.0;     // root MLP: sample loss of the quantile start
    double learned_trained_loss = 0.0;  // root MLP: sample loss after training

    // partition directory of the partitioned INLJ (gj_index_prepare_partitioned):
    // sector of the lower bound per key bucket, 2^pdir_bits + 4 entries, or null
    const uint32_t* pdir = nullptr;
    uint32_t pdir_bits = 0;

    size_t smem_bytes = 0;          // dynamic shared memory of the lookup kernels
    const uint64_t* smem_src = nullptr;  // device source of the staged cache
    uint32_t smem_words = 0;        // 64-bit words staged
};

namespace gj {
// lookup entry points shared between translation units (gj_lookup.cu)
int launch_lookup(const gj_index* idx, const uint64_t* d_probes, uint64_t m, uint32_t* d_out, cudaStream_t s);
int launch_sorted_lookup(const gj_index* idx, const uint64_t* d_probes, uint64_t m, uint32_t* d_out, cudaStream_t s);
int launch_scatter_lookup(const gj_index* idx, const uint64_t* d_keys, const uint32_t* d_rows, uint64_t m,
                          uint32_t* d_out, cudaStream_t s);
// Pairs are written from offset *d_base (0 if null); *d_count = base +
// matches.  With d_stash the probes take two passes (search, then ordered
// compaction) and their positions are parked in d_stash: m u32 inside the
// pairs buffer at or after u32 index 2 * (largest possible base) + m, so
// that pair o only overlaps stash entries j <= o.  Without it, one pass.
int launch_pairs(const gj_index* idx, const uint64_t* d_probes, uint64_t m, const uint32_t* d_rows,
                 uint32_t* d_pairs, const uint64_t* d_base, uint64_t* d_count, void* ws, size_t ws_bytes,
                 uint32_t* d_stash, cudaStream_t s);
// Pairs of a partitioned relation (keys grouped by key range, row ids
// attached): every tile of probes is sorted by key before it is searched.
// Pairs are appended at *d_base; the order inside a tile is not fixed.
// Workspace: pairs_workspace_bytes(m).
int launch_partitioned_pairs(const gj_index* idx, const uint64_t* d_keys, const uint32_t* d_rows, uint64_t m,
                             uint32_t* d_pairs, const uint64_t* d_base, uint64_t* d_count, void* ws, size_t ws_bytes,
                             cudaStream_t s);
size_t pairs_workspace_bytes(uint64_t m);
// launch_pairs for the test of the bounded waits: look-backs give up after
// spin_limit polls, and tile 0 is never claimed (so every wait runs out)
int launch_pairs_stalled(const gj_index* idx, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                         uint64_t* d_count, void* ws, size_t ws_bytes, uint32_t spin_limit, cudaStream_t s);
// launch_pairs in one pass with each tile's pairs placed by one atomicAdd
// (in the order tiles finish) instead of in probe order; the same set
int launch_pairs_unordered(const gj_index* idx, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                           uint64_t* d_count, void* ws, size_t ws_bytes, cudaStream_t s);
int pairs_error_flag(void* ws, size_t ws_bytes, uint64_t m, unsigned int* flag, cudaStream_t s);

// range partition of probe keys (gj_partition.cu): partition(k) =
// min((k - min_key) >> shift, 2^radix_bits - 1), keys <= min_key in 0;
// d_out_* in partition order, d_offsets (2^radix_bits + 1, optional) the
// partition starts; rows are row_base + input index
size_t partition_ws_bytes(uint64_t m, uint32_t radix_bits, int sm_count);
int range_partition_impl(const uint64_t* d_keys, uint64_t m, uint64_t min_key, uint32_t shift, uint32_t radix_bits,
                         uint64_t row_base, uint64_t* d_out_keys, uint32_t* d_out_rows, uint64_t* d_offsets, void* ws,
                         size_t ws_bytes, cudaStream_t s);
// fanout for an index of n keys (about 2^21 keys a partition, 2^5..2^12)
uint32_t default_radix_bits(uint64_t n);
// smallest shift that maps [min_key, max_key] onto 2^radix_bits partitions
uint32_t shift_for(uint64_t min_key, uint64_t max_key, uint32_t radix_bits);

// device-wide inclusive scans over uint64 (gj_gen.cu); workspace scan_workspace_bytes(n)
size_t scan_workspace_bytes(uint64_t n);
int inclusive_scan_sum(uint64_t* d_data, uint64_t n, void* ws, size_t ws_bytes, cudaStream_t s);
int inclusive_scan_max_signed(int64_t* d_data, uint64_t n, void* ws, size_t ws_bytes, cudaStream_t s);

// B+tree variants compiled: W in {4, 8, 16, 32, 64} separators per node and
// W = 7, 15 (compressed one-sector nodes); fn receives integral_constant<int, W>
template <class Fn>
int btree_dispatch(uint32_t w, Fn&& fn) {
    using std::integral_constant;
    switch (w) {
        case 4: return fn(integral_constant<int, 4>{});
        case 7: return fn(integral_constant<int, 7>{});
        case 8: return fn(integral_constant<int, 8>{});
        case 15: return fn(integral_constant<int, 15>{});
        case 16: return fn(integral_constant<int, 16>{});
        case 32: return fn(integral_constant<int, 32>{});
        case 64: return fn(integral_constant<int, 64>{});
        default:
            set_error("btree: unsupported node width %u", w);
            return GJ_ERR_UNSUPPORTED;
    }
}

// counter-based hashing shared by the generators and the learned trainer
__host__ __device__ inline uint64_t mix64(uint64_t x) {
    uint64_t z = x + 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
}  // namespace gj
