// A probe written the way the reference's code is written -- index class
// templates, construct(h_column, d_column), a kernel taking the index's
// device_index by value and calling cooperative_lookup(active, key), the
// partitioned path through partitioned_relation<T> and partitioned_lookup,
// and the experiment_config / parse_options command line -- built against
// include/gpujoin/indexes.cuh, include/gpujoin/partitioned_relation.hpp and
// libgpujoin.so.  Used by tests/test_drop_in.py to show that such code
// compiles and probes correctly without changes to its structure.
#include <cstdint>
#include <exception>
#include <vector>

#include "gpujoin/indexes.cuh"
#include "gpujoin/partitioned_relation.hpp"

using index_key_t = uint64_t;
using value_t = uint64_t;

template <class IndexStructureType>
__global__ void probe_all(const IndexStructureType index_structure, uint64_t n, const index_key_t* __restrict__ keys,
                          value_t* __restrict__ tids) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // the loop bound is rounded up to whole warps so every lane reaches the lookup
    const uint64_t limit = (n + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < limit; i += stride) {
        const bool active = i < n;
        const index_key_t key = active ? keys[i] : 0;
        const value_t tid = index_structure.cooperative_lookup(active, key);
        if (active) tids[i] = tid;
    }
}

// the reference's lookup_kernel with a warp-collective lookup: every lane
// of a warp reaches the call, inactive ones with active = false
template <class IndexStructureType, unsigned Degree>
__global__ void probe_all_warp(const IndexStructureType index_structure, uint64_t n,
                               const index_key_t* __restrict__ keys, value_t* __restrict__ tids) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t limit = (n + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < limit; i += stride) {
        const bool active = i < n;
        const index_key_t key = active ? keys[i] : 0;
        const value_t tid = index_structure.template warp_cooperative_lookup<Degree>(active, key);
        if (active) tids[i] = tid;
    }
}

template <class IndexType, unsigned Degree>
static int run_warp(const index_key_t* d_col, const index_key_t* h_col, uint64_t n, const index_key_t* d_keys,
                    uint64_t m, value_t* d_tids) {
    IndexType index;
    index.construct(vector_view<index_key_t>(const_cast<index_key_t*>(h_col), n), d_col);
    const int block = 128;
    const uint64_t blocks = (m + block - 1) / block;
    probe_all_warp<typename IndexType::device_index_t, Degree>
        <<<(unsigned)(blocks ? (blocks < 65535 ? blocks : 65535) : 1), block>>>(index.device_index, m, d_keys, d_tids);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
}

// warp-collective lookups: kind 1 = harmonia, 2 = binary_search; degree 1..5
extern "C" int drop_in_probe_warp(int kind, int degree, const index_key_t* d_col, const index_key_t* h_col,
                                  uint64_t n, const index_key_t* d_keys, uint64_t m, value_t* d_tids) {
    try {
        using H = harmonia_index<index_key_t, value_t>;
        using B = binary_search_index<index_key_t, value_t>;
        switch (kind * 10 + degree) {
            case 11: return run_warp<H, 1>(d_col, h_col, n, d_keys, m, d_tids);
            case 12: return run_warp<H, 2>(d_col, h_col, n, d_keys, m, d_tids);
            case 14: return run_warp<H, 4>(d_col, h_col, n, d_keys, m, d_tids);
            case 15: return run_warp<H, 5>(d_col, h_col, n, d_keys, m, d_tids);
            case 21: return run_warp<B, 1>(d_col, h_col, n, d_keys, m, d_tids);
            case 22: return run_warp<B, 2>(d_col, h_col, n, d_keys, m, d_tids);
            case 24: return run_warp<B, 4>(d_col, h_col, n, d_keys, m, d_tids);
            case 25: return run_warp<B, 5>(d_col, h_col, n, d_keys, m, d_tids);
            default: return 3;
        }
    } catch (const std::exception&) {
        return 1;
    }
}

template <class IndexType>
static int run(const index_key_t* d_col, const index_key_t* h_col, uint64_t n, const index_key_t* d_keys,
               uint64_t m, value_t* d_tids) {
    IndexType index;
    index.construct(vector_view<index_key_t>(const_cast<index_key_t*>(h_col), n), d_col);
    const int block = 128;
    const uint64_t blocks = (m + block - 1) / block;
    probe_all<<<(unsigned)(blocks ? (blocks < 65535 ? blocks : 65535) : 1), block>>>(index.device_index, m, d_keys,
                                                                                     d_tids);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 2;
}

extern "C" int drop_in_probe(int kind, const index_key_t* d_col, const index_key_t* h_col, uint64_t n,
                             const index_key_t* d_keys, uint64_t m, value_t* d_tids) {
    try {
        switch (parse_index_type(kind == 0 ? "btree" : kind == 1 ? "harmonia" : kind == 2 ? "binary_search"
                                 : kind == 3 ? "radix_spline" : kind == 4 ? "no_op" : "learned")) {
            case index_type_enum::btree: return run<btree_index<index_key_t, value_t>>(d_col, h_col, n, d_keys, m, d_tids);
            case index_type_enum::harmonia:
                return run<harmonia_index<index_key_t, value_t>>(d_col, h_col, n, d_keys, m, d_tids);
            case index_type_enum::binary_search:
                return run<binary_search_index<index_key_t, value_t>>(d_col, h_col, n, d_keys, m, d_tids);
            case index_type_enum::radix_spline:
                return run<radix_spline_index<index_key_t, value_t>>(d_col, h_col, n, d_keys, m, d_tids);
            case index_type_enum::no_op: return run<no_op_index<index_key_t, value_t>>(d_col, h_col, n, d_keys, m, d_tids);
            case index_type_enum::learned:
                return run<learned_index<index_key_t, value_t>>(d_col, h_col, n, d_keys, m, d_tids);
        }
    } catch (const std::exception&) {
        return 1;
    }
    return 3;
}

extern "C" const char* drop_in_type_name() { return type_name<btree_index<index_key_t, value_t>>::value(); }

// the tuple type of the reference's partitioned relation (fast-interconnects'
// Tuple<key, value>); the SoA relation here only takes it as a tag
template <class K, class V>
struct Tuple {
    K key;
    V value;
};

struct device_allocator_tag {};

template <class IndexType>
static int run_partitioned(const index_key_t* d_col, const index_key_t* h_col, uint64_t n, const index_key_t* d_keys,
                           uint64_t m, uint32_t bits, uint32_t* d_tids) {
    IndexType index;
    index.construct(vector_view<index_key_t>(const_cast<index_key_t*>(h_col), n), d_col);
    device_allocator_tag alloc;
    partitioned_relation<Tuple<index_key_t, value_t>> rel(m, 1, bits, alloc);
    partition_offsets offs(1, bits, alloc);
    range_partition(index, d_keys, m, rel);
    partitioned_lookup(index, rel, d_tids);
    return cudaDeviceSynchronize() == cudaSuccess && rel.padding_length() == 0 &&
                   offs.offsets.size() == gpu_prefix_sum::fanout(bits) + 1
               ? 0
               : 2;
}

extern "C" int drop_in_partitioned_probe(int kind, const index_key_t* d_col, const index_key_t* h_col, uint64_t n,
                                         const index_key_t* d_keys, uint64_t m, uint32_t bits, uint32_t* d_tids) {
    try {
        if (kind == 0) return run_partitioned<btree_index<index_key_t, value_t>>(d_col, h_col, n, d_keys, m, bits, d_tids);
        if (kind == 2)
            return run_partitioned<binary_search_index<index_key_t, value_t>>(d_col, h_col, n, d_keys, m, bits, d_tids);
        return 3;
    } catch (const std::exception&) {
        return 1;
    }
}

// the join pairs by the reference's approach names (inlj_pairs_by_approach
// with experiment_config::approach set from the command line's -a); 0, or 4
// for an unknown approach, 1 for a library error
template <class IndexType>
static int run_approach(const char* approach, uint64_t window, const index_key_t* d_col, const index_key_t* h_col,
                        uint64_t n, const index_key_t* d_keys, uint64_t m, uint32_t* d_pairs, uint64_t* d_count) {
    IndexType index;
    index.construct(vector_view<index_key_t>(const_cast<index_key_t*>(h_col), n), d_col);
    experiment_config config;
    config.approach = approach;
    config.partitioning_approach_window_size = window;
    try {
        inlj_pairs_by_approach(index, d_keys, m, d_pairs, d_count, config);
    } catch (const std::invalid_argument&) {
        return 4;
    }
    return 0;
}

// 1 when approach_order knows the name, 0 when it throws
extern "C" int drop_in_approach_name_known(const char* approach) {
    try {
        approach_order(approach);
        return 1;
    } catch (const std::invalid_argument&) {
        return 0;
    }
}

extern "C" int drop_in_approach_pairs(int kind, const char* approach, uint64_t window, const index_key_t* d_col,
                                      const index_key_t* h_col, uint64_t n, const index_key_t* d_keys, uint64_t m,
                                      uint32_t* d_pairs, uint64_t* d_count) {
    try {
        if (kind == 0)
            return run_approach<btree_index<index_key_t, value_t>>(approach, window, d_col, h_col, n, d_keys, m,
                                                                   d_pairs, d_count);
        if (kind == 2)
            return run_approach<binary_search_index<index_key_t, value_t>>(approach, window, d_col, h_col, n, d_keys,
                                                                           m, d_pairs, d_count);
        return 3;
    } catch (const std::exception&) {
        return 1;
    }
}

// parse_options on a reference-style command line; out[] = the parsed
// fields, return 0, 1 when -h was given, -1 when parsing threw
extern "C" int drop_in_parse_options(int argc, char** argv, uint64_t* out, char* approach, char* index) {
    get_experiment_config() = experiment_config();
    try {
        const bool help = parse_options(argc, argv);
        const experiment_config& c = get_experiment_config();
        out[0] = c.num_elements;
        out[1] = c.num_lookups;
        out[2] = c.max_bits;
        out[3] = c.partitioning_approach_window_size;
        out[4] = (uint64_t)c.dataset;
        out[5] = (uint64_t)c.lookup_pattern;
        out[6] = c.sorted_lookups ? 1 : 0;
        out[7] = (uint64_t)c.block_size;
        out[8] = (uint64_t)(c.zipf_factor * 1000.0 + 0.5);
        out[9] = radix_bits;
        std::strncpy(approach, c.approach.c_str(), 31);
        std::strncpy(index, c.index_type.c_str(), 31);
        return help ? 1 : 0;
    } catch (const std::exception&) {
        return -1;
    }
}
