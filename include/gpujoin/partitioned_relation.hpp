// gpujoin/partitioned_relation.hpp -- C++ mirror of the reference's
// partitioned probe types and experiment configuration on top of
// libgpujoin.so:
//
//   partition_offsets, partitioned_relation<T>   src/partitioned_relation.hpp:12-50
//   experiment_config, parse_options,
//   get_experiment_config, radix_bits            src/index_lookup_config.hpp:18-72,
//                                                src/index_lookup_config.cpp:31-97
//   device_array_wrapper, create_device_array    src/device_array.hpp:132-236
//   inlj_pairs_by_approach                       src/index_lookup_new.cu:302-308
//
// Code written against the reference keeps its shape:
//
//   parse_options(argc, argv);
//   auto& config = get_experiment_config();
//   btree_index<uint64_t, uint64_t> index;  index.construct(h_view, d_keys);
//   partitioned_relation<Tuple<uint64_t, uint64_t>> rel(n, 1, radix_bits, alloc);
//   range_partition(index, d_probes, n, rel);           // the reference's run_on_stream
//   partitioned_lookup(index, rel, d_tids);             // partitioned_lookup_kernel
//
// Differences, each needed by the GB300 layout: the relation is SoA (keys and
// row ids in partition order, no 128-byte padding: padding_length() is 0)
// instead of an array of Tuple<key, value>; offsets holds fanout + 1 entries
// (partition starts and the total); the partition function is a range split
// of the index's key range (min((key - min) >> shift, fanout - 1)) instead of
// key bits.  Device memory of these types is allocated here, in the caller's
// code, with cudaMalloc (the reference's device_array_wrapper does the same);
// the library itself allocates nothing for them.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>

#include "../gpujoin.h"

// ---------------------------------------------------------------------------
// device_array_wrapper (src/device_array.hpp:132-236): an owning device array
// ---------------------------------------------------------------------------
template <class T>
struct device_array_wrapper {
    std::shared_ptr<T> ptr_;
    size_t size_ = 0;

    device_array_wrapper() = default;
    explicit device_array_wrapper(size_t n) : size_(n) {
        void* p = nullptr;
        if (n && cudaMalloc(&p, n * sizeof(T)) != cudaSuccess)
            throw std::runtime_error("device_array_wrapper: cudaMalloc failed");
        ptr_.reset(static_cast<T*>(p), [](T* q) {
            if (q) cudaFree(q);
        });
    }
    T* data() const { return ptr_.get(); }
    size_t size() const { return size_; }
};

template <class T>
device_array_wrapper<T> create_device_array(size_t n) {
    return device_array_wrapper<T>(n);
}

namespace gpu_prefix_sum {
// number of partitions for a radix width (the reference's gpu_prefix_sum::fanout)
inline uint32_t fanout(uint32_t radix_bits) { return 1u << radix_bits; }
}  // namespace gpu_prefix_sum

// ---------------------------------------------------------------------------
// partition_offsets / partitioned_relation<T> (src/partitioned_relation.hpp)
// ---------------------------------------------------------------------------
struct partition_offsets {
    device_array_wrapper<unsigned long long> offsets;        // fanout + 1: partition starts, then the total
    device_array_wrapper<unsigned long long> local_offsets;  // fanout * max_chunks (per-chunk starts)

    partition_offsets() = default;
    partition_offsets(uint32_t max_chunks, uint32_t radix_bits)
        : offsets(gpu_prefix_sum::fanout(radix_bits) + 1),
          local_offsets((size_t)gpu_prefix_sum::fanout(radix_bits) * (max_chunks ? max_chunks : 1)) {}
    template <class Allocator>
    partition_offsets(uint32_t max_chunks, uint32_t radix_bits, Allocator&)
        : partition_offsets(max_chunks, radix_bits) {}
};

template <class T>
struct partitioned_relation {
    device_array_wrapper<uint64_t> keys;     // key of each partitioned tuple (the reference's Tuple::key)
    device_array_wrapper<uint32_t> rows;     // its probe row (Tuple::value)
    device_array_wrapper<uint64_t> offsets;  // fanout + 1: partition p is [offsets[p], offsets[p + 1])
    size_t len = 0;
    uint32_t radix_bits = 0;

    partitioned_relation() = default;
    partitioned_relation(size_t n, uint32_t /*max_chunks*/, uint32_t bits)
        : keys(n ? n : 1), rows(n ? n : 1), offsets(gpu_prefix_sum::fanout(bits) + 1), len(n), radix_bits(bits) {}
    template <class Allocator>
    partitioned_relation(size_t n, uint32_t max_chunks, uint32_t bits, Allocator&)
        : partitioned_relation(n, max_chunks, bits) {}

    unsigned padding_length() const { return 0; }
    uint32_t fanout() const { return gpu_prefix_sum::fanout(radix_bits); }
};

namespace gj {
namespace detail {
inline void check_rc(int rc) {
    if (rc != GJ_OK) throw std::runtime_error(gj_last_error_string());
}
}  // namespace detail
}  // namespace gj

// Partition m probe keys on the index's key range into rel (the reference's
// run_on_stream: prefix sum + radix partition, src/index_lookup_partitioning.cu:
// 300-359).  rel must hold at least m tuples.  Asynchronous on stream; the
// workspace is allocated and freed here (device_array_wrapper).
template <class Index, class T>
void range_partition(const Index& index, const uint64_t* d_keys, size_t m, partitioned_relation<T>& rel,
                     cudaStream_t stream = nullptr) {
    if (m > rel.len) throw std::runtime_error("range_partition: relation smaller than the input");
    uint64_t min_key = 0, max_key = 0;
    uint32_t shift = 0;
    gj::detail::check_rc(gj_index_key_range(index.handle.get(), &min_key, &max_key));
    gj::detail::check_rc(gj_partition_shift(min_key, max_key, rel.radix_bits, &shift));
    size_t need = 0;
    gj::detail::check_rc(gj_partition_workspace_size(m, rel.radix_bits, &need));
    device_array_wrapper<unsigned char> ws(need);
    gj::detail::check_rc(gj_range_partition(d_keys, m, min_key, shift, rel.radix_bits, rel.keys.data(),
                                            rel.rows.data(), rel.offsets.data(), ws.data(), need, stream));
    if (cudaStreamSynchronize(stream) != cudaSuccess) throw std::runtime_error("range_partition: stream failed");
}

// partitioned_lookup_kernel (src/index_lookup_partitioning.cu:218-248):
// tids[row] = the index's result for every tuple of rel.
template <class Index, class T>
void partitioned_lookup(const Index& index, const partitioned_relation<T>& rel, uint32_t* d_tids,
                        cudaStream_t stream = nullptr) {
    gj::detail::check_rc(gj_partitioned_lookup(index.handle.get(), rel.keys.data(), rel.rows.data(), rel.len, d_tids,
                                               stream));
}

// ---------------------------------------------------------------------------
// experiment configuration (src/index_lookup_config.hpp:18-72)
// ---------------------------------------------------------------------------
enum class dataset_type : unsigned { dense, sparse };
enum class lookup_pattern_type : unsigned { uniform, uniform_unique, zipf };

struct experiment_config {
    std::string approach = "plain";
    std::string index_type = "btree";
    std::string scenario = "single";
    std::string output_file = "";
    uint64_t num_lookups = 100000000ull;
    uint64_t num_elements = 1000000ull;
    unsigned max_bits = 0;
    double zipf_factor = 1.25;
    int block_size = 128;
    dataset_type dataset = dataset_type::sparse;
    lookup_pattern_type lookup_pattern = lookup_pattern_type::uniform;
    bool sorted_lookups = false;
    unsigned partitioning_approach_ignore_bits = 4;
    bool partitioning_approach_dynamic_bit_range = true;
    uint64_t partitioning_approach_window_size = 10000;
};

// the reference's fixed fanout (src/index_lookup_config.hpp:37)
static const uint32_t radix_bits = 11;

inline experiment_config& get_experiment_config() {
    static experiment_config config;
    return config;
}

// The reference's command line (src/index_lookup_config.cpp:35-97): -a/--approach,
// -i/--index, -e/--elements, -l/--lookups, -b/--blocksize, -m/--maxbits,
// -z/--zipf, -d/--dataset, -p/--lookup_pattern, -s/--sorted_lookups,
// -o/--output, -w/--window, -h/--help ("--name=value" or "--name value").
// Unknown options, missing values and unknown dataset / pattern names throw
// std::invalid_argument (the reference's cxxopts throws, or asserts, on them).
// -h returns true (the reference prints its usage and exits; the caller
// decides here).
inline bool parse_options(int argc, char** argv) {
    experiment_config& c = get_experiment_config();
    auto want = [](const std::string& opt, const char* v) -> std::string {
        if (!v) throw std::invalid_argument("option " + opt + " needs a value");
        return std::string(v);
    };
    auto to_u64 = [](const std::string& opt, const std::string& v) -> uint64_t {
        char* end = nullptr;
        const double d = std::strtod(v.c_str(), &end);  // accepts 1e8 as the reference's defaults are written
        if (v.empty() || *end != '\0' || d < 0) throw std::invalid_argument("option " + opt + ": bad number " + v);
        return static_cast<uint64_t>(d);
    };
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i], name, value;
        bool has_value = false;
        if (a.rfind("--", 0) == 0) {
            const size_t eq = a.find('=');
            name = a.substr(2, eq == std::string::npos ? std::string::npos : eq - 2);
            if (eq != std::string::npos) {
                value = a.substr(eq + 1);
                has_value = true;
            }
        } else if (a.size() == 2 && a[0] == '-') {
            static const char* longs[][2] = {{"a", "approach"}, {"i", "index"},   {"e", "elements"},
                                             {"l", "lookups"},  {"b", "blocksize"}, {"m", "maxbits"},
                                             {"z", "zipf"},     {"d", "dataset"}, {"p", "lookup_pattern"},
                                             {"s", "sorted_lookups"}, {"o", "output"}, {"w", "window"},
                                             {"h", "help"}};
            for (auto& l : longs)
                if (a.substr(1) == l[0]) name = l[1];
            if (name.empty()) throw std::invalid_argument("unknown option " + a);
        } else {
            throw std::invalid_argument("unexpected argument " + a);
        }
        if (name == "help") return true;
        if (name == "sorted_lookups") {
            c.sorted_lookups = has_value ? (value == "true" || value == "1") : true;
            continue;
        }
        if (!has_value) value = want(a, i + 1 < argc ? argv[++i] : nullptr);
        if (name == "approach") c.approach = value;
        else if (name == "index") c.index_type = value;
        else if (name == "elements") c.num_elements = to_u64(a, value);
        else if (name == "lookups") c.num_lookups = to_u64(a, value);
        else if (name == "blocksize") c.block_size = (int)to_u64(a, value);
        else if (name == "maxbits") c.max_bits = (unsigned)to_u64(a, value);
        else if (name == "zipf") c.zipf_factor = std::strtod(value.c_str(), nullptr);
        else if (name == "output") c.output_file = value;
        else if (name == "window") c.partitioning_approach_window_size = to_u64(a, value);
        else if (name == "dataset") {
            if (value == "sparse") c.dataset = dataset_type::sparse;
            else if (value == "dense") c.dataset = dataset_type::dense;
            else throw std::invalid_argument("unknown dataset type " + value);
        } else if (name == "lookup_pattern") {
            if (value == "uniform") c.lookup_pattern = lookup_pattern_type::uniform;
            else if (value == "uniform_unique") c.lookup_pattern = lookup_pattern_type::uniform_unique;
            else if (value == "zipf") c.lookup_pattern = lookup_pattern_type::zipf;
            else throw std::invalid_argument("unknown lookup pattern " + value);
        } else {
            throw std::invalid_argument("unknown option " + a);
        }
    }
    return false;
}

// ---------------------------------------------------------------------------
// approaches (the reference's approach map, src/index_lookup_new.cu:302-308)
// ---------------------------------------------------------------------------
// The join pairs of m probes against index by config.approach:
//   "plain"         gj_inlj_pairs (plain_approach): pairs in probe order
//   "bws"           gj_inlj_pairs_sorted (blockwise_sorting_approach): tile by
//                   tile in probe order, key order inside a tile
//   "partitioning"  gj_partitioned_inlj (partitioning_approach): windows of
//                   config.partitioning_approach_window_size probes (0: all),
//                   the library's default fanout; pairs grouped by partition
//                   tile
//   "auto"          whichever of the three gj_autotune_ordering times fastest
//                   on these probes
// Every approach gives the same set of pairs.  The reference's "hj" (its hash
// join) is an index kind here (GJ_INDEX_HASH), joined by any of them.
// d_pairs (2m u32: probe row, build position) and d_count (one u64) are device
// memory.  Unknown approach names throw std::invalid_argument, library errors
// std::runtime_error.  Workspaces are allocated and freed here, so the call
// synchronises the stream.
static const uint32_t approach_auto = 0xFFFFFFFFu;

// the GJ_ORDER_* of an approach name, approach_auto for "auto"
inline uint32_t approach_order(const std::string& a) {
    if (a == "plain") return GJ_ORDER_PROBE;
    if (a == "bws") return GJ_ORDER_SORTED_TILES;
    if (a == "partitioning") return GJ_ORDER_PARTITIONED;
    if (a == "auto") return approach_auto;
    throw std::invalid_argument("unknown approach " + a);
}

template <class Index>
void inlj_pairs_by_approach(const Index& index, const uint64_t* d_probes, size_t m, uint32_t* d_pairs,
                            uint64_t* d_count, const experiment_config& config = get_experiment_config(),
                            cudaStream_t stream = nullptr) {
    const gj_index* ix = index.handle.get();
    uint32_t order = approach_order(config.approach);
    if (order == approach_auto) {
        order = GJ_ORDER_PROBE;
        if (m > 0) gj::detail::check_rc(gj_autotune_ordering(ix, d_probes, m, stream, &order, nullptr));
    }
    if (order == GJ_ORDER_PARTITIONED) {
        const uint64_t w = config.partitioning_approach_window_size ? config.partitioning_approach_window_size
                                                                    : (m ? m : 1);
        size_t need = 0;
        gj::detail::check_rc(gj_partitioned_inlj_workspace_size(ix, w, 0, &need));
        device_array_wrapper<unsigned char> ws(need);
        gj::detail::check_rc(
            gj_partitioned_inlj(ix, d_probes, m, w, 0, nullptr, d_pairs, d_count, ws.data(), need, stream));
    } else {
        size_t need = 0;
        gj::detail::check_rc(gj_inlj_pairs_workspace_size(m, &need));
        device_array_wrapper<unsigned char> ws(need);
        gj::detail::check_rc(order == GJ_ORDER_SORTED_TILES
                                 ? gj_inlj_pairs_sorted(ix, d_probes, m, d_pairs, d_count, ws.data(), need, stream)
                                 : gj_inlj_pairs(ix, d_probes, m, d_pairs, d_count, ws.data(), need, stream));
    }
    if (cudaStreamSynchronize(stream) != cudaSuccess)
        throw std::runtime_error("inlj_pairs_by_approach: stream failed");
}
