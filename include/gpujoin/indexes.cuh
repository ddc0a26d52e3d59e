// gpujoin/indexes.cuh -- C++ mirror of the reference's index API
// (src/indexes.cuh, src/indexes.hpp) on top of libgpujoin.so.
//
// Code written against the reference keeps its shape:
//
//   btree_index<uint64_t, uint64_t> index;            // same template shape
//   index.construct(make_vector_view(h_keys), d_keys);
//   my_kernel<<<g, b>>>(index.device_index, ...);     // by-value device view
//   ... index_structure.cooperative_lookup(active, key) in device code
//
// cooperative_lookup(active, key) keeps the reference's per-index result
// semantics (lower bound for binary_search / radix_spline / learned, equal
// key for btree / harmonia, invalid for no_op) and returns
// numeric_limits<Value>::max() where the reference returns invalid_tid.  It
// does not need the whole warp: lanes may call it independently.
// binary_search_index and harmonia_index also offer
// warp_cooperative_lookup<Degree>(active, key), the reference's
// warp-collective protocol (groups of 2^Degree lanes per query, the whole
// warp calling), with the same results.
//
// Keys must be uint64 (the reference's index_key_t, src/index_lookup_config.hpp:45).
// The allocator template parameters are accepted for source compatibility;
// device memory is owned by the library.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../gpujoin.h"
#include "device.cuh"

// ---------------------------------------------------------------------------
// vector_view (src/vector_view.hpp): a non-owning view of a host column
// ---------------------------------------------------------------------------
template <class T>
struct vector_view {
    using value_type = T;
    T* ptr_ = nullptr;
    size_t size_ = 0;
    vector_view() = default;
    vector_view(T* p, size_t n) : ptr_(p), size_(n) {}
    T* data() const { return ptr_; }
    size_t size() const { return size_; }
    T* begin() const { return ptr_; }
    T* end() const { return ptr_ + size_; }
    T& operator[](size_t i) const { return ptr_[i]; }
};

template <class Vector>
vector_view<typename Vector::value_type> make_vector_view(Vector& v) {
    return vector_view<typename Vector::value_type>(v.data(), v.size());
}

// ---------------------------------------------------------------------------
// index_type_enum / parse_index_type (src/indexes.hpp:5-7, src/indexes.cpp:5-19)
// ---------------------------------------------------------------------------
enum class index_type_enum : unsigned { btree, harmonia, binary_search, radix_spline, no_op, learned };

inline index_type_enum parse_index_type(const std::string& index_name) {
    int t = 0;
    if (gj_parse_index_type(index_name.c_str(), &t) != GJ_OK) throw std::runtime_error("unknown index type");
    return static_cast<index_type_enum>(t);
}

template <class T>
struct type_name;

// ---------------------------------------------------------------------------
// abstract_index (src/indexes.cuh:30-39)
// ---------------------------------------------------------------------------
template <class Key>
struct abstract_index {
    using key_t = Key;
    virtual ~abstract_index() = default;
    virtual void construct(const vector_view<key_t>& h_column, const key_t* d_column) = 0;
    virtual size_t memory_consumption() const = 0;
};

namespace gj {
namespace detail {

inline void check(int rc) {
    if (rc != GJ_OK) throw std::runtime_error(gj_last_error_string());
}

// B+tree lookup over the node widths the library builds
GJ_DEVICE_INLINE uint32_t btree_lookup_any(const btree_view& v, uint64_t key) {
    switch (v.node_keys) {
        case 4: return btree_lookup<4>(v, nullptr, key);
        case 7: return btree_lookup<7>(v, nullptr, key);
        case 8: return btree_lookup<8>(v, nullptr, key);
        case 15: return btree_lookup<15>(v, nullptr, key);
        case 16: return btree_lookup<16>(v, nullptr, key);
        case 32: return btree_lookup<32>(v, nullptr, key);
        default: return btree_lookup<64>(v, nullptr, key);
    }
}

// common host part: owns the library index and fetches its device view
template <int Type, class View, class Key>
struct index_base : public abstract_index<Key> {
    static_assert(std::is_same<Key, uint64_t>::value, "gpujoin indexes take uint64 keys");
    gj_index_params params;
    std::shared_ptr<gj_index> handle;

    index_base() { gj_index_params_default(&params); }

    void build(const vector_view<Key>& h_column, const Key* d_column, View* view) {
        gj_index* ix = nullptr;
        check(gj_index_build(Type, d_column, h_column.data(), h_column.size(), &params, nullptr, &ix));
        handle.reset(ix, [](gj_index* p) { gj_index_free(p); });
        if (view) check(gj_index_device_view(ix, view, sizeof(View)));
    }

    size_t memory_consumption() const override {
        return handle ? static_cast<size_t>(gj_index_memory_consumption(handle.get())) : 0;
    }
};

template <class Value>
GJ_DEVICE_INLINE Value to_tid(uint32_t r) {
    return r == GJ_INVALID_POS ? static_cast<Value>(~static_cast<Value>(0)) : static_cast<Value>(r);
}

}  // namespace detail
}  // namespace gj

// ---------------------------------------------------------------------------
// the index types (src/indexes.cuh:93-147, 176-248, 257-307, 336-375, 384-406)
// ---------------------------------------------------------------------------
template <class Key, class Value, template <class T> class DeviceAllocator = std::allocator,
          template <class T> class HostAllocator = std::allocator, class IndexConfiguration = void>
struct btree_index : public gj::detail::index_base<GJ_INDEX_BTREE, gj::btree_view, Key> {
    using key_t = Key;
    using value_t = Value;
    static constexpr value_t invalid_tid = std::numeric_limits<value_t>::max();

    struct device_index_t {
        gj::btree_view v;
        __device__ __forceinline__ value_t cooperative_lookup(const bool active, const key_t key) const {
            return active ? gj::detail::to_tid<value_t>(gj::detail::btree_lookup_any(v, key)) : invalid_tid;
        }
    } device_index;

    void construct(const vector_view<key_t>& h_column, const key_t* d_column) override {
        this->build(h_column, d_column, &device_index.v);
    }
};

template <class Key, class Value, template <class T> class DeviceAllocator = std::allocator,
          template <class T> class HostAllocator = std::allocator>
struct harmonia_index : public gj::detail::index_base<GJ_INDEX_HARMONIA, gj::harmonia_view, Key> {
    using key_t = Key;
    using value_t = Value;
    static constexpr value_t invalid_tid = std::numeric_limits<value_t>::max();

    struct device_index_t {
        gj::harmonia_view v;
        __device__ __forceinline__ value_t cooperative_lookup(const bool active, const key_t key) const {
            return active ? gj::detail::to_tid<value_t>(gj::harmonia_lookup(v, nullptr, key)) : invalid_tid;
        }
        // harmonia_tree::lookup<Degree> (src/harmonia.cuh:740-786): groups of
        // 2^Degree lanes per node; the whole warp calls it, converged
        template <unsigned Degree = 4>
        __device__ __forceinline__ value_t warp_cooperative_lookup(const bool active, const key_t key) const {
            const uint32_t r = gj::harmonia_lookup_cooperative<Degree>(active, v, key);
            return active ? gj::detail::to_tid<value_t>(r) : invalid_tid;
        }
    } device_index;

    void construct(const vector_view<key_t>& h_column, const key_t* d_column) override {
        this->build(h_column, d_column, &device_index.v);
    }
};

template <class Key, class Value, template <class T> class DeviceAllocator = std::allocator,
          template <class T> class HostAllocator = std::allocator, class IndexConfiguration = void>
struct binary_search_index : public gj::detail::index_base<GJ_INDEX_BINARY_SEARCH, gj::bs_view, Key> {
    using key_t = Key;
    using value_t = Value;
    static constexpr value_t invalid_tid = std::numeric_limits<value_t>::max();

    struct device_index_t {
        gj::bs_view v;
        __device__ __forceinline__ value_t cooperative_lookup(const bool active, const key_t key) const {
            return active ? gj::detail::to_tid<value_t>(gj::bs_lookup(v, v.fence, key)) : invalid_tid;
        }
        // cooperative_binary_search (src/search.cuh:355-386): groups of
        // 2^Degree lanes per query; the whole warp calls it, converged
        template <unsigned Degree = 4>
        __device__ __forceinline__ value_t warp_cooperative_lookup(const bool active, const key_t key) const {
            const uint64_t r = gj::cooperative_lower_bound<Degree>(active, key, v.col, v.n);
            return active && r < v.n ? static_cast<value_t>(r) : invalid_tid;
        }
    } device_index;

    void construct(const vector_view<key_t>& h_column, const key_t* d_column) override {
        this->build(h_column, d_column, &device_index.v);
    }
};

template <class Key, class Value, template <class T> class DeviceAllocator = std::allocator,
          template <class T> class HostAllocator = std::allocator, class IndexConfiguration = void>
struct radix_spline_index : public gj::detail::index_base<GJ_INDEX_RADIX_SPLINE, gj::rs_view, Key> {
    using key_t = Key;
    using value_t = Value;
    static constexpr value_t invalid_tid = std::numeric_limits<value_t>::max();

    struct device_index_t {
        gj::rs_view v;
        __device__ __forceinline__ value_t cooperative_lookup(const bool active, const key_t key) const {
            return active ? gj::detail::to_tid<value_t>(gj::rs_lookup(v, key)) : invalid_tid;
        }
    } device_index;

    void construct(const vector_view<key_t>& h_column, const key_t* d_column) override {
        this->build(h_column, d_column, &device_index.v);
    }
};

template <class Key, class Value, template <class T> class DeviceAllocator = std::allocator,
          template <class T> class HostAllocator = std::allocator>
struct learned_index : public gj::detail::index_base<GJ_INDEX_LEARNED, gj::learned_view, Key> {
    using key_t = Key;
    using value_t = Value;
    static constexpr value_t invalid_tid = std::numeric_limits<value_t>::max();

    struct device_index_t {
        gj::learned_view v;
        __device__ __forceinline__ value_t cooperative_lookup(const bool active, const key_t key) const {
            return active ? gj::detail::to_tid<value_t>(gj::learned_lookup(v, v.root, key)) : invalid_tid;
        }
    } device_index;

    void construct(const vector_view<key_t>& h_column, const key_t* d_column) override {
        this->build(h_column, d_column, &device_index.v);
    }
};

// the reference's hash-join table (src/linear_probing_hashtable.cuh) with the
// index interface: position of the equal key, else invalid_tid
template <class Key, class Value, template <class T> class DeviceAllocator = std::allocator,
          template <class T> class HostAllocator = std::allocator>
struct hash_index : public gj::detail::index_base<GJ_INDEX_HASH, gj::hash_view, Key> {
    using key_t = Key;
    using value_t = Value;
    static constexpr value_t invalid_tid = std::numeric_limits<value_t>::max();

    struct device_index_t {
        gj::hash_view v;
        __device__ __forceinline__ value_t cooperative_lookup(const bool active, const key_t key) const {
            return active ? gj::detail::to_tid<value_t>(gj::hash_lookup(v, key)) : invalid_tid;
        }
    } device_index;

    void construct(const vector_view<key_t>& h_column, const key_t* d_column) override {
        this->build(h_column, d_column, &device_index.v);
    }
};

template <class Key, class Value, template <class T> class DeviceAllocator = std::allocator,
          template <class T> class HostAllocator = std::allocator>
struct no_op_index : public abstract_index<Key> {
    using key_t = Key;
    using value_t = Value;
    static constexpr value_t invalid_tid = std::numeric_limits<value_t>::max();

    struct device_index_t {
        __device__ __forceinline__ value_t cooperative_lookup(const bool, const key_t) const { return invalid_tid; }
    } device_index;

    void construct(const vector_view<key_t>&, const key_t*) override {}
    size_t memory_consumption() const override { return 0; }
};

template <class K, class V, template <class T> class D, template <class T> class H, class C>
struct type_name<btree_index<K, V, D, H, C>> {
    static const char* value() { return "btree"; }
};
template <class K, class V, template <class T> class D, template <class T> class H>
struct type_name<harmonia_index<K, V, D, H>> {
    static const char* value() { return "harmonia"; }
};
template <class K, class V, template <class T> class D, template <class T> class H, class C>
struct type_name<binary_search_index<K, V, D, H, C>> {
    static const char* value() { return "binary_search"; }
};
template <class K, class V, template <class T> class D, template <class T> class H, class C>
struct type_name<radix_spline_index<K, V, D, H, C>> {
    static const char* value() { return "radix_spline"; }
};
template <class K, class V, template <class T> class D, template <class T> class H>
struct type_name<learned_index<K, V, D, H>> {
    static const char* value() { return "learned"; }
};
template <class K, class V, template <class T> class D, template <class T> class H>
struct type_name<no_op_index<K, V, D, H>> {
    static const char* value() { return "no_op"; }
};
