// gj_lookup.cu -- the library's entry to the probe kernels: dispatch over
// the index kind to the unit that compiles its kernels, and the kinds
// compiled here (binary search, hash table, no-op).  Kernels: gj_lookup_kernels.cuh.
#include "gj_lookup_kernels.cuh"

namespace gj {

int lookup_call_bs(const gj_index* idx, const lookup_call& c) { return run_call(op_bs{idx->bs}, idx, c); }
int lookup_call_noop(const gj_index* idx, const lookup_call& c) { return run_call(op_noop{}, idx, c); }
int lookup_call_hash(const gj_index* idx, const lookup_call& c) { return run_call(op_hash{idx->hs}, idx, c); }

namespace {

int dispatch(const gj_index* idx, const lookup_call& c) {
    switch (idx->type) {
        case GJ_INDEX_BINARY_SEARCH: return lookup_call_bs(idx, c);
        case GJ_INDEX_BTREE:
            return btree_dispatch(idx->bt.node_keys,
                                  [&](auto w) { return lookup_call_btree<decltype(w)::value>(idx, c); });
        case GJ_INDEX_HARMONIA: return lookup_call_harmonia(idx, c);
        case GJ_INDEX_RADIX_SPLINE: return lookup_call_rs(idx, c);
        case GJ_INDEX_LEARNED: return lookup_call_learned(idx, c);
        case GJ_INDEX_NO_OP: return lookup_call_noop(idx, c);
        case GJ_INDEX_HASH: return lookup_call_hash(idx, c);
        default: set_error("unknown index type %d", idx->type); return GJ_ERR_INVALID_ARGUMENT;
    }
}

}  // namespace

size_t pairs_workspace_bytes(uint64_t m) {
    const uint64_t states = (m + kStateTile - 1) / kStateTile;
    return workspace_carver::need({(size_t)(states ? states : 1) * 8, 8, 16});
}

int launch_lookup(const gj_index* idx, const uint64_t* d_probes, uint64_t m, uint32_t* d_out, cudaStream_t s) {
    if (m == 0) return GJ_OK;
    return dispatch(idx, {lookup_action::positions, d_probes, nullptr, m, d_out, nullptr, nullptr, nullptr, 0,
                          nullptr, s});
}

int launch_sorted_lookup(const gj_index* idx, const uint64_t* d_probes, uint64_t m, uint32_t* d_out, cudaStream_t s) {
    if (m == 0) return GJ_OK;
    return dispatch(idx, {lookup_action::sorted_positions, d_probes, nullptr, m, d_out, nullptr, nullptr, nullptr, 0,
                          nullptr, s});
}

int launch_scatter_lookup(const gj_index* idx, const uint64_t* d_keys, const uint32_t* d_rows, uint64_t m,
                          uint32_t* d_out, cudaStream_t s) {
    if (m == 0) return GJ_OK;
    return dispatch(idx, {lookup_action::scatter, d_keys, d_rows, m, d_out, nullptr, nullptr, nullptr, 0, nullptr, s});
}

int launch_pairs(const gj_index* idx, const uint64_t* d_probes, uint64_t m, const uint32_t* d_rows, uint32_t* d_pairs,
                 const uint64_t* d_base, uint64_t* d_count, void* ws, size_t ws_bytes, uint32_t* d_stash,
                 cudaStream_t s) {
    return dispatch(idx, {lookup_action::pairs, d_probes, d_rows, m, d_pairs, d_base, d_count, ws, ws_bytes, d_stash,
                          s});
}

int launch_partitioned_pairs(const gj_index* idx, const uint64_t* d_keys, const uint32_t* d_rows, uint64_t m,
                             uint32_t* d_pairs, const uint64_t* d_base, uint64_t* d_count, void* ws, size_t ws_bytes,
                             cudaStream_t s) {
    return dispatch(idx, {lookup_action::sorted_pairs, d_keys, d_rows, m, d_pairs, d_base, d_count, ws, ws_bytes,
                          nullptr, s});
}

int launch_pairs_stalled(const gj_index* idx, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                         uint64_t* d_count, void* ws, size_t ws_bytes, uint32_t spin_limit, cudaStream_t s) {
    lookup_call c{lookup_action::pairs, d_probes, nullptr, m, d_pairs, nullptr, d_count, ws, ws_bytes,
                  d_pairs ? d_pairs + m : nullptr, s};
    c.spin_limit = spin_limit;
    c.skip_first_tile = true;
    return dispatch(idx, c);
}

int launch_pairs_unordered(const gj_index* idx, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                           uint64_t* d_count, void* ws, size_t ws_bytes, cudaStream_t s) {
    lookup_call c{lookup_action::pairs, d_probes, nullptr, m, d_pairs, nullptr, d_count, ws, ws_bytes, nullptr, s};
    c.unordered = true;
    return dispatch(idx, c);
}

int pairs_error_flag(void* ws, size_t ws_bytes, uint64_t m, unsigned int* flag, cudaStream_t s) {
    pairs_ws pw;
    size_t used = 0;
    if (!carve_pairs_ws(ws, ws_bytes, m, &pw, &used)) return GJ_ERR_WORKSPACE;
    GJ_CUDA_TRY(cudaMemcpyAsync(flag, pw.error, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    return GJ_OK;
}

}  // namespace gj
