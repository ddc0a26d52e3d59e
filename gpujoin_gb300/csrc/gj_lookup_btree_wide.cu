// gj_lookup_btree_wide.cu -- B+tree probe kernels for plain nodes of 16, 32 and 64 separators.
#include "gj_lookup_kernels.cuh"

namespace gj {

template <>
int lookup_call_btree<16>(const gj_index* idx, const lookup_call& c) {
    return run_call(op_btree<16>{idx->bt}, idx, c);
}

template <>
int lookup_call_btree<32>(const gj_index* idx, const lookup_call& c) {
    return run_call(op_btree<32>{idx->bt}, idx, c);
}

template <>
int lookup_call_btree<64>(const gj_index* idx, const lookup_call& c) {
    return run_call(op_btree<64>{idx->bt}, idx, c);
}

}  // namespace gj
