// gj_lookup_btree.cu -- B+tree probe kernels for plain nodes of 4 and 8 separators.
#include "gj_lookup_kernels.cuh"

namespace gj {

template <>
int lookup_call_btree<4>(const gj_index* idx, const lookup_call& c) {
    return run_call(op_btree<4>{idx->bt}, idx, c);
}

template <>
int lookup_call_btree<8>(const gj_index* idx, const lookup_call& c) {
    return run_call(op_btree<8>{idx->bt}, idx, c);
}

}  // namespace gj
