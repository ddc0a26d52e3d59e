// gj_lookup_harmonia_rs.cu -- Harmonia and RadixSpline probe kernels.
#include "gj_lookup_kernels.cuh"

namespace gj {

int lookup_call_harmonia(const gj_index* idx, const lookup_call& c) { return run_call(op_harmonia{idx->hm}, idx, c); }
int lookup_call_rs(const gj_index* idx, const lookup_call& c) { return run_call(op_rs{idx->rs}, idx, c); }

}  // namespace gj
