// gj_lookup_cooperative.cu -- gj_index_lookup_cooperative: the probe pass
// with the warp-collective searches of include/gpujoin/device.cuh, the
// counterparts of the reference's cooperative_binary_search
// (src/search.cuh:355-386) and harmonia_tree::lookup<Degree>
// (src/harmonia.cuh:740-786), launched as the reference launches
// lookup_kernel (src/index_lookup_common.cuh:217-245: the loop bound rounded
// up to whole warps, so that every lane reaches the collective call).
#include <cuda_runtime.h>

#include "gj_internal.h"

namespace gj {
namespace {

constexpr int kCoopBlock = 256;

template <unsigned kDegree, bool kHarmonia>
__global__ void __launch_bounds__(kCoopBlock) k_lookup_cooperative(const bs_view bs, const harmonia_view hm,
                                                                   const uint64_t* __restrict__ probes, uint64_t m,
                                                                   uint32_t* __restrict__ out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t limit = (m + 31) & ~31ull;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < limit; i += stride) {
        const bool active = i < m;
        const uint64_t key = active ? __ldcs(reinterpret_cast<const unsigned long long*>(probes) + i) : 0ull;
        uint32_t r;
        if constexpr (kHarmonia) {
            r = harmonia_lookup_cooperative<kDegree>(active, hm, key);
        } else {
            const uint64_t lb = cooperative_lower_bound<kDegree>(active, key, bs.col, bs.n);
            r = lb < bs.n ? (uint32_t)lb : kInvalid;
        }
        if (active) out[i] = r;
    }
}

template <unsigned kDegree>
int launch(const gj_index* idx, const uint64_t* probes, uint64_t m, uint32_t* out, cudaStream_t s) {
    device_info di;
    GJ_TRY(current_device_info(&di));
    const uint64_t want = (m + kCoopBlock - 1) / kCoopBlock;
    const uint64_t cap = (uint64_t)di.sm_count * 8;  // a grid-stride loop over 8 blocks per SM
    const unsigned grid = (unsigned)(want < cap ? (want ? want : 1) : cap);
    if (idx->type == GJ_INDEX_HARMONIA)
        k_lookup_cooperative<kDegree, true><<<grid, kCoopBlock, 0, s>>>(idx->bs, idx->hm, probes, m, out);
    else
        k_lookup_cooperative<kDegree, false><<<grid, kCoopBlock, 0, s>>>(idx->bs, idx->hm, probes, m, out);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

}  // namespace
}  // namespace gj

using namespace gj;

extern "C" int gj_index_lookup_cooperative(const gj_index* index, const uint64_t* d_probes, uint64_t m,
                                           uint32_t* d_positions, uint32_t degree, void* stream) {
    GJ_CHECK_ARG(index, "gj_index_lookup_cooperative: null index");
    GJ_CHECK_ARG(m == 0 || (d_probes && d_positions), "gj_index_lookup_cooperative: null buffer");
    GJ_CHECK_ARG(degree >= 1 && degree <= 5, "gj_index_lookup_cooperative: degree not in [1, 5]");
    if (index->type != GJ_INDEX_BINARY_SEARCH && index->type != GJ_INDEX_HARMONIA) {
        set_error("gj_index_lookup_cooperative: warp-collective searches exist for binary search and Harmonia");
        return GJ_ERR_UNSUPPORTED;
    }
    if (m == 0) return GJ_OK;
    cudaStream_t s = as_stream(stream);
    switch (degree) {
        case 1: return launch<1>(index, d_probes, m, d_positions, s);
        case 2: return launch<2>(index, d_probes, m, d_positions, s);
        case 3: return launch<3>(index, d_probes, m, d_positions, s);
        case 4: return launch<4>(index, d_probes, m, d_positions, s);
        default: return launch<5>(index, d_probes, m, d_positions, s);
    }
}
