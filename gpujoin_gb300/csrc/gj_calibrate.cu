// gj_calibrate.cu -- the random 32-byte sector read rate of this GPU, the
// second roofline of the probe path (besides HBM bandwidth): a scattered
// lookup whose column does not fit L2 must read at least one random sector
// per probe, so probes/s cannot exceed random sectors/s.  No counterpart in
// the reference.
//
// k_random_sectors reads m sectors at pseudo-random sector indexes of a
// buffer of n_sectors sectors (a counter-based hash of the load number, so
// the addresses do not depend on earlier loads and every thread keeps
// kSectorsInFlight loads in flight), and folds the loaded words into one
// word per thread so that the loads cannot be dropped.  fill64 = 1 asks L2
// to fill 64 bytes on a miss (.L2::64B), as the probe kernels' scattered
// loads do; 0 leaves the default fill.
#include <cuda_runtime.h>

#include <cstdint>

#include "gj_internal.h"

namespace gj {
namespace {

constexpr int kCalBlock = 256;
constexpr int kSectorsInFlight = 4;
constexpr int kCalBlocksPerSM = 4;  // resident blocks per SM at the register cap below

__device__ __forceinline__ uint64_t mix(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

template <bool kFill64>
__global__ void __launch_bounds__(kCalBlock, kCalBlocksPerSM)
    k_random_sectors(const uint64_t* __restrict__ buf, uint64_t n_sectors, uint64_t m, uint64_t seed,
                     uint64_t* __restrict__ sink) {
    const uint64_t tid = (uint64_t)blockIdx.x * kCalBlock + threadIdx.x;
    const uint64_t stride = (uint64_t)gridDim.x * kCalBlock * kSectorsInFlight;
    uint64_t acc = 0;
    for (uint64_t base = tid * kSectorsInFlight; base < m; base += stride) {
        uint64_t k[kSectorsInFlight][4];
#pragma unroll
        for (int u = 0; u < kSectorsInFlight; ++u) {
            const uint64_t i = base + u;
            const uint64_t s = mix(i ^ seed) % n_sectors;
            if (i < m) {
                if constexpr (kFill64) ld_sector_64(buf + 4 * s, k[u]);
                else ld_sector(buf + 4 * s, k[u]);
            } else {
                k[u][0] = k[u][1] = k[u][2] = k[u][3] = 0;
            }
        }
#pragma unroll
        for (int u = 0; u < kSectorsInFlight; ++u) acc ^= k[u][0] ^ k[u][1] ^ k[u][2] ^ k[u][3];
    }
    sink[tid] = acc;
}

}  // namespace
}  // namespace gj

using namespace gj;

extern "C" {

int gj_calibrate_sink_words(uint64_t* words) {
    GJ_CHECK_ARG(words, "gj_calibrate_sink_words: null argument");
    device_info di;
    GJ_TRY(current_device_info(&di));
    *words = (uint64_t)di.sm_count * kCalBlocksPerSM * kCalBlock;
    return GJ_OK;
}

int gj_calibrate_random_sectors(const uint64_t* d_buf, uint64_t n_sectors, uint64_t m, uint64_t seed, uint32_t fill64,
                                uint64_t* d_sink, void* stream) {
    GJ_CHECK_ARG(d_buf && d_sink && n_sectors > 0, "gj_calibrate_random_sectors: null buffer or no sectors");
    GJ_CHECK_ARG((reinterpret_cast<uintptr_t>(d_buf) & 31) == 0, "gj_calibrate_random_sectors: buffer not 32-byte aligned");
    device_info di;
    GJ_TRY(current_device_info(&di));
    const unsigned grid = (unsigned)di.sm_count * kCalBlocksPerSM;
    cudaStream_t s = as_stream(stream);
    if (fill64)
        k_random_sectors<true><<<grid, kCalBlock, 0, s>>>(d_buf, n_sectors, m, seed, d_sink);
    else
        k_random_sectors<false><<<grid, kCalBlock, 0, s>>>(d_buf, n_sectors, m, seed, d_sink);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

}  // extern "C"
