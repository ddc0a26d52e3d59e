// gj_gen.cu -- synthetic build and probe columns, plus the device-wide scans
// they use.
//
// Replaces generate_datasets and its helpers (src/index_lookup_common.cuh:
// 44-206) and the Zipf sampler (src/zipf.hpp:13-102).  Unlike the reference,
// every generator is seeded and counter-based, so a (seed, size) pair always
// yields the same column on the same device code.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "gj_internal.h"

namespace gj {
namespace {

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr uint32_t kScanTile = kScanBlock * kScanItems;
constexpr uint32_t kScanMaxBlocks = 4096;

struct op_sum {
    __device__ __forceinline__ uint64_t operator()(uint64_t a, uint64_t b) const { return a + b; }
    static constexpr uint64_t identity = 0;
};
struct op_smax {
    __device__ __forceinline__ uint64_t operator()(uint64_t a, uint64_t b) const {
        return (int64_t)a > (int64_t)b ? a : b;
    }
    static constexpr uint64_t identity = 0x8000000000000000ull;  // INT64_MIN
};

template <class Op>
__device__ __forceinline__ uint64_t block_inclusive_scan(uint64_t v, uint64_t* s_warp, uint64_t* total) {
    Op op;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint64_t t = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v = op(t, v);
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = lane < kScanBlock / 32 ? s_warp[lane] : Op::identity;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t t = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w = op(t, w);
        }
        if (lane < kScanBlock / 32) s_warp[lane] = w;
    }
    __syncthreads();
    if (warp > 0) v = op(s_warp[warp - 1], v);
    *total = s_warp[kScanBlock / 32 - 1];
    __syncthreads();
    return v;
}

// phase 1: per-block reduction of a contiguous chunk
template <class Op>
__global__ void __launch_bounds__(kScanBlock) k_scan_reduce(const uint64_t* __restrict__ d, uint64_t n, uint64_t chunk,
                                                            uint64_t* __restrict__ block_sums) {
    __shared__ uint64_t s_warp[kScanBlock / 32];
    Op op;
    const uint64_t b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    uint64_t acc = Op::identity;
    for (uint64_t i = b0 + threadIdx.x; i < b1; i += kScanBlock) acc = op(acc, d[i]);
    uint64_t total;
    block_inclusive_scan<Op>(acc, s_warp, &total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// phase 2: exclusive scan of the block sums (one block)
template <class Op>
__global__ void __launch_bounds__(kScanBlock) k_scan_block_sums(uint64_t* __restrict__ block_sums, uint32_t nb) {
    __shared__ uint64_t s_warp[kScanBlock / 32];
    Op op;
    uint64_t carry = Op::identity;
    for (uint32_t base = 0; base < nb; base += kScanBlock) {
        const uint32_t i = base + threadIdx.x;
        const uint64_t v = i < nb ? block_sums[i] : Op::identity;
        uint64_t total;
        const uint64_t incl = block_inclusive_scan<Op>(v, s_warp, &total);
        // exclusive value = carry op (incl without v): recompute via shuffle of inclusive
        uint64_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
        __shared__ uint64_t s_last[kScanBlock / 32];
        if ((threadIdx.x & 31) == 31) s_last[threadIdx.x >> 5] = incl;
        __syncthreads();
        if ((threadIdx.x & 31) == 0) excl = (threadIdx.x == 0) ? Op::identity : s_last[(threadIdx.x >> 5) - 1];
        __syncthreads();
        if (i < nb) block_sums[i] = op(carry, excl);
        carry = op(carry, total);
        __syncthreads();
    }
}

// phase 3: scan each chunk with its block prefix
template <class Op>
__global__ void __launch_bounds__(kScanBlock) k_scan_apply(uint64_t* __restrict__ d, uint64_t n, uint64_t chunk,
                                                           const uint64_t* __restrict__ block_prefix) {
    __shared__ uint64_t s_warp[kScanBlock / 32];
    Op op;
    const uint64_t b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
    uint64_t carry = block_prefix[blockIdx.x];
    for (uint64_t t = b0; t < b1; t += kScanTile) {
        // each thread owns kScanItems consecutive elements of the tile
        uint64_t v[kScanItems];
        uint64_t local = Op::identity;
        const uint64_t my0 = t + (uint64_t)threadIdx.x * kScanItems;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            const uint64_t i = my0 + k;
            v[k] = i < b1 ? d[i] : Op::identity;
            local = op(local, v[k]);
        }
        uint64_t total;
        const uint64_t incl = block_inclusive_scan<Op>(local, s_warp, &total);
        uint64_t run = op(carry, Op::identity);
        // exclusive prefix of this thread = incl without local
        uint64_t excl = __shfl_up_sync(0xffffffffu, incl, 1);
        __shared__ uint64_t s_last[kScanBlock / 32];
        if ((threadIdx.x & 31) == 31) s_last[threadIdx.x >> 5] = incl;
        __syncthreads();
        if ((threadIdx.x & 31) == 0) excl = (threadIdx.x == 0) ? Op::identity : s_last[(threadIdx.x >> 5) - 1];
        run = op(carry, excl);
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            const uint64_t i = my0 + k;
            run = op(run, v[k]);
            if (i < b1) d[i] = run;
        }
        carry = op(carry, total);
        __syncthreads();
    }
}

template <class Op>
int scan_impl(uint64_t* d, uint64_t n, void* ws, size_t ws_bytes, cudaStream_t s) {
    if (n == 0) return GJ_OK;
    uint64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb > kScanMaxBlocks) nb = kScanMaxBlocks;
    uint64_t chunk = (n + nb - 1) / nb;
    chunk = (chunk + kScanTile - 1) / kScanTile * kScanTile;
    nb = (n + chunk - 1) / chunk;
    workspace_carver wc(ws, ws_bytes);
    uint64_t* sums = wc.take<uint64_t>(nb);
    if (!sums) {
        set_error("scan: workspace too small");
        return GJ_ERR_WORKSPACE;
    }
    k_scan_reduce<Op><<<(unsigned)nb, kScanBlock, 0, s>>>(d, n, chunk, sums);
    k_scan_block_sums<Op><<<1, kScanBlock, 0, s>>>(sums, (uint32_t)nb);
    k_scan_apply<Op><<<(unsigned)nb, kScanBlock, 0, s>>>(d, n, chunk, sums);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

// ---------------------------------------------------------------------------
// random variates
// ---------------------------------------------------------------------------
__device__ __forceinline__ double u01_open(uint64_t seed, uint64_t index, uint64_t attempt) {
    // (0, 1]: never zero, so log() stays finite
    const uint64_t h = mix64(mix64(seed ^ 0x5851f42d4c957f2dull) + index * 0x2545f4914f6cdd1dull + attempt);
    return ((double)(h >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

// exponential spacings: gap_i = floor(E_i * mean) + 2, E_i ~ Exp(1)
__global__ void k_gaps(uint64_t* __restrict__ g, uint64_t n, double mean, uint64_t seed) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const double e = -log(u01_open(seed, i, 0));
        g[i] = (uint64_t)(e * mean) + 2;
    }
}

// T = S_{n-1} + the (n+1)-th spacing, computed before any key is rescaled
__global__ void k_total(const uint64_t* __restrict__ d, uint64_t n, uint64_t* __restrict__ aux) {
    aux[1] = d[n - 1] + aux[0];
}

// key_i = floor(S_i * upper / T), exact in 128 bits (strictly increasing
// because every gap >= 2 and upper / T > 1)
__global__ void k_scale(uint64_t* __restrict__ d, uint64_t n, uint64_t upper, const uint64_t* __restrict__ aux) {
    const uint64_t T = aux[1];
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned __int128 p = (unsigned __int128)d[i] * upper;
        d[i] = (uint64_t)(p / T);
    }
}

// lognormal(0, 2) * 2^60 restricted to [0, upper): monotone transform of
// sorted uniforms u in (0, cdf_upper)
__global__ void k_lognormal(uint64_t* __restrict__ d, uint64_t n, double inv_unit, double cdf_upper, uint64_t upper) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        double u = ((double)d[i] + 0.5) * inv_unit * cdf_upper;
        if (u <= 0.0) u = 1e-300;
        const double z = normcdfinv(u);
        double v = exp(2.0 * z) * 1152921504606846976.0;  // 2^60
        uint64_t k = v >= (double)upper ? upper - 1 : (uint64_t)v;
        d[i] = k;
    }
}

// a_i = key_i - i (as signed) so that a max-scan makes the column strictly increasing
__global__ void k_sub_index(uint64_t* __restrict__ d, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        d[i] = (uint64_t)((int64_t)d[i] - (int64_t)i);
}
__global__ void k_add_index(uint64_t* __restrict__ d, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        d[i] = (uint64_t)((int64_t)d[i] + (int64_t)i);
}

// clustered keys: cluster c covers positions [start[c], start[c+1]) with
// keys base[c] + (i - start[c])
__global__ void k_clusters(uint64_t* __restrict__ d, uint64_t n, const uint64_t* __restrict__ start,
                           const uint64_t* __restrict__ base, uint32_t nc) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = nc;  // last c with start[c] <= i
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (start[mid] <= i) lo = mid; else hi = mid;
        }
        d[i] = base[lo] + (i - start[lo]);
    }
}

// --- Zipf by rejection-inversion (Hoermann & Derflinger 1996), as used by
// src/zipf.hpp:13-102: hat h(x) = x^-q, H(x) its integral, H^-1 its inverse
__device__ __forceinline__ double zf_expm1_over(double t) {
    return fabs(t) > 1e-8 ? expm1(t) / t : 1.0 + t * 0.5 * (1.0 + t / 3.0 * (1.0 + t * 0.25));
}
__device__ __forceinline__ double zf_log1p_over(double t) {
    return fabs(t) > 1e-8 ? log1p(t) / t : 1.0 - t * (0.5 - t * (1.0 / 3.0 - t * 0.25));
}
__device__ __forceinline__ double zf_H(double x, double q) {
    const double lx = log(x);
    return zf_expm1_over((1.0 - q) * lx) * lx;
}
__device__ __forceinline__ double zf_Hinv(double u, double q) {
    double t = u * (1.0 - q);
    if (t < -1.0) t = -1.0;
    return exp(zf_log1p_over(t) * u);
}

__device__ __forceinline__ uint64_t zipf_rank(uint64_t n, double q, double hx1, double hn, uint64_t seed, uint64_t i) {
    for (uint64_t a = 0; a < 1000; ++a) {
        const double u = hx1 + u01_open(seed, i, a) * (hn - hx1);
        const double x = zf_Hinv(u, q);
        const double kr = floor(x + 0.5);
        const uint64_t k = kr < 1.0 ? 1 : (kr > (double)n ? n : (uint64_t)kr);
        if (u >= zf_H((double)k + 0.5, q) - exp(-q * log((double)k))) return k;
    }
    return 1 + (mix64(seed ^ i) % n);  // unreachable in practice: bounded retries
}

// four-round Feistel permutation of [0, n) with cycle walking
__device__ __forceinline__ uint64_t permute(uint64_t x, uint64_t n, uint64_t seed, unsigned half) {
    const uint64_t mask = (1ull << half) - 1;
    for (int guard = 0; guard < 4096; ++guard) {
        uint64_t l = x >> half, r = x & mask;
#pragma unroll
        for (unsigned round = 0; round < 4; ++round) {
            const uint64_t f = mix64(r ^ (seed + 0x632be59bd9b4e019ull * (round + 1))) & mask;
            const uint64_t nl = r;
            r = l ^ f;
            l = nl;
        }
        x = (l << half) | r;
        if (x < n) return x;
    }
    return x % n;
}

__device__ uint64_t absent_key(const uint64_t* __restrict__ col, uint64_t n, uint64_t h) {
    uint64_t p = h % n;
    const uint64_t h2 = mix64(h);
    for (int step = 0; step < 64; ++step, ++p) {
        if (p + 1 >= n) break;
        const uint64_t a = col[p], b = col[p + 1];
        if (b - a >= 2) return a + 1 + (h2 % (b - a - 1));
    }
    if (col[n - 1] < UINT64_MAX - 1024) return col[n - 1] + 1 + (h2 % 1024);
    if (col[0] > 0) return h2 % col[0];
    return col[n - 1];  // no gap exists anywhere near: degenerate column
}

__global__ void k_probes(const uint64_t* __restrict__ col, uint64_t n, uint64_t* __restrict__ probes, uint64_t m,
                         double q, double hx1, double hn, double absent_fraction, uint64_t seed, unsigned half) {
    const uint64_t perm_seed = mix64(seed ^ 0xa0761d6478bd642full);
    const uint64_t absent_cut = (uint64_t)(absent_fraction * 18446744073709551615.0);
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h = mix64(mix64(seed + 0x9e3779b97f4a7c15ull) ^ (i * 0xbf58476d1ce4e5b9ull));
        if (absent_fraction > 0.0 && mix64(h) < absent_cut) {
            probes[i] = absent_key(col, n, h);
            continue;
        }
        uint64_t rank;
        if (q == 0.0) rank = 1 + (h % n);
        else rank = zipf_rank(n, q, hx1, hn, seed, i);
        const uint64_t pos = permute(rank - 1, n, perm_seed, half);
        probes[i] = col[pos];
    }
}

double host_zf_H(double x, double q) {
    const double lx = std::log(x);
    const double t = (1.0 - q) * lx;
    const double f = std::fabs(t) > 1e-8 ? std::expm1(t) / t : 1.0 + t * 0.5 * (1.0 + t / 3.0 * (1.0 + t * 0.25));
    return f * lx;
}

int grid_of(uint64_t work) {
    uint64_t g = (work + 255) / 256;
    if (g > 8192) g = 8192;
    return (int)(g ? g : 1);
}

}  // namespace

size_t scan_workspace_bytes(uint64_t) { return workspace_carver::need({kScanMaxBlocks * sizeof(uint64_t)}); }

int inclusive_scan_sum(uint64_t* d, uint64_t n, void* ws, size_t ws_bytes, cudaStream_t s) {
    return scan_impl<op_sum>(d, n, ws, ws_bytes, s);
}

int inclusive_scan_max_signed(int64_t* d, uint64_t n, void* ws, size_t ws_bytes, cudaStream_t s) {
    return scan_impl<op_smax>(reinterpret_cast<uint64_t*>(d), n, ws, ws_bytes, s);
}

}  // namespace gj

using namespace gj;

extern "C" {

int gj_generate_workspace_size(uint64_t n, size_t* bytes) {
    GJ_CHECK_ARG(bytes, "gj_generate_workspace_size: null argument");
    *bytes = workspace_carver::need({scan_workspace_bytes(n), 64, 2048 * sizeof(uint64_t)});
    return GJ_OK;
}

int gj_generate_sorted_keys(uint64_t* d_keys, uint64_t n, uint32_t distribution, uint64_t upper, uint64_t seed,
                            void* d_workspace, size_t workspace_bytes, void* stream) {
    GJ_CHECK_ARG(d_keys || n == 0, "gj_generate_sorted_keys: null buffer");
    GJ_CHECK_ARG(distribution <= GJ_DIST_CLUSTERS, "gj_generate_sorted_keys: unknown distribution");
    if (n == 0) return GJ_OK;
    if (upper < 4 * n || upper > (1ull << 63)) {
        set_error("gj_generate_sorted_keys: need 4n <= upper <= 2^63");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = as_stream(stream);
    workspace_carver wc(d_workspace, workspace_bytes);
    void* scan_ws = wc.take<char>(scan_workspace_bytes(n));
    uint64_t* aux = wc.take<uint64_t>(8);
    uint64_t* cl = wc.take<uint64_t>(2048);
    if (!scan_ws || !aux || !cl) {
        set_error("gj_generate_sorted_keys: workspace too small");
        return GJ_ERR_WORKSPACE;
    }
    const size_t scan_bytes = scan_workspace_bytes(n);
    const int grid = grid_of(n);

    if (distribution == GJ_DIST_CLUSTERS) {
        // 1024 runs of consecutive keys; run sizes ~ exponential weights,
        // gaps between runs uniform in [2^24, 2^44)
        const uint32_t nc = (uint32_t)std::min<uint64_t>(1024, n);
        std::vector<double> w(nc);
        double sum = 0;
        for (uint32_t c = 0; c < nc; ++c) {
            const uint64_t h = mix64(mix64(seed ^ 0xc1u) + c);
            w[c] = -std::log(((double)(h >> 11) + 1.0) / 9007199254740992.0);
            sum += w[c];
        }
        std::vector<uint64_t> start(nc), base(nc);
        uint64_t pos = 0, key = mix64(seed ^ 0xba5eull) % (1ull << 40);
        for (uint32_t c = 0; c < nc; ++c) {
            uint64_t size = (c + 1 == nc) ? n - pos : (uint64_t)((double)n * w[c] / sum);
            if (size == 0) size = 1;
            if (pos + size > n - (nc - c - 1)) size = n - (nc - c - 1) - pos;
            start[c] = pos;
            base[c] = key;
            pos += size;
            key += size + (1ull << 24) + mix64(mix64(seed ^ 0x9a9u) + c) % ((1ull << 44) - (1ull << 24));
        }
        if (key > upper) {
            set_error("gj_generate_sorted_keys: clustered keys exceed the upper bound");
            return GJ_ERR_INVALID_ARGUMENT;
        }
        GJ_CUDA_TRY(cudaMemcpyAsync(cl, start.data(), nc * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
        GJ_CUDA_TRY(cudaMemcpyAsync(cl + 1024, base.data(), nc * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
        k_clusters<<<grid, 256, 0, s>>>(d_keys, n, cl, cl + 1024, nc);
        GJ_CUDA_TRY(cudaGetLastError());
        GJ_CUDA_TRY(cudaStreamSynchronize(s));  // host vectors go out of scope
        return GJ_OK;
    }

    // sorted uniform order statistics in [0, U): exponential spacings
    const uint64_t U = distribution == GJ_DIST_UNIFORM ? upper : (1ull << 53);
    // spacings are drawn at 1/64 of their final scale: an Exp(1) variate from a
    // 53-bit uniform is at most 36.8, so the n+1 spacings sum to at most
    // 0.58 * U < 2^63 and never overflow; the rescale below multiplies by > 1
    const double mean = (double)U / (double)(n + 1) / 64.0;
    k_gaps<<<grid, 256, 0, s>>>(d_keys, n, mean, seed);
    k_gaps<<<1, 32, 0, s>>>(aux, 1, mean, mix64(seed ^ 0x7a11ull));  // the (n+1)-th spacing
    GJ_TRY(inclusive_scan_sum(d_keys, n, scan_ws, scan_bytes, s));
    k_total<<<1, 1, 0, s>>>(d_keys, n, aux);
    k_scale<<<grid, 256, 0, s>>>(d_keys, n, U, aux);
    GJ_CUDA_TRY(cudaGetLastError());
    if (distribution == GJ_DIST_LOGNORMAL) {
        // P(lognormal(0,2) * 2^60 < upper)
        const double zu = std::log((double)upper / 1152921504606846976.0) / 2.0;
        const double cdf_upper = 0.5 * std::erfc(-zu / std::sqrt(2.0));
        k_lognormal<<<grid, 256, 0, s>>>(d_keys, n, 1.0 / (double)U, cdf_upper, upper);
        // enforce strict increase: key'_i = max_{j<=i}(key_j - j) + i
        k_sub_index<<<grid, 256, 0, s>>>(d_keys, n);
        GJ_TRY(inclusive_scan_max_signed(reinterpret_cast<int64_t*>(d_keys), n, scan_ws, scan_bytes, s));
        k_add_index<<<grid, 256, 0, s>>>(d_keys, n);
        GJ_CUDA_TRY(cudaGetLastError());
    }
    return GJ_OK;
}

int gj_generate_probes(const uint64_t* d_keys, uint64_t n, uint64_t* d_probes, uint64_t m, double theta,
                       double absent_fraction, uint64_t seed, void* stream) {
    GJ_CHECK_ARG(d_keys && n > 0, "gj_generate_probes: empty build column");
    GJ_CHECK_ARG(d_probes || m == 0, "gj_generate_probes: null output");
    GJ_CHECK_ARG(theta >= 0.0 && theta < 8.0, "gj_generate_probes: theta out of range");
    GJ_CHECK_ARG(absent_fraction >= 0.0 && absent_fraction <= 1.0, "gj_generate_probes: bad absent fraction");
    if (m == 0) return GJ_OK;
    unsigned bits = n <= 1 ? 2 : 64u - (unsigned)__builtin_clzll(n - 1);
    if (bits < 2) bits = 2;
    if (bits & 1u) bits++;
    const double hx1 = theta == 0.0 ? 0.0 : host_zf_H(1.5, theta) - 1.0;
    const double hn = theta == 0.0 ? 0.0 : host_zf_H((double)n + 0.5, theta);
    k_probes<<<grid_of(m), 256, 0, as_stream(stream)>>>(d_keys, n, d_probes, m, theta, hx1, hn, absent_fraction,
                                                       seed, bits / 2);
    GJ_CUDA_TRY(cudaGetLastError());
    return GJ_OK;
}

}  // extern "C"
