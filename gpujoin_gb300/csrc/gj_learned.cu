// gj_learned.cu -- learned position model: a root model (1 -> H -> H -> 1 ReLU
// MLP, a linear model, or a table of equal-width key segments with the CDF at
// their ends) routes a key to one of L linear leaf models; the
// leaf predicts the position and a recorded error window bounds an exact
// search (device side in gpujoin/device.cuh: learned_lookup).
//
// Not in the reference.  Training runs on the GPU with the kernels below:
//   k_make_samples      (key, position) training pairs, stratified over the column
//   k_mlp_grad          forward + backward of the root MLP over a mini-batch,
//                       per-block partial gradients (fixed reduction order)
//   k_reduce_partials   sum of the block partials -> gradient
//   k_adam              Adam step
//   k_linear_sums       least-squares sums for the linear root
//   k_segment_ends      positions of the segment ends of the segment-table root
//   k_route             leaf of every build key (the lookup's own arithmetic)
//   k_leaf_params       leaf anchors (first key, position) and slopes
//   k_leaf_error        largest under/over-prediction per leaf
// Determinism: every reduction runs in a fixed order, so the same column,
// parameters and seed give the same model on the same device code.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "gj_internal.h"

namespace gj {

int device_alloc_for(gj_index* idx, size_t bytes, void** out);  // gj_index.cu
uint32_t column_aligned32(const void* p);                        // gj_index.cu

namespace {

constexpr int kTrainBlock = 256;
constexpr int kMaxHidden = 32;

__host__ __device__ inline uint32_t mlp_param_count(uint32_t H) { return 2 * H + H * H + H + H + 1; }

__device__ __forceinline__ double u01(uint64_t seed, uint64_t i) {
    return (double)(mix64(mix64(seed) ^ (i * 0x9e3779b97f4a7c15ull)) >> 11) * (1.0 / 9007199254740992.0);
}

// samples: position p_s = floor((s + u_s) * n / S), x = norm(key[p]), y = p / n
__global__ void k_make_samples(const uint64_t* __restrict__ col, uint64_t n, uint64_t S, uint64_t min_key,
                               float inv_range, uint64_t max_key, uint64_t seed, float* __restrict__ x,
                               float* __restrict__ y) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < S; s += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t p = (uint64_t)(((double)s + u01(seed, s)) * (double)n / (double)S);
        if (p >= n) p = n - 1;
        const uint64_t key = col[p];
        x[s] = key <= min_key ? 0.f : (key >= max_key ? 1.f : (float)(key - min_key) * inv_range);
        y[s] = (float)((double)p / (double)n);
    }
}

// Forward + backward for kTrainBlock samples per block.  The gradient of the
// summed squared error (scaled by `scale`) is written as this block's partial.
// Shared memory: parameters, then a1, d2, d1 (kTrainBlock x H floats each),
// then x and dL/dout per sample.
__global__ void __launch_bounds__(kTrainBlock) k_mlp_grad(const float* __restrict__ P, int H,
                                                          const float* __restrict__ xs, const float* __restrict__ ys,
                                                          uint64_t count, const uint32_t* __restrict__ batch_idx,
                                                          float scale, float* __restrict__ partial,
                                                          double* __restrict__ loss_partial) {
    extern __shared__ float sm[];
    const int np = 2 * H + H * H + H + H + 1;
    float* sP = sm;                       // np
    float* sH1 = sP + ((np + 3) & ~3);    // kTrainBlock * H: pre-activations a1
    float* sD2 = sH1 + kTrainBlock * H;   // kTrainBlock * H
    float* sD1 = sD2 + kTrainBlock * H;   // kTrainBlock * H
    float* sX = sD1 + kTrainBlock * H;    // kTrainBlock
    float* sDout = sX + kTrainBlock;      // kTrainBlock
    __shared__ double s_loss[kTrainBlock / 32];
    for (int i = threadIdx.x; i < np; i += blockDim.x) sP[i] = P[i];
    __syncthreads();
    const float* W1 = sP;
    const float* b1 = sP + H;
    const float* W2 = sP + 2 * H;
    const float* b2 = W2 + H * H;
    const float* W3 = b2 + H;
    const float b3 = W3[H];

    const uint64_t s = (uint64_t)blockIdx.x * kTrainBlock + threadIdx.x;
    const bool valid = s < count;
    float xv = 0.f, yv = 0.f;
    if (valid) {
        const uint64_t j = batch_idx ? batch_idx[s] : s;
        xv = xs[j];
        yv = ys[j];
    }
    float h1[kMaxHidden], a2v[kMaxHidden];
#pragma unroll
    for (int j = 0; j < kMaxHidden; ++j) {
        if (j < H) {
            const float a = fmaf(W1[j], xv, b1[j]);
            h1[j] = a > 0.f ? a : 0.f;
            sH1[threadIdx.x * H + j] = a;  // pre-activation a1
        }
    }
    float out = b3;
    for (int o = 0; o < H; ++o) {
        float a = b2[o];
#pragma unroll
        for (int j = 0; j < kMaxHidden; ++j)
            if (j < H) a = fmaf(W2[o * H + j], h1[j], a);
        a2v[o] = a;
        out = fmaf(W3[o], a > 0.f ? a : 0.f, out);
    }
    const float diff = valid ? out - yv : 0.f;
    const float dout = valid ? 2.f * diff * scale : 0.f;
    double l = valid ? (double)diff * (double)diff : 0.0;
    // d2 = dout * W3 * relu'(a2); d1 = W2^T d2 * relu'(a1)
    for (int o = 0; o < H; ++o) sD2[threadIdx.x * H + o] = a2v[o] > 0.f ? dout * W3[o] : 0.f;
    for (int j = 0; j < H; ++j) {
        float acc = 0.f;
        for (int o = 0; o < H; ++o) acc = fmaf(sD2[threadIdx.x * H + o], W2[o * H + j], acc);
        sD1[threadIdx.x * H + j] = sH1[threadIdx.x * H + j] > 0.f ? acc : 0.f;
    }
    sX[threadIdx.x] = xv;
    sDout[threadIdx.x] = dout;
    // loss (double) block reduction
    for (int d = 16; d > 0; d >>= 1) l += __shfl_down_sync(0xffffffffu, l, d);
    if ((threadIdx.x & 31) == 0) s_loss[threadIdx.x >> 5] = l;
    __syncthreads();
    // per-parameter sums over the block's samples (fixed order)
    float* part = partial + (uint64_t)blockIdx.x * np;
    for (int p = threadIdx.x; p < np; p += blockDim.x) {
        float acc = 0.f;
        if (p < H) {  // W1[j]: sum d1[s][j] * x[s]
            for (int t = 0; t < kTrainBlock; ++t) acc = fmaf(sD1[t * H + p], sX[t], acc);
        } else if (p < 2 * H) {  // b1
            const int j = p - H;
            for (int t = 0; t < kTrainBlock; ++t) acc += sD1[t * H + j];
        } else if (p < 2 * H + H * H) {  // W2[o][j]: sum d2[s][o] * h1[s][j]
            const int q = p - 2 * H, o = q / H, j = q % H;
            for (int t = 0; t < kTrainBlock; ++t) acc = fmaf(sD2[t * H + o], fmaxf(sH1[t * H + j], 0.f), acc);
        } else if (p < 3 * H + H * H) {  // b2
            const int o = p - 2 * H - H * H;
            for (int t = 0; t < kTrainBlock; ++t) acc += sD2[t * H + o];
        } else if (p < 4 * H + H * H) {  // W3[o]: sum dout * h2[o]; h2 = d2/(dout*W3) is not stored, recompute
            acc = 0.f;  // filled below
        } else {  // b3
            for (int t = 0; t < kTrainBlock; ++t) acc += sDout[t];
        }
        part[p] = acc;
    }
    __syncthreads();
    // W3 needs h2 = relu(a2); reuse the D1 buffer for h2 of every sample
    for (int o = 0; o < H; ++o) sD1[threadIdx.x * H + o] = a2v[o] > 0.f ? a2v[o] : 0.f;
    __syncthreads();
    for (int o = threadIdx.x; o < H; o += blockDim.x) {
        float acc = 0.f;
        for (int t = 0; t < kTrainBlock; ++t) acc = fmaf(sDout[t], sD1[t * H + o], acc);
        part[3 * H + H * H + o] = acc;
    }
    if (threadIdx.x == 0 && loss_partial) {
        double tot = 0;
        for (int w = 0; w < kTrainBlock / 32; ++w) tot += s_loss[w];
        loss_partial[blockIdx.x] = tot;
    }
}

__global__ void k_reduce_partials(const float* __restrict__ partial, int np, int nblocks, float* __restrict__ grad,
                                  const double* __restrict__ loss_partial, double* __restrict__ loss) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int b = 0; b < nblocks; ++b) acc += partial[(uint64_t)b * np + p];
        grad[p] = acc;
    }
    if (loss && blockIdx.x == 0 && threadIdx.x == 0) {
        double t = 0;
        for (int b = 0; b < nblocks; ++b) t += loss_partial[b];
        *loss = t;
    }
}

__global__ void k_adam(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, int np, float lr, float b1, float b2, float eps, float c1, float c2) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const float gi = g[p];
        const float a = b1 * m1[p] + (1.f - b1) * gi;
        const float v = b2 * m2[p] + (1.f - b2) * gi * gi;
        m1[p] = a;
        m2[p] = v;
        P[p] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
    }
}

__global__ void k_batch_indices(uint32_t* __restrict__ idx, uint32_t B, uint64_t S, uint64_t seed, uint32_t step) {
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x)
        idx[b] = (uint32_t)(mix64(mix64(seed + step) ^ ((uint64_t)b * 0xbf58476d1ce4e5b9ull)) % S);
}

// least-squares sums over the samples for the linear root (per block, fixed order)
__global__ void __launch_bounds__(kTrainBlock) k_linear_sums(const float* __restrict__ xs, const float* __restrict__ ys,
                                                             uint64_t S, double* __restrict__ partial) {
    double sx = 0, sy = 0, sxx = 0, sxy = 0;
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < S; s += (uint64_t)gridDim.x * blockDim.x) {
        const double x = xs[s], y = ys[s];
        sx += x;
        sy += y;
        sxx += x * x;
        sxy += x * y;
    }
    __shared__ double sh[4][kTrainBlock];
    sh[0][threadIdx.x] = sx;
    sh[1][threadIdx.x] = sy;
    sh[2][threadIdx.x] = sxx;
    sh[3][threadIdx.x] = sxy;
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0;
        for (int i = 0; i < kTrainBlock; ++i) t += sh[threadIdx.x][i];
        partial[blockIdx.x * 4 + threadIdx.x] = t;
    }
}

// leaf of every build key; per leaf: first / last position and key count
// (warp-aggregated atomics: consecutive keys mostly share a leaf)
__global__ void k_route(learned_view v, const float* __restrict__ root, uint32_t* __restrict__ leaf_of,
                        unsigned int* __restrict__ first, unsigned int* __restrict__ last,
                        unsigned int* __restrict__ count) {
    extern __shared__ __align__(8) float s_root[];
    const int np = v.root_kind == GJ_LEARNED_ROOT_MLP ? kMlpParams : 2;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s_root[i] = root[i];
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_round = (v.n + 31) & ~31ull;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_round; i += stride) {
        const bool valid = i < v.n;
        uint32_t leaf = 0xFFFFFFFFu;
        if (valid) {
            leaf = learned_route(v, s_root, learned_norm(v, v.col[i]));
            leaf_of[i] = leaf;
        }
        const unsigned group = __match_any_sync(0xffffffffu, leaf);
        if (!valid) continue;
        const int leader = __ffs(group) - 1;
        const int tail = 31 - __clz(group);
        const int lane = threadIdx.x & 31;
        if (lane == leader) {
            atomicMin(&first[leaf], (unsigned int)i);
            atomicAdd(&count[leaf], (unsigned int)__popc(group));
        }
        if (lane == tail) atomicMax(&last[leaf], (unsigned int)i);
    }
}

__global__ void k_leaf_params(const uint64_t* __restrict__ col, uint32_t L, const unsigned int* __restrict__ first,
                              const unsigned int* __restrict__ last, const unsigned int* __restrict__ count,
                              learned_leaf* __restrict__ leaves) {
    for (uint32_t l = blockIdx.x * blockDim.x + threadIdx.x; l < L; l += gridDim.x * blockDim.x) {
        learned_leaf lf{};
        if (count[l] > 0) {
            const uint32_t a = first[l], b = last[l];
            lf.x0 = col[a];
            lf.base = a;
            const uint64_t dk = col[b] - col[a];
            lf.slope = (b > a && dk > 0) ? (float)((double)(b - a) / (double)dk) : 0.f;
        }
        lf.err_lo = 0;
        lf.err_hi = 0;
        leaves[l] = lf;
    }
}

__global__ void k_leaf_error(learned_view v, const uint32_t* __restrict__ leaf_of, learned_leaf* __restrict__ leaves) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t n_round = (v.n + 31) & ~31ull;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n_round; i += stride) {
        const bool valid = i < v.n;
        uint32_t leaf = 0xFFFFFFFFu, lo = 0, hi = 0;
        if (valid) {
            leaf = leaf_of[i];
            const learned_leaf lf = leaves[leaf];
            const int64_t d = (int64_t)i - learned_predict(lf, v.col[i]);
            const int64_t cap = 0xFFFFFFFFll;
            hi = d > 0 ? (uint32_t)(d > cap ? cap : d) : 0u;
            lo = d < 0 ? (uint32_t)(-d > cap ? cap : -d) : 0u;
        }
        const unsigned group = __match_any_sync(0xffffffffu, leaf);
        const unsigned ghi = __reduce_max_sync(group, hi);
        const unsigned glo = __reduce_max_sync(group, lo);
        if (valid && (int)(threadIdx.x & 31) == __ffs(group) - 1) {
            if (ghi) atomicMax(reinterpret_cast<unsigned int*>(&leaves[leaf].err_hi), ghi);
            if (glo) atomicMax(reinterpret_cast<unsigned int*>(&leaves[leaf].err_lo), glo);
        }
    }
}

// position of the first key >= the start of segment k (k in [0, S]) of the
// key range [min_key, max_key] cut into S equal-width segments; S itself ends
// at n
__global__ void k_segment_ends(const uint64_t* __restrict__ col, uint64_t n, uint64_t min_key, uint64_t max_key,
                               uint32_t S, uint64_t* __restrict__ pos) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > S) return;
    if (k == S) {
        pos[k] = n;
        return;
    }
    // min_key + floor(k * range / S) without overflow: S is a power of two
    const uint64_t range = max_key - min_key;
    const uint64_t key = min_key + (range / S) * k + ((range % S) * k) / S;
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        const uint64_t mid = lo + (hi - lo) / 2;
        if (col[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    pos[k] = lo;
}

int grid_for_n(uint64_t n) {
    uint64_t g = (n + 255) / 256;
    return (int)std::min<uint64_t>(g ? g : 1, 4096);
}

struct scratch {
    std::vector<void*> ptrs;
    ~scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    int alloc(size_t count, T** out) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e != cudaSuccess) {
            set_error("learned index: cudaMalloc(%zu) failed: %s", count * sizeof(T), cudaGetErrorString(e));
            return GJ_ERR_OUT_OF_MEMORY;
        }
        ptrs.push_back(p);
        *out = static_cast<T*>(p);
        return GJ_OK;
    }
};

// Quantile initialisation: the network starts as the piecewise-linear CDF
// through H + 1 sample quantiles (q_j, y_j): h1_j = relu(x - q_j), layer 2
// passes h1 through (identity weights; h1 >= 0), and the output weights are
// the slope changes at the knots.  Training then refines this fit.
void init_mlp_quantiles(std::vector<float>& P, uint32_t H, const std::vector<float>& q, const std::vector<float>& y) {
    const uint32_t np = mlp_param_count(H);
    P.assign(np, 0.f);
    float* W1 = P.data();
    float* b1 = W1 + H;
    float* W2 = b1 + H;
    float* b2 = W2 + H * H;
    float* W3 = b2 + H;
    float* b3 = W3 + H;
    double prev = 0.0;
    for (uint32_t j = 0; j < H; ++j) {
        W1[j] = 1.f;
        b1[j] = -q[j];
        W2[j * H + j] = 1.f;
        b2[j] = 0.f;
        const double dq = std::max(1e-7, (double)q[j + 1] - (double)q[j]);
        const double slope = ((double)y[j + 1] - (double)y[j]) / dq;
        W3[j] = (float)(slope - prev);
        prev = slope;
    }
    b3[0] = y[0];
}

}  // namespace

// gradient of the summed squared error over `count` samples (the GPU
// backward pass, exposed for checking against the CPU oracle)
int mlp_grad(const float* d_params, uint32_t H, const float* d_x, const float* d_y, uint64_t count, float* d_grad,
             double* d_loss, cudaStream_t s) {
    if (H == 0 || H > (uint32_t)kMaxHidden) {
        set_error("mlp: hidden width must be in [1, 32]");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    const int np = (int)mlp_param_count(H);
    const int nblocks = (int)std::max<uint64_t>(1, (count + kTrainBlock - 1) / kTrainBlock);
    scratch sc;
    float* partial = nullptr;
    double* lp = nullptr;
    GJ_TRY(sc.alloc(nblocks * (size_t)np, &partial));
    GJ_TRY(sc.alloc(nblocks, &lp));
    const size_t smem = (((np + 3) & ~3) + 3 * kTrainBlock * H + 2 * kTrainBlock) * sizeof(float);
    GJ_CUDA_TRY(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_mlp_grad<<<nblocks, kTrainBlock, smem, s>>>(d_params, (int)H, d_x, d_y, count, nullptr, 1.0f, partial, lp);
    k_reduce_partials<<<(np + 255) / 256, 256, 0, s>>>(partial, np, nblocks, d_grad, lp, d_loss);
    GJ_CUDA_TRY(cudaGetLastError());
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    return GJ_OK;
}

int build_learned(gj_index* idx, cudaStream_t s) {
    const gj_index_params& p = idx->params;
    const uint64_t n = idx->n;
    // leaves: as given, or (0) about 128 keys per leaf -- a power of two in
    // [2^10, 2^20]; the leaf array (32 B a leaf) stays at most 32 MB
    uint32_t L = p.learned_leaves;
    if (L == 0) {
        L = 1u << 10;
        while (L < (1u << 20) && (uint64_t)L * 2 * 128 <= n) L <<= 1;
    }
    if (L > (1u << 24)) {
        set_error("learned index: leaves must be in [1, 2^24]");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    if (p.learned_root != GJ_LEARNED_ROOT_LINEAR && p.learned_root != GJ_LEARNED_ROOT_MLP &&
        p.learned_root != GJ_LEARNED_ROOT_SEGMENTS) {
        set_error("learned index: unknown root model");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    const uint32_t H = p.learned_root == GJ_LEARNED_ROOT_MLP ? p.learned_hidden : 0;
    if (p.learned_root == GJ_LEARNED_ROOT_MLP && (H == 0 || H > (uint32_t)kMaxHidden)) {
        set_error("learned index: hidden width must be in [1, 32]");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    uint64_t ends[2] = {0, 0};
    GJ_CUDA_TRY(cudaMemcpyAsync(&ends[0], idx->d_col, 8, cudaMemcpyDefault, s));
    GJ_CUDA_TRY(cudaMemcpyAsync(&ends[1], idx->d_col + n - 1, 8, cudaMemcpyDefault, s));
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    learned_view& v = idx->ln;
    v.col = idx->d_col;
    v.n = n;
    v.min_key = ends[0];
    v.max_key = ends[1];
    v.inv_range = ends[1] > ends[0] ? (float)(1.0 / (double)(ends[1] - ends[0])) : 0.f;
    v.num_leaves = L;
    v.root_kind = p.learned_root;
    v.hidden = H;
    v.col_aligned = column_aligned32(idx->d_col);
    const bool segments = p.learned_root == GJ_LEARNED_ROOT_SEGMENTS;
    v.segments = segments ? kLearnedSegments : 0;

    const uint32_t np = p.learned_root == GJ_LEARNED_ROOT_MLP ? mlp_param_count(H) : 2;  // trained parameters
    const uint32_t nstored = p.learned_root == GJ_LEARNED_ROOT_MLP ? (uint32_t)kMlpParams
                             : segments                           ? 2 * kLearnedSegments
                                                                  : 2u;
    void* root_mem = nullptr;
    void* leaf_mem = nullptr;
    GJ_TRY(device_alloc_for(idx, nstored * sizeof(float), &root_mem));
    GJ_TRY(device_alloc_for(idx, (size_t)L * sizeof(learned_leaf), &leaf_mem));
    float* d_root = static_cast<float*>(root_mem);
    v.root = d_root;
    v.leaves = static_cast<learned_leaf*>(leaf_mem);
    idx->smem_words = 0;  // the lookup kernels take the root parameters by value
    idx->bytes = nstored * sizeof(float) + (uint64_t)L * sizeof(learned_leaf);
    std::memset(&idx->ln_root, 0, sizeof(idx->ln_root));

    scratch sc;
    if (segments) {
        // y = position / n at every segment end; a segment holds {y, dy}
        const uint32_t S = kLearnedSegments;
        uint64_t* d_pos = nullptr;
        GJ_TRY(sc.alloc(S + 1, &d_pos));
        k_segment_ends<<<(S + 1 + 255) / 256, 256, 0, s>>>(idx->d_col, n, v.min_key, v.max_key, S, d_pos);
        GJ_CUDA_TRY(cudaGetLastError());
        std::vector<uint64_t> pos(S + 1);
        GJ_CUDA_TRY(cudaMemcpyAsync(pos.data(), d_pos, pos.size() * sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        GJ_CUDA_TRY(cudaStreamSynchronize(s));
        std::vector<float> table(2 * S);
        for (uint32_t i = 0; i < S; ++i) {
            const double y0 = (double)pos[i] / (double)n, y1 = (double)pos[i + 1] / (double)n;
            table[2 * i] = (float)y0;
            table[2 * i + 1] = (float)(y1 - y0);
        }
        GJ_CUDA_TRY(cudaMemcpyAsync(d_root, table.data(), table.size() * sizeof(float), cudaMemcpyDefault, s));
        // the table's copy must land before `table` goes out of scope
        GJ_CUDA_TRY(cudaStreamSynchronize(s));
    }
    // training samples
    const uint64_t S = std::min<uint64_t>(n, 1u << 20);
    float *xs = nullptr, *ys = nullptr;
    GJ_TRY(sc.alloc(S, &xs));
    GJ_TRY(sc.alloc(S, &ys));
    k_make_samples<<<grid_for_n(S), 256, 0, s>>>(idx->d_col, n, S, v.min_key, v.inv_range, v.max_key, p.seed, xs, ys);
    GJ_CUDA_TRY(cudaGetLastError());

    if (p.learned_root == GJ_LEARNED_ROOT_LINEAR) {
        const int nb = 256;
        double* part = nullptr;
        GJ_TRY(sc.alloc(nb * 4, &part));
        k_linear_sums<<<nb, kTrainBlock, 0, s>>>(xs, ys, S, part);
        std::vector<double> h(nb * 4);
        GJ_CUDA_TRY(cudaMemcpyAsync(h.data(), part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
        GJ_CUDA_TRY(cudaStreamSynchronize(s));
        double sx = 0, sy = 0, sxx = 0, sxy = 0;
        for (int b = 0; b < nb; ++b) {
            sx += h[b * 4 + 0];
            sy += h[b * 4 + 1];
            sxx += h[b * 4 + 2];
            sxy += h[b * 4 + 3];
        }
        const double N = (double)S;
        const double den = N * sxx - sx * sx;
        const double a = den != 0.0 ? (N * sxy - sx * sy) / den : 0.0;
        const double b = (sy - a * sx) / N;
        idx->ln_root.w[0] = (float)a;
        idx->ln_root.w[1] = (float)b;
    } else if (!segments) {
        // start from the piecewise-linear CDF through H + 1 sample quantiles
        std::vector<float> hx(S), hy(S);
        GJ_CUDA_TRY(cudaMemcpyAsync(hx.data(), xs, S * sizeof(float), cudaMemcpyDeviceToHost, s));
        GJ_CUDA_TRY(cudaMemcpyAsync(hy.data(), ys, S * sizeof(float), cudaMemcpyDeviceToHost, s));
        GJ_CUDA_TRY(cudaStreamSynchronize(s));
        std::vector<float> q(H + 1), qy(H + 1);
        for (uint32_t j = 0; j < H; ++j) {
            const uint64_t at = (uint64_t)j * S / H;
            q[j] = hx[at];
            qy[j] = hy[at];
        }
        q[H] = 1.f;
        qy[H] = 1.f;
        std::vector<float> P0;
        init_mlp_quantiles(P0, H, q, qy);
        float* d_train = nullptr;  // trained parameters (H wide)
        GJ_TRY(sc.alloc(np, &d_train));
        GJ_CUDA_TRY(cudaMemcpyAsync(d_train, P0.data(), np * sizeof(float), cudaMemcpyHostToDevice, s));
        const uint32_t B = std::max<uint32_t>(kTrainBlock, std::min<uint32_t>(p.learned_batch, 1u << 16));
        const int nblocks = (int)((B + kTrainBlock - 1) / kTrainBlock);
        float *partial = nullptr, *grad = nullptr, *m1 = nullptr, *m2 = nullptr;
        uint32_t* bidx = nullptr;
        GJ_TRY(sc.alloc((size_t)nblocks * np, &partial));
        GJ_TRY(sc.alloc(np, &grad));
        GJ_TRY(sc.alloc(np, &m1));
        GJ_TRY(sc.alloc(np, &m2));
        GJ_TRY(sc.alloc(B, &bidx));
        GJ_CUDA_TRY(cudaMemsetAsync(m1, 0, np * sizeof(float), s));
        GJ_CUDA_TRY(cudaMemsetAsync(m2, 0, np * sizeof(float), s));
        const size_t smem = (((np + 3) & ~3u) + 3 * kTrainBlock * H + 2 * kTrainBlock) * sizeof(float);
        GJ_CUDA_TRY(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        const float b1 = 0.9f, b2 = 0.999f;
        float c1 = 1.f, c2 = 1.f;
        const uint32_t T = p.learned_steps;  // 0: the quantile start, untrained
        for (uint32_t t = 0; t < T; ++t) {
            c1 *= b1;
            c2 *= b2;
            // cosine-decayed learning rate
            const float lr = p.learned_lr * 0.5f * (1.f + std::cos(3.14159265f * (float)t / (float)T));
            k_batch_indices<<<(B + 255) / 256, 256, 0, s>>>(bidx, B, S, p.seed ^ 0xb47c4ull, t);
            k_mlp_grad<<<nblocks, kTrainBlock, smem, s>>>(d_train, (int)H, xs, ys, B, bidx, 1.0f / (float)B, partial,
                                                          nullptr);
            k_reduce_partials<<<(np + 255) / 256, 256, 0, s>>>(partial, (int)np, nblocks, grad, nullptr, nullptr);
            k_adam<<<(np + 255) / 256, 256, 0, s>>>(d_train, grad, m1, m2, (int)np, lr, b1, b2, 1e-8f, 1.f - c1,
                                                    1.f - c2);
        }
        GJ_CUDA_TRY(cudaGetLastError());
        // keep the trained network unless it fits the samples worse than its start
        std::vector<float> P1(np);
        GJ_CUDA_TRY(cudaMemcpyAsync(P1.data(), d_train, np * sizeof(float), cudaMemcpyDeviceToHost, s));
        double* d_loss = nullptr;
        GJ_TRY(sc.alloc(2, &d_loss));
        GJ_TRY(mlp_grad(d_train, H, xs, ys, S, grad, d_loss, s));
        GJ_CUDA_TRY(cudaMemcpyAsync(d_train, P0.data(), np * sizeof(float), cudaMemcpyHostToDevice, s));
        GJ_TRY(mlp_grad(d_train, H, xs, ys, S, grad, d_loss + 1, s));
        double losses[2] = {0, 0};
        GJ_CUDA_TRY(cudaMemcpyAsync(losses, d_loss, sizeof(losses), cudaMemcpyDeviceToHost, s));
        GJ_CUDA_TRY(cudaStreamSynchronize(s));
        const std::vector<float>& best = losses[0] <= losses[1] ? P1 : P0;
        idx->learned_trained_loss = losses[0];
        idx->learned_init_loss = losses[1];
        // store zero-padded to the 32-wide layout of the lookup
        constexpr uint32_t W = kMlpWidth;
        float* out = idx->ln_root.w;
        for (uint32_t j = 0; j < H; ++j) {
            out[j] = best[j];              // W1
            out[W + j] = best[H + j];      // b1
            for (uint32_t i = 0; i < H; ++i) out[2 * W + j * W + i] = best[2 * H + j * H + i];  // W2 row j
            out[2 * W + W * W + j] = best[2 * H + H * H + j];                                  // b2
            out[3 * W + W * W + j] = best[3 * H + H * H + j];                                  // W3
        }
        out[4 * W + W * W] = best[4 * H + H * H];  // b3
    }
    if (!segments) GJ_CUDA_TRY(cudaMemcpyAsync(d_root, idx->ln_root.w, nstored * sizeof(float), cudaMemcpyDefault, s));

    // route every key, fit the leaves, measure their error windows
    uint32_t* leaf_of = nullptr;
    unsigned int *first = nullptr, *last = nullptr, *count = nullptr;
    GJ_TRY(sc.alloc(n, &leaf_of));
    GJ_TRY(sc.alloc(L, &first));
    GJ_TRY(sc.alloc(L, &last));
    GJ_TRY(sc.alloc(L, &count));
    GJ_CUDA_TRY(cudaMemsetAsync(first, 0xFF, L * sizeof(unsigned int), s));
    GJ_CUDA_TRY(cudaMemsetAsync(last, 0, L * sizeof(unsigned int), s));
    GJ_CUDA_TRY(cudaMemsetAsync(count, 0, L * sizeof(unsigned int), s));
    // k_route stages the by-value parameters (none for the segment table)
    const size_t route_smem = (p.learned_root == GJ_LEARNED_ROOT_MLP ? kMlpParams : 2) * sizeof(float);
    k_route<<<grid_for_n(n), 256, route_smem, s>>>(v, v.root, leaf_of, first, last, count);
    k_leaf_params<<<(L + 255) / 256, 256, 0, s>>>(idx->d_col, L, first, last, count,
                                                 const_cast<learned_leaf*>(v.leaves));
    k_leaf_error<<<grid_for_n(n), 256, 0, s>>>(v, leaf_of, const_cast<learned_leaf*>(v.leaves));
    GJ_CUDA_TRY(cudaGetLastError());

    // statistics: largest window and key-weighted mean window
    std::vector<learned_leaf> hl(L);
    std::vector<unsigned int> hc(L);
    GJ_CUDA_TRY(cudaMemcpyAsync(hl.data(), v.leaves, L * sizeof(learned_leaf), cudaMemcpyDefault, s));
    GJ_CUDA_TRY(cudaMemcpyAsync(hc.data(), count, L * sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    GJ_CUDA_TRY(cudaStreamSynchronize(s));
    uint64_t max_err = 0;
    double weighted = 0;
    for (uint32_t l = 0; l < L; ++l) {
        if (!hc[l]) continue;
        const uint64_t w = (uint64_t)hl[l].err_lo + hl[l].err_hi + 1;
        max_err = std::max<uint64_t>(max_err, (uint64_t)std::max(hl[l].err_lo, hl[l].err_hi));
        weighted += (double)w * hc[l];
    }
    idx->learned_max_error = max_err;
    idx->learned_mean_window = weighted / (double)n;
    return GJ_OK;
}

}  // namespace gj

using namespace gj;

extern "C" int gj_learned_mlp_grad(const float* d_params, uint32_t hidden, const float* d_x, const float* d_y,
                                   uint64_t count, float* d_grad, double* d_loss, void* stream) {
    GJ_CHECK_ARG(d_params && d_grad && d_loss, "gj_learned_mlp_grad: null argument");
    GJ_CHECK_ARG(count == 0 || (d_x && d_y), "gj_learned_mlp_grad: null samples");
    return mlp_grad(d_params, hidden, d_x, d_y, count, d_grad, d_loss, as_stream(stream));
}
