/*
 * Host stand-ins for the CUDA warp intrinsics named by the reference's
 * search/btree/harmonia headers, so that those headers compile as plain
 * C++ for the CPU checker in oracle/_ref.  Only the single-thread lookups
 * (btree::lookup, harmonia_tree::lookup, lower_bound, branch-free search)
 * are executed on the host; the warp-cooperative paths are only parsed.
 */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
static inline int __clz(unsigned x) { return x ? __builtin_clz(x) : 32; }
static inline int __clzll(unsigned long long x) { return x ? __builtin_clzll(x) : 64; }
static inline int __ffs(unsigned x) { return __builtin_ffs((int)x); }
static inline int __popc(unsigned x) { return __builtin_popcount(x); }
template <class T> static inline T __shfl_sync(unsigned, T v, int, int = 32) { return v; }
static inline unsigned __ballot_sync(unsigned, int p) { return p ? 1u : 0u; }
static inline void __syncwarp(unsigned = 0xffffffffu) {}
static inline unsigned __activemask() { return 0xffffffffu; }
static inline unsigned __funnelshift_l(unsigned lo, unsigned hi, unsigned s) {
    s &= 31u;
    return s ? (hi << s) | (lo >> (32u - s)) : hi;
}
using std::max;
using std::min;
