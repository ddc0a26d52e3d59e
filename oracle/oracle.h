/*
 * oracle.h -- CPU restatement of the gpujoin INLJ probe path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * product in gpujoin_gb300/: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load it.  Nothing in the product
 * links, calls or falls back to it.
 *
 * Every function restates one piece of the reference (josefschmeisser/gpujoin)
 * and cites the file:line it follows.  Positions are uint32; a probe without
 * a result yields ORC_INV (= numeric_limits<uint32_t>::max(), the reference's
 * invalid_tid narrowed to the 32-bit tid_t of src/tpch/tpch_14_common.cuh:18).
 */
#ifndef GJ_ORACLE_H
#define GJ_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_INV 0xFFFFFFFFu

/* ---- search primitives (src/search.cuh) -------------------------------- */
/* count/step lower bound, src/search.cuh:26-41 */
uint64_t orc_lower_bound(const uint64_t* arr, uint64_t n, uint64_t key);
/* power-of-two branch-free lower bound, src/search.cuh:143-158 (n >= 2) */
uint64_t orc_branch_free_lower_bound(const uint64_t* arr, uint64_t n, uint64_t key);
/* equality-or-lower-bound binary search, src/search.cuh:86-101 */
uint64_t orc_branchy_binary_search(const uint64_t* arr, uint64_t n, uint64_t key);

/* ---- index semantics ---------------------------------------------------- */
/* binary_search_index::cooperative_lookup, src/indexes.cuh:357-361:
 * pos = lower_bound; pos < n ? pos : INV (no equality check). */
void orc_bs_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes,
                   uint64_t m, uint32_t* out, int threads);
/* same through the branch-free search (src/search.cuh:143-158) */
void orc_bs_branch_free_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes,
                               uint64_t m, uint32_t* out, int threads);

/* Clustered B+tree (src/btree.cuh): leaves are slices of the sorted column
 * with at most leaf_keys keys (:50-55, :242-246); inner nodes hold at most
 * inner_keys separators, separator = max key of the child (:176-206);
 * lookup = branchy_binary_search per level, exact match on the leaf slice
 * (:504-531).  The reference uses leaf_keys=247, inner_keys=246 for u64. */
typedef struct orc_btree orc_btree;
orc_btree* orc_btree_build(const uint64_t* col, uint64_t n, uint32_t leaf_keys,
                           uint32_t inner_keys);
void orc_btree_lookup(const orc_btree* t, const uint64_t* probes, uint64_t m,
                      uint32_t* out, int threads);
/* lower bound (INV at n) through the same tree: orc_bs_lookup's results, faster */
void orc_btree_lower_bound(const orc_btree* t, const uint64_t* probes, uint64_t m, uint32_t* out, int threads);
uint32_t orc_btree_depth(const orc_btree* t);
void orc_btree_free(orc_btree* t);
/* The tree as the reference lays it out in device memory (src/btree.cuh:30-64,
 * migrate :440-476): one page_bytes page per inner node, at page
 * pages_base + page_bytes * node; header {u16 count, bool isLeaf = 0, bool
 * isFinalInner} at offset 0; count separators at keys_off (UINT64_MAX after
 * them); count + 1 child pointers at children_off -- pages of the inner
 * nodes below, or for a final inner node pointers into the column at
 * col_base.  out holds orc_btree_nodes() * page_bytes bytes; returns the
 * root's node number, or -1 if the offsets do not fit the page. */
uint64_t orc_btree_nodes(const orc_btree* t);
int64_t orc_btree_write_pages(const orc_btree* t, uint8_t* out, uint64_t page_bytes, uint64_t keys_off,
                              uint64_t children_off, uint64_t pages_base, uint64_t col_base);

/* Harmonia (src/harmonia.cuh:133-404 construction, :640-668 host lookup),
 * Reuse_Input_Memory: the leaf level is the column itself; n % max_keys == 0. */
typedef struct orc_harmonia orc_harmonia;
/* returns NULL and sets *err (1 = n not a multiple of max_keys, 2 = too deep,
 * 3 = separator overflow) on failure */
orc_harmonia* orc_harmonia_build(const uint64_t* col, uint64_t n, uint32_t max_keys, int* err);
uint64_t orc_harmonia_lookup_one(const orc_harmonia* h, uint64_t key); /* UINT64_MAX = not found */
void orc_harmonia_lookup(const orc_harmonia* h, const uint64_t* probes, uint64_t m,
                         uint32_t* out, int threads);
/* expose the built arrays (inner key array, children prefix array, depth) */
void orc_harmonia_arrays(const orc_harmonia* h, const uint64_t** keys, uint64_t* nkeys,
                         const uint64_t** children, uint64_t* nchildren, uint32_t* depth);
void orc_harmonia_free(orc_harmonia* h);

/* RadixSpline.  Builder: GreedySplineCorridor + radix table, restated from the
 * published algorithm (Kipf et al., aiDM 2020; learnedsystems/RadixSpline,
 * unpinned in lib/RadixSpline.cmake:8-15).  Lookup: src/rs.cuh:118-154 and
 * src/indexes.cuh:205-215, plus a window check that falls back to a full
 * lower bound so the result is always the exact lower bound. */
typedef struct orc_rs orc_rs;
orc_rs* orc_rs_build(const uint64_t* col, uint64_t n, uint32_t radix_bits, uint32_t max_error);
void orc_rs_lookup(const orc_rs* r, const uint64_t* col, const uint64_t* probes, uint64_t m,
                   uint32_t* out, int threads);
double orc_rs_estimate(const orc_rs* r, uint64_t key);
void orc_rs_arrays(const orc_rs* r, const uint32_t** radix_table, uint64_t* table_len,
                   const uint64_t** spline_x, const double** spline_y, uint64_t* npoints,
                   uint32_t* shift_bits);
void orc_rs_free(orc_rs* r);

/* exact-match lookup: pos if col[pos]==key else INV (the semantics the
 * B+tree and Harmonia lookups reduce to for unique sorted build keys) */
void orc_exact_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes,
                      uint64_t m, uint32_t* out, int threads);

/* ---- partitioning (src/index_lookup_partitioning.cu:300-375) ------------- */
/* Stable range partition of (key, row) on ((key - min_key) >> shift), clamped
 * to fanout-1.  offsets has fanout+1 entries (start of each partition). */
void orc_range_partition(const uint64_t* keys, uint64_t m, uint64_t min_key, uint32_t shift,
                         uint32_t radix_bits, uint64_t* out_keys, uint32_t* out_rows,
                         uint64_t* offsets);

/* ---- join materialisation (src/tpch/tpch_14_ij.cu:371-407) -------------- */
/* (probe row, build pos) for every probe with pos != INV, in probe order. */
uint64_t orc_pairs_from_positions(const uint32_t* pos, uint64_t m, uint32_t* out_rows,
                                  uint32_t* out_pos);

/* ---- star-join aggregate (src/tpch/cpu_only.cpp:230-275) ----------------- */
/* out[0] = sum over flagged dim rows ("numerator"), out[1] = sum over all
 * ("denominator"); summand = price * (100 - discount); date filter
 * lo <= date < hi; the dimension lookup is an exact match on dim_keys. */
void orc_star_join(const uint32_t* fk, const uint32_t* date, const int64_t* price,
                   const int64_t* disc, uint64_t nfact, const uint64_t* dim_keys,
                   const uint8_t* dim_flag, uint64_t ndim, uint32_t lo, uint32_t hi,
                   int64_t out[2]);

/* ---- generators (src/zipf.hpp, src/index_lookup_common.cuh:51-206) -------- */
uint64_t orc_mix64(uint64_t x);
/* Zipf rank in [1, n] by rejection-inversion (Hoermann & Derflinger 1996),
 * the method of src/zipf.hpp:13-102, driven by a counter-based stream. */
uint64_t orc_zipf_rank(uint64_t n, double q, uint64_t seed, uint64_t index);
/* bijective seeded permutation of [0, n) (Feistel + cycle walking) */
uint64_t orc_permute(uint64_t x, uint64_t n, uint64_t seed);
/* m probes = col[permute(zipf_rank(n, q) - 1)] (q = 0: uniform), threaded */
void orc_zipf_probes(const uint64_t* col, uint64_t n, uint64_t* out, uint64_t m, double q, uint64_t seed,
                     int threads);

/* ---- learned position model (CPU restatement of the training math) ------- */
/* Root MLP 1 -> H -> H -> 1 (ReLU), parameters packed as
 * [W1(H), b1(H), W2(H*H, row-major out x in), b2(H), W3(H), b3(1)].
 * Forward on normalised inputs x, mean-squared-error loss against targets y,
 * gradient accumulated (summed, not averaged) into grad; returns the loss sum. */
double orc_mlp_loss_grad(const float* params, int hidden, const float* x, const float* y,
                         uint64_t count, double* grad);
float orc_mlp_forward(const float* params, int hidden, float x);

/* ---- threading helper for the CPU baselines ------------------------------ */
int orc_hardware_threads(void);

#ifdef __cplusplus
}
#endif
#endif
