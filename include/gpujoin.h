/*
 * gpujoin.h -- C ABI of the GB300 index-nested-loop-join (INLJ) probe engine.
 *
 * Plain C: pointers, sizes and status codes only.  Device pointers are
 * marked d_*, host pointers h_*; a stream is passed as void* (a cudaStream_t,
 * NULL = the legacy default stream).  Every call returns GJ_OK (0) or a
 * GJ_ERR_* code; gj_last_error_string() describes the last failure of the
 * calling thread.  Calls are asynchronous on the given stream unless noted.
 *
 * Ownership: the caller owns every input, output and workspace buffer; the
 * library owns the memory of a gj_index (its search structure) and frees it
 * in gj_index_free().  An index borrows the caller's device column (d_keys),
 * which must stay alive and unchanged for the lifetime of the index
 * (binary_search_index / radix_spline_index borrow it the same way,
 * src/indexes.cuh:223,365).
 *
 * Each entry point names the reference interface it replaces (file:line in
 * josefschmeisser/gpujoin).
 */
#ifndef GPUJOIN_H
#define GPUJOIN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GJ_ABI_VERSION 1u

/* status codes */
#define GJ_OK 0
#define GJ_ERR_INVALID_ARGUMENT 1   /* null pointer, bad size, bad enum */
#define GJ_ERR_CUDA 2               /* a CUDA runtime call failed */
#define GJ_ERR_UNSUPPORTED 3        /* valid request this build cannot serve */
#define GJ_ERR_OUT_OF_MEMORY 4      /* device or host allocation failed */
#define GJ_ERR_TIMEOUT 5            /* a bounded device wait gave up */
#define GJ_ERR_UNSORTED 6           /* build keys not strictly increasing */
#define GJ_ERR_WORKSPACE 7          /* workspace missing or too small */
#define GJ_ERR_TOO_LARGE 8          /* size exceeds a documented limit */

/* not-found marker of every position output:
 * numeric_limits<value_t>::max() (src/indexes.cuh:101,184,262,344) with the
 * 32-bit tid_t of src/tpch/tpch_14_common.cuh:18 */
#define GJ_INVALID_POS 0xFFFFFFFFu

/* index kinds; the first five keep the order of index_type_enum
 * (src/indexes.hpp:5) */
typedef enum gj_index_type {
    GJ_INDEX_BTREE = 0,
    GJ_INDEX_HARMONIA = 1,
    GJ_INDEX_BINARY_SEARCH = 2,
    GJ_INDEX_RADIX_SPLINE = 3,
    GJ_INDEX_NO_OP = 4,
    GJ_INDEX_LEARNED = 5, /* not in the reference: trained position model */
    GJ_INDEX_HASH = 6     /* the reference's hash-join table (src/linear_probing_hashtable.cuh) as an index:
                             position of the equal key, else GJ_INVALID_POS */
} gj_index_type;

/* learned root models */
/* gj_index_params.index_memory.  The reference keeps its index in host
 * memory read over NVLink 2.0 (src/index_lookup_config.hpp:52-66); on GB300
 * that is pinned Grace memory read over NVLink-C2C. */
#define GJ_INDEX_MEMORY_DEVICE 0u
#define GJ_INDEX_MEMORY_HOST 1u

#define GJ_LEARNED_ROOT_LINEAR 0u
#define GJ_LEARNED_ROOT_MLP 1u
#define GJ_LEARNED_ROOT_AUTO 2u /* a linear root, a segment table, a 16-wide and a 32-wide MLP are built, in
                                   that order of lookup cost; the cheapest whose mean search window is at
                                   most twice the narrowest (+16 keys) is kept */
#define GJ_LEARNED_ROOT_SEGMENTS 3u /* piecewise-linear CDF over 4096 equal-width key segments, exact at the
                                       segment ends: one table load and one FMA per lookup */

/* Build parameters.  Call gj_index_params_default() first, then override.
 * Replaces the compile-time IndexConfiguration / constants of the reference
 * (src/indexes.cuh:88-91,169-174,329-334; src/index_lookup_config.hpp:18-37). */
typedef struct gj_index_params {
    uint32_t struct_size;       /* = sizeof(gj_index_params) */
    uint32_t btree_node_keys;   /* separators per B+tree inner node (fanout - 1): 4, 8, 16, 32 or 64 uint64
                                   separators, or a compressed node of one 32-byte sector holding its
                                   separators as deltas from a base the search carries: 7 (32-bit deltas,
                                   fanout 8) or 15 (default; 14-bit deltas, fanout 16) */
    uint32_t btree_leaf_keys;   /* keys per B+tree leaf (column slice), a power of two <= 4096 (default 4:
                                   one 32-byte sector) */
    uint32_t rs_radix_bits;     /* RadixSpline radix table bits (default 18) */
    uint32_t rs_max_error;      /* RadixSpline spline error (default 32) */
    uint32_t bs_cache_keys;     /* binary search: sampled keys staged in shared memory (default 4096, 0 = off) */
    uint32_t smem_cache_bytes;  /* B+tree / Harmonia: upper levels staged in shared memory (default 16384) */
    uint32_t learned_leaves;    /* learned index: linear leaf models (default 0: about 128 keys per leaf, a
                                   power of two in [2^10, 2^20]) */
    uint32_t learned_root;      /* GJ_LEARNED_ROOT_LINEAR, _MLP, _SEGMENTS or _AUTO (default AUTO) */
    uint32_t learned_hidden;    /* MLP hidden width (default 32, max 32) */
    uint32_t learned_steps;     /* root training steps (default 600; 0 keeps the MLP's quantile start) */
    uint32_t learned_batch;     /* root training batch (default 8192) */
    float learned_lr;           /* root learning rate (Adam, default 1e-3) */
    uint32_t index_memory;      /* where the index's own arrays live: GJ_INDEX_MEMORY_DEVICE (HBM, default)
                                   or GJ_INDEX_MEMORY_HOST (pinned Grace memory, read by the kernels over
                                   NVLink-C2C; pair it with a column in pinned host memory) */
    uint32_t btree_start_bits;  /* B+tree and Harmonia start table: the key range cut into 2^bits buckets, each
                                   mapped to the deepest node its keys share, where lookups start (default 0:
                                   about one bucket per 64 keys, at most 2^20; 1..24 as given) */
    uint64_t seed;              /* training / sampling seed */
} gj_index_params;

typedef struct gj_index gj_index; /* opaque */

/* ---- library ------------------------------------------------------------ */
uint32_t gj_abi_version(void);
const char* gj_last_error_string(void);
void gj_index_params_default(gj_index_params* params);

/* parse_index_type (src/indexes.cpp:5-19): "btree", "harmonia",
 * "binary_search", "radix_spline", "no_op" (+ "learned").  Unknown names
 * return GJ_ERR_INVALID_ARGUMENT ("unknown index type", as the reference). */
int gj_parse_index_type(const char* name, int* out_type);
/* type_name<...>::value() (src/indexes.cuh:149-154 etc.) */
const char* gj_index_type_name(int type);

/* ---- index build / lookup ------------------------------------------------ */
/* abstract_index::construct (src/indexes.cuh:36) + the per-index construct()
 * overrides (:126,218,285,364).  d_keys: n strictly increasing uint64 keys
 * on the device.  h_keys may be NULL (the builder copies what it needs).
 * Errors: n == 0 or n >= 2^32-1 (GJ_ERR_TOO_LARGE, the reference's
 * "'value_t' does not suffice"), Harmonia with n % 32 != 0
 * (GJ_ERR_INVALID_ARGUMENT, src/harmonia.cuh:350-352), unsorted keys
 * (GJ_ERR_UNSORTED).  Synchronous: returns when the index is usable. */
int gj_index_build(int type, const uint64_t* d_keys, const uint64_t* h_keys, uint64_t n,
                   const gj_index_params* params, void* stream, gj_index** out_index);
int gj_index_free(gj_index* index);
/* abstract_index::memory_consumption (src/indexes.cuh:38) in bytes */
uint64_t gj_index_memory_consumption(const gj_index* index);
/* bytes of the index's own arrays that live in pinned host memory
 * (index_memory = GJ_INDEX_MEMORY_HOST); 0 for an index in HBM */
uint64_t gj_index_host_memory(const gj_index* index);
int gj_index_get_type(const gj_index* index, int* out_type);
uint64_t gj_index_size(const gj_index* index);
/* learned index: recorded maximum prediction error (positions) and mean
 * search-window width over the build keys */
int gj_index_learned_stats(const gj_index* index, uint64_t* max_error, double* mean_window);
/* the root model a learned index was built with (GJ_LEARNED_ROOT_LINEAR,
 * _MLP or _SEGMENTS; the one kept when the build asked for GJ_LEARNED_ROOT_AUTO) */
int gj_index_learned_root(const gj_index* index, uint32_t* root);
/* learned index with an MLP root: the mean squared error of the root on its
 * training sample (positions scaled to [0, 1]) at the quantile start and
 * after training; the build keeps the network with the smaller one
 * (learned_steps = 0 keeps the start untrained).  No counterpart in the
 * reference. */
int gj_index_learned_losses(const gj_index* index, double* init_loss, double* trained_loss);

/* The index's device view -- the struct passed by value to kernels, like
 * the reference's device_index_t member (src/indexes.cuh:18-22,116-124) --
 * for kernels written against include/gpujoin/device.cuh.  view_bytes must
 * equal the size of the view of the index kind (gj::bs_view, btree_view,
 * harmonia_view, rs_view, learned_view; 0 for no_op).  The view does not
 * use the shared-memory caches of the library's own kernels.  Valid while
 * the index lives. */
int gj_index_device_view(const gj_index* index, void* view, size_t view_bytes);

/* Plain INLJ probe, lookup_kernel (src/index_lookup_common.cuh:217-245):
 * d_positions[i] = device_index_t::cooperative_lookup(d_probes[i]) with the
 * reference's per-index result semantics:
 *   binary_search, radix_spline, learned: lower bound, GJ_INVALID_POS at n
 *     (src/indexes.cuh:357-361, :205-215);
 *   btree, harmonia: position of an equal key, else GJ_INVALID_POS
 *     (src/btree.cuh:504-531, src/harmonia.cuh:740-786);
 *   no_op: GJ_INVALID_POS (src/indexes.cuh:384-406). */
int gj_index_lookup(const gj_index* index, const uint64_t* d_probes, uint64_t m,
                    uint32_t* d_positions, void* stream);

/* ---- join materialisation ------------------------------------------------ */
/* ij_lookup_kernel (src/tpch/tpch_14_ij.cu:371-407): probe and emit one
 * (probe row, build position) pair -- two uint32 at d_pairs[2k], [2k+1] --
 * per probe with a result, in probe order (deterministic; the reference's
 * order follows its atomics).  *d_count (device) receives the pair count.
 * d_pairs must hold 2*m uint32.  Workspace: gj_inlj_pairs_workspace_size. */
int gj_inlj_pairs_workspace_size(uint64_t m, size_t* bytes);
int gj_inlj_pairs(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                  uint64_t* d_count, void* d_workspace, size_t workspace_bytes, void* stream);
/* gj_inlj_pairs in one pass with each tile's pairs placed by one atomicAdd
 * in the order tiles finish (as the reference's join kernels place theirs,
 * src/tpch/tpch_14_ij.cu:371-407): the same set of pairs and count, no
 * ordered compaction.  Same arguments and workspace; d_pairs holds 2*m
 * uint32 and nothing is parked in it. */
int gj_inlj_pairs_unordered(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                            uint64_t* d_count, void* d_workspace, size_t workspace_bytes, void* stream);

/* ---- warp-collective searches ---------------------------------------------- */
/* gj_index_lookup with the reference's warp-collective search protocol:
 * groups of 2^degree lanes (degree 1..5) serve their members' probes one
 * after another, one round of loads per step -- cooperative_binary_search
 * (src/search.cuh:355-386) for a binary-search index, harmonia_tree::
 * lookup<Degree> (src/harmonia.cuh:740-786) for a Harmonia index.  Results
 * equal gj_index_lookup's; other index kinds return GJ_ERR_UNSUPPORTED.
 * The per-thread gj_index_lookup is the faster form for independent probes
 * (a warp keeps 32 searches in flight instead of 32 / 2^degree). */
int gj_index_lookup_cooperative(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_positions,
                                uint32_t degree, void* stream);

/* ---- block-wise sorted probe order ---------------------------------------- */
/* bws_lookup (src/index_lookup_common.cuh:398-549): each tile of 1024 probes
 * is sorted by key in shared memory and searched in that order, so lanes of
 * a warp share index paths (skewed probes repeat keys).
 * gj_index_lookup_sorted: the positions of gj_index_lookup, in probe order.
 * gj_inlj_pairs_sorted: the pairs of gj_inlj_pairs, tile by tile in probe
 * order, inside a tile in key order (the same set).  Same workspace. */
int gj_index_lookup_sorted(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_positions,
                           void* stream);
int gj_inlj_pairs_sorted(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                         uint64_t* d_count, void* d_workspace, size_t workspace_bytes, void* stream);
#define GJ_ORDER_PROBE 0u        /* gj_inlj_pairs */
#define GJ_ORDER_SORTED_TILES 1u /* gj_inlj_pairs_sorted */
#define GJ_ORDER_PARTITIONED 2u  /* gj_partitioned_inlj, one window, default fanout */
/* the fastest probe order for these probes (pairs), timed on the caller's
 * data: probe order, sorted tiles, or range-partitioned (the pairs of
 * gj_partitioned_inlj: the same set, grouped by partition tile; timed as the
 * index stands, so an index not prepared with gj_index_prepare_partitioned
 * pays for building the directory each call).  Allocates the workspaces it
 * times with. */
int gj_autotune_ordering(const gj_index* index, const uint64_t* d_probes, uint64_t m, void* stream,
                         uint32_t* ordering, float* best_ms);

/* gj_inlj_pairs with the probes, the pairs and the count in HOST memory
 * (the reference's driver starts from host columns, src/index_lookup_new.cu:
 * 375-434).  No copies are issued: one kernel reads each tile's probes over
 * the host link (NVLink-C2C on GB300), searches them and writes the tile's
 * pairs (and finally *h_count) back, so transfers of some tiles overlap the
 * searches of others.  The host buffers must be reachable from the GPU:
 * pinned or registered
 * (cudaHostAlloc / cudaHostRegister), managed, or pageable on systems whose
 * GPU uses the CPU's page tables; otherwise GJ_ERR_INVALID_ARGUMENT.
 * h_pairs holds 2*m uint32; results are valid once the stream has passed
 * the call (m = 0 waits for the stream and writes *h_count = 0 on the host).
 * Workspace (device): gj_inlj_pairs_host_workspace_size; gj_inlj_pairs_status
 * reports a timed-out wait as for gj_inlj_pairs. */
int gj_inlj_pairs_host_workspace_size(uint64_t m, size_t* bytes);
int gj_inlj_pairs_host(const gj_index* index, const uint64_t* h_probes, uint64_t m, uint32_t* h_pairs,
                       uint64_t* h_count, void* d_workspace, size_t workspace_bytes, void* stream);
/* gj_inlj_pairs_host with the pairs in the order their tiles finish (one
 * atomicAdd per tile, as the reference's join kernels place theirs,
 * src/tpch/tpch_14_ij.cu:371-407) instead of in probe order: the same set
 * of pairs and the same count, with no tile waiting for its predecessors
 * (19 % faster on GB300 for 2^28 probes: the link, not the ordering, is the
 * limit).  Same arguments and workspace; nothing waits, so
 * gj_inlj_pairs_status has nothing to report. */
int gj_inlj_pairs_host_unordered(const gj_index* index, const uint64_t* h_probes, uint64_t m, uint32_t* h_pairs,
                                 uint64_t* h_count, void* d_workspace, size_t workspace_bytes, void* stream);

/* Outcome of the last gj_inlj_pairs run on this workspace with this m:
 * waits on the stream, then returns GJ_OK or
 * GJ_ERR_TIMEOUT when a bounded device wait of the ordered compaction gave up
 * (the pairs and *d_count are then incomplete).  No counterpart in the
 * reference, whose compaction does not wait. */
int gj_inlj_pairs_status(const void* d_workspace, size_t workspace_bytes, uint64_t m, void* stream);

/* Test hook of the bounded waits, with no counterpart in the reference: runs
 * gj_inlj_pairs with the first tile left unclaimed and a look-back limit of
 * spin_limit polls, so every later tile's wait runs out and the kernel
 * returns with the error word set (gj_inlj_pairs_status then returns
 * GJ_ERR_TIMEOUT; *d_count is not written).  Nothing faults or hangs: the
 * waits are bounded and every block exits. */
int gj_debug_inlj_pairs_stalled(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                                uint64_t* d_count, void* d_workspace, size_t workspace_bytes,
                                uint32_t spin_limit, void* stream);

/* Same pairs as gj_inlj_pairs, for callers that cannot allocate device
 * memory when they probe (a frozen allocator, someone else's memory arena,
 * or a probe path that must not call cudaMalloc/cudaFree because they
 * synchronise the device).  No counterpart in the reference.  Its scratch is a
 * fixed array inside the library (about 2 MiB on every GPU that loads the
 * library, held until the process exits), so it needs no workspace argument
 * and allocates nothing.  At most GJ_NOALLOC_MAX_PROBES probes per call;
 * larger m returns GJ_ERR_TOO_LARGE.  The first call on a device looks up the
 * array's device address; under lazy module loading that lookup may also
 * load the library's device code and back the array, i.e. allocate and
 * synchronise once.  So warm it up at start-up: make one call per device
 * (m = 0 is enough) before the probe path runs and before capturing a
 * stream.  The address is kept per device ordinal and is valid in the
 * device's primary context only (the runtime API's default).  All calls
 * share the array: calls whose kernels overlap on the GPU (other streams,
 * other host threads) must be serialised by the caller.
 * A bounded device wait that gives up is NOT reported on this path: the
 * error word lives in the library's array, which gj_inlj_pairs_status
 * cannot see, and the next call clears it.  The wait only gives up when a
 * predecessor tile makes no progress for about 2^22 polls (seconds), which
 * the kernel's in-order tile claims rule out short of a GPU preemption of
 * that length; a caller that must detect it uses gj_inlj_pairs with its own
 * workspace and gj_inlj_pairs_status. */
#define GJ_NOALLOC_MAX_PROBES (1ull << 28)
int gj_inlj_pairs_noalloc(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint32_t* d_pairs,
                          uint64_t* d_count, void* stream);

/* ---- partitioned INLJ ---------------------------------------------------- */
/* Range partition of the probe side, replacing gpu_contiguous_prefix_sum_int64
 * + gpu_chunked_laswwc_radix_partition_int64_int64 as called from
 * run_on_stream (src/index_lookup_partitioning.cu:300-359).  Partition of a
 * key = min(((key - min_key) >> shift), 2^radix_bits - 1), keys <= min_key in
 * partition 0.  Partitions follow each other in key order; inside a
 * partition the tuples of earlier probe chunks come first, the order within
 * one chunk is not fixed.  d_out_keys / d_out_rows hold m entries, d_offsets
 * 2^radix_bits + 1.  radix_bits in [1, 12]. */
int gj_partition_workspace_size(uint64_t m, uint32_t radix_bits, size_t* bytes);
/* The key range an index was built over (its column's first and last key),
 * from which its partitions are cut; no counterpart in the reference, whose
 * partitioning uses fixed key bits (src/index_lookup_new.cu:63-67). */
int gj_index_key_range(const gj_index* index, uint64_t* min_key, uint64_t* max_key);
/* The shift of gj_range_partition that maps [min_key, max_key] onto
 * 2^radix_bits partitions (the smallest such shift). */
int gj_partition_shift(uint64_t min_key, uint64_t max_key, uint32_t radix_bits, uint32_t* shift);
int gj_range_partition(const uint64_t* d_keys, uint64_t m, uint64_t min_key, uint32_t shift,
                       uint32_t radix_bits, uint64_t* d_out_keys, uint32_t* d_out_rows,
                       uint64_t* d_offsets, void* d_workspace, size_t workspace_bytes, void* stream);
/* partitioned_lookup_kernel (src/index_lookup_partitioning.cu:218-248):
 * probe a partitioned relation and scatter d_positions[row] = result. */
int gj_partitioned_lookup(const gj_index* index, const uint64_t* d_part_keys, const uint32_t* d_part_rows,
                          uint64_t m, uint32_t* d_positions, void* stream);
/* The windowed partitioned INLJ (partitioning_approach::run,
 * src/index_lookup_partitioning.cu:436-507): the probe column is cut into
 * windows of window_size probes; each window is range-partitioned on the
 * index's key range and every partition is probed against its slice of the
 * index's column through a partition directory built once per call (each
 * index kind's result semantics kept).  Emits d_positions in probe order
 * (equal to gj_index_lookup) when d_positions != NULL, and/or the (row, pos)
 * pairs of the matches when d_pairs != NULL (*d_count = number of pairs);
 * the set of pairs is fixed, their order is not (tiles of a window append
 * in the order they finish, as the reference's atomics do,
 * src/tpch/tpch_14_ij.cu:371-407).  radix_bits = 0 picks the fanout from
 * the index size.  Workspace: gj_partitioned_inlj_workspace_size. */
int gj_partitioned_inlj_workspace_size(const gj_index* index, uint64_t window_size, uint32_t radix_bits,
                                       size_t* bytes);
/* Builds the index's partition directory (the radix table over its column
 * that gj_partitioned_inlj probes through, about 4 bytes per key) and keeps
 * it with the index, like the B+tree's start table; later partitioned calls
 * skip building it and need less workspace.  Synchronous; idempotent.  No
 * counterpart in the reference. */
int gj_index_prepare_partitioned(gj_index* index, void* stream);
int gj_partitioned_inlj(const gj_index* index, const uint64_t* d_probes, uint64_t m, uint64_t window_size,
                        uint32_t radix_bits, uint32_t* d_positions, uint32_t* d_pairs, uint64_t* d_count,
                        void* d_workspace, size_t workspace_bytes, void* stream);

/* ---- star-join aggregate -------------------------------------------------- */
/* ij_plain_kernel (src/tpch/tpch_14_ij.cu:34-85) with the semantics of
 * query_14_part_build (src/tpch/cpu_only.cpp:230-275): over fact rows with
 * lo <= date < hi whose foreign key is found in the dimension index,
 * summand = price * (100 - discount); d_out[1] += summand, and d_out[0] +=
 * summand when d_dim_flag[dim position] != 0.  d_out (2 x int64, device) is
 * overwritten.  dim_index must be an exact-match index (btree or harmonia). */
int gj_star_join_sum(const gj_index* dim_index, const uint32_t* d_fk, const uint32_t* d_date,
                     const int64_t* d_price, const int64_t* d_discount, uint64_t nfact,
                     const uint8_t* d_dim_flag, uint32_t lo, uint32_t hi, int64_t* d_out, void* stream);
/* The same sums in the reference's pipelined order, ij_pbws
 * (src/tpch/tpch_14_ij.cu:95-362): the rows that pass the date filter are
 * buffered per block across tiles, sorted by foreign key in batches of 2048
 * and probed in key order.  nfact < 2^32. */
int gj_star_join_sum_sorted(const gj_index* dim_index, const uint32_t* d_fk, const uint32_t* d_date,
                            const int64_t* d_price, const int64_t* d_discount, uint64_t nfact,
                            const uint8_t* d_dim_flag, uint32_t lo, uint32_t hi, int64_t* d_out, void* stream);

/* ---- TPC-H Q14 from dbgen .tbl files -------------------------------------- */
/* The columns of Q14 (load_tables_with_aria_parser, src/tpch/common.cpp:
 * 82-220), parsed on the host (all threads) into malloc'ed arrays:
 * lineitem l_partkey, l_shipdate (days since 1970-01-01), l_extendedprice
 * and l_discount (decimals x 100); part p_partkey (strictly increasing, as
 * dbgen writes them; else GJ_ERR_UNSORTED) and p_promo (p_type LIKE
 * 'PROMO%').  Malformed rows: GJ_ERR_INVALID_ARGUMENT naming the row.
 * Release with gj_tpch_free_q14. */
typedef struct gj_q14_tables {
    uint64_t n_lineitem, n_part;
    uint32_t* l_partkey;
    uint32_t* l_shipdate;
    int64_t* l_extendedprice;
    int64_t* l_discount;
    uint64_t* p_partkey;
    uint8_t* p_promo;
} gj_q14_tables;
int gj_tpch_load_q14(const char* lineitem_tbl, const char* part_tbl, gj_q14_tables* out);
void gj_tpch_free_q14(gj_q14_tables* tables);
/* the loader's day number of a date (days since 1970-01-01) */
int gj_tpch_day(int year, int month, int day, uint32_t* out_day);
/* Q14 (query_14_part_build, src/tpch/cpu_only.cpp:230-275) on the GPU: the
 * columns are copied to HBM, a B+tree is built over p_partkey and the star
 * join sums summand = price * (100 - discount) over lineitems shipped in
 * [1995-09-01, 1995-10-01) with a matching part: sums[0] over PROMO parts,
 * sums[1] over all; *promo_revenue = 100 * sums[0] / sums[1] (0 when
 * sums[1] is 0).  Synchronous on the stream. */
int gj_tpch_q14(const gj_q14_tables* tables, void* stream, int64_t sums[2], double* promo_revenue);

/* ---- learned position model ---------------------------------------------- */
/* The root MLP's backward pass as the learned index's trainer runs it:
 * d_grad (same layout as d_params: W1[H] b1[H] W2[HxH, out-major] b2[H]
 * W3[H] b3) receives the gradient of sum_s (mlp(x_s) - y_s)^2 over the
 * count samples, *d_loss (device) that sum.  hidden in [1, 32].  Allocates
 * its scratch internally; synchronous.  Exposed so that the gradient can be
 * checked against an independent implementation. */
int gj_learned_mlp_grad(const float* d_params, uint32_t hidden, const float* d_x, const float* d_y, uint64_t count,
                        float* d_grad, double* d_loss, void* stream);

/* ---- batched lookup stream ------------------------------------------------ */
/* Many probe batches against several indexes (not in the reference, whose
 * driver runs one index and one probe column per process,
 * src/index_lookup_new.cu:375-434).  Batch b probes
 * d_probes[probe_offset[b] .. +batch_size[b]) against indexes[batch_index[b]]
 * and writes d_positions at the same offsets, with the per-index result
 * semantics of gj_index_lookup.
 *
 * A plan uploads the batch descriptors once (device memory owned by the
 * plan; the indexes must outlive it).  tile_items (2, 4, 8 or 16; 0 = 8)
 * sets the persistent kernel's tile: 256 threads x tile_items probes.
 * Synchronous. */
typedef struct gj_batch_plan gj_batch_plan;
int gj_batch_plan_create(gj_index* const* indexes, uint32_t num_indexes, const uint32_t* h_batch_index,
                         const uint64_t* h_probe_offset, const uint64_t* h_batch_size, uint32_t num_batches,
                         uint32_t tile_items, void* stream, gj_batch_plan** plan);
int gj_batch_plan_free(gj_batch_plan* plan);
int gj_batch_plan_tile_items(const gj_batch_plan* plan, uint32_t* tile_items);
/* Enqueue a run on the stream: mode 0 = one persistent kernel over all
 * batches, mode 1 = one lookup launch per batch (the baseline).  Only device
 * work is enqueued (no host synchronisation, no allocation), so a run can be
 * captured in a CUDA graph.  If d_batch_done_ns != NULL (num_batches + 1
 * entries) it receives, per batch, the device globaltimer (ns) when the
 * batch's last probe finished, and in its last entry the start of the run.
 * Runs of one plan must not overlap (they share its counters). */
int gj_batch_plan_run(gj_batch_plan* plan, const uint64_t* d_probes, uint32_t* d_positions, uint32_t mode,
                      uint64_t* d_batch_done_ns, void* stream);
/* The same run through a CUDA graph: captured on first use (and again when
 * the buffers, mode or tile shape change), then replayed with one graph
 * launch on the stream. */
int gj_batch_plan_run_graph(gj_batch_plan* plan, const uint64_t* d_probes, uint32_t* d_positions, uint32_t mode,
                            uint64_t* d_batch_done_ns, void* stream);
/* Autotuner: time the persistent kernel with every tile shape on these
 * buffers and keep the fastest in the plan.  Synchronous.  Writes the chosen
 * tile_items and its time per run (ms) when the pointers are non-null. */
int gj_batch_plan_autotune(gj_batch_plan* plan, const uint64_t* d_probes, uint32_t* d_positions, void* stream,
                           uint32_t* tile_items, float* best_ms);

/* ---- autotuners ------------------------------------------------------------ */
/* Time every candidate on the caller's data (CUDA events on the stream, one
 * warm-up, best of two) and return the fastest.  They allocate scratch and
 * synchronise: set-up calls, not part of the probe path.  No counterpart in
 * the reference, whose experiment_config takes these values as options
 * (src/index_lookup_config.hpp:18-37).
 *   partitioned INLJ (pairs): fanout 2^5..2^12 x window {m, m/4, m/16};
 *   B+tree lookups: node width {4, 7 (compressed), 8, 15 (compressed), 16} x leaf width {4, 8, 16, 32}. */
int gj_autotune_partitioned(const gj_index* index, const uint64_t* d_probes, uint64_t m, void* stream,
                            uint32_t* radix_bits, uint64_t* window_size, float* best_ms);
int gj_autotune_btree(const uint64_t* d_keys, uint64_t n, const uint64_t* d_probes, uint64_t m, void* stream,
                      uint32_t* node_keys, uint32_t* leaf_keys, float* best_ms);
/* B+tree node format together with partition fanout and window for the
 * partitioned INLJ of these probes.  Partitioned probes search their
 * partition's column slice through the partition directory, so the node
 * format does not change their time: the default format (15 x 4) is
 * returned with gj_autotune_partitioned's fanout and window for it. */
int gj_autotune_partitioned_btree(const uint64_t* d_keys, uint64_t n, const uint64_t* d_probes, uint64_t m,
                                  void* stream, uint32_t* node_keys, uint32_t* leaf_keys, uint32_t* radix_bits,
                                  uint64_t* window_size, float* best_ms);

/* ---- calibration ---------------------------------------------------------- */
/* The random 32-byte sector read rate, the roofline of scattered probes
 * whose column does not fit L2 (each needs at least one random sector); no
 * counterpart in the reference.  Reads m sectors at pseudo-random indexes
 * (a hash of the load number and seed) of d_buf (n_sectors 32-byte sectors,
 * 32-byte aligned); fill64 != 0 asks L2 for 64-byte fills on misses, as the
 * probe kernels' scattered loads do.  d_sink: gj_calibrate_sink_words
 * uint64 words (the loaded data folded, so that no load is dropped). */
int gj_calibrate_sink_words(uint64_t* words);
int gj_calibrate_random_sectors(const uint64_t* d_buf, uint64_t n_sectors, uint64_t m, uint64_t seed,
                                uint32_t fill64, uint64_t* d_sink, void* stream);

/* ---- synthetic inputs (src/index_lookup_common.cuh:44-206, src/zipf.hpp) --- */
/* n strictly increasing keys, iid-uniform in distribution over [0, upper)
 * (sorted order statistics from exponential spacings).  Workspace:
 * gj_generate_workspace_size. */
int gj_generate_workspace_size(uint64_t n, size_t* bytes);
int gj_generate_sorted_keys(uint64_t* d_keys, uint64_t n, uint32_t distribution, uint64_t upper,
                            uint64_t seed, void* d_workspace, size_t workspace_bytes, void* stream);
#define GJ_DIST_UNIFORM 0u
#define GJ_DIST_LOGNORMAL 1u   /* lognormal(0, 2) scaled by 2^60, clipped to [0, upper) */
#define GJ_DIST_CLUSTERS 2u    /* 1024 dense runs separated by random gaps */
/* m probes d_probes[i] = d_keys[perm(rank_i - 1)], rank_i ~ Zipf(theta) over
 * [1, n] (theta = 0: uniform), perm a seeded permutation of [0, n).
 * absent_fraction of the probes are replaced by keys not in the column. */
int gj_generate_probes(const uint64_t* d_keys, uint64_t n, uint64_t* d_probes, uint64_t m, double theta,
                       double absent_fraction, uint64_t seed, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GPUJOIN_H */
