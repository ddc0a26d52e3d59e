/*
 * oracle.c -- CPU restatement of the gpujoin INLJ probe path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker): loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU baseline legs.  The CUDA
 * product never calls into this file.
 *
 * Each routine names the reference file:line whose behaviour it restates.
 * Plain C11 + pthreads so it builds with gcc on both x86_64 and aarch64.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ------------------------------------------------------------------------ */
/* threading helper: split [0, m) into contiguous chunks                      */
/* ------------------------------------------------------------------------ */
typedef void (*orc_range_fn)(void* ctx, uint64_t begin, uint64_t end);
typedef struct {
    orc_range_fn fn;
    void* ctx;
    uint64_t begin, end;
} orc_job;

static void* orc_job_main(void* p) {
    orc_job* j = (orc_job*)p;
    j->fn(j->ctx, j->begin, j->end);
    return NULL;
}

int orc_hardware_threads(void) {
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

static void orc_parallel_for(uint64_t m, int threads, orc_range_fn fn, void* ctx) {
    if (threads <= 0) threads = orc_hardware_threads();
    if (threads > 256) threads = 256;
    if (threads == 1 || m < 4096) {
        fn(ctx, 0, m);
        return;
    }
    pthread_t tid[256];
    orc_job jobs[256];
    uint64_t chunk = (m + (uint64_t)threads - 1) / (uint64_t)threads;
    int started = 0;
    for (int t = 0; t < threads; ++t) {
        uint64_t b = (uint64_t)t * chunk;
        uint64_t e = b + chunk < m ? b + chunk : m;
        if (b >= e) break;
        jobs[t].fn = fn; jobs[t].ctx = ctx; jobs[t].begin = b; jobs[t].end = e;
        if (pthread_create(&tid[t], NULL, orc_job_main, &jobs[t]) != 0) {
            fn(ctx, b, e);           /* run inline if a thread cannot start */
            jobs[t].fn = NULL;
        }
        started = t + 1;
    }
    for (int t = 0; t < started; ++t)
        if (jobs[t].fn) pthread_join(tid[t], NULL);
}

/* ------------------------------------------------------------------------ */
/* search primitives                                                          */
/* ------------------------------------------------------------------------ */
/* src/search.cuh:26-41 */
uint64_t orc_lower_bound(const uint64_t* arr, uint64_t n, uint64_t key) {
    uint64_t lower = 0, count = n;
    while (count > 0) {
        uint64_t step = count / 2;
        uint64_t mid = lower + step;
        if (arr[mid] < key) {
            lower = mid + 1;
            count -= step + 1;
        } else {
            count = step;
        }
    }
    return lower;
}

/* src/search.cuh:143-158; the reference leaves size 1 undefined (clz(0)),
 * here size 1 is answered directly. */
uint64_t orc_branch_free_lower_bound(const uint64_t* arr, uint64_t n, uint64_t key) {
    if (n == 0) return 0;
    if (n == 1) return arr[0] < key ? 1 : 0;
    unsigned steps = 63u - (unsigned)__builtin_clzll(n - 1);
    uint64_t mid = (uint64_t)1 << steps;
    uint64_t ret = (arr[mid] < key) ? (n - mid) : 0;
    for (unsigned s = 1; s <= steps; ++s) {
        mid >>= 1;
        ret += (arr[ret + mid] < key) ? mid : 0;
    }
    ret += (arr[ret] < key) ? 1 : 0;
    return ret;
}

/* src/search.cuh:86-101 (reads arr[0] even when n == 0, as the reference) */
uint64_t orc_branchy_binary_search(const uint64_t* arr, uint64_t n, uint64_t key) {
    uint64_t lower = 0, upper = n;
    do {
        uint64_t mid = ((upper - lower) / 2) + lower;
        if (key < arr[mid]) upper = mid;
        else if (key > arr[mid]) lower = mid + 1;
        else return mid;
    } while (lower < upper);
    return lower;
}

/* ------------------------------------------------------------------------ */
/* binary_search_index (src/indexes.cuh:336-375)                              */
/* ------------------------------------------------------------------------ */
typedef struct {
    const uint64_t* col; uint64_t n; const uint64_t* probes; uint32_t* out; int branch_free;
} bs_ctx;

static void bs_range(void* p, uint64_t b, uint64_t e) {
    bs_ctx* c = (bs_ctx*)p;
    for (uint64_t i = b; i < e; ++i) {
        uint64_t pos = c->branch_free ? orc_branch_free_lower_bound(c->col, c->n, c->probes[i])
                                      : orc_lower_bound(c->col, c->n, c->probes[i]);
        c->out[i] = pos < c->n ? (uint32_t)pos : ORC_INV;
    }
}

void orc_bs_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes, uint64_t m,
                   uint32_t* out, int threads) {
    bs_ctx c = {col, n, probes, out, 0};
    orc_parallel_for(m, threads, bs_range, &c);
}

void orc_bs_branch_free_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes,
                               uint64_t m, uint32_t* out, int threads) {
    bs_ctx c = {col, n, probes, out, 1};
    orc_parallel_for(m, threads, bs_range, &c);
}

typedef struct { const uint64_t* col; uint64_t n; const uint64_t* probes; uint32_t* out; } ex_ctx;
static void exact_range(void* p, uint64_t b, uint64_t e) {
    ex_ctx* c = (ex_ctx*)p;
    for (uint64_t i = b; i < e; ++i) {
        uint64_t pos = orc_lower_bound(c->col, c->n, c->probes[i]);
        c->out[i] = (pos < c->n && c->col[pos] == c->probes[i]) ? (uint32_t)pos : ORC_INV;
    }
}
void orc_exact_lookup(const uint64_t* col, uint64_t n, const uint64_t* probes, uint64_t m,
                      uint32_t* out, int threads) {
    ex_ctx c = {col, n, probes, out};
    orc_parallel_for(m, threads, exact_range, &c);
}

/* ------------------------------------------------------------------------ */
/* clustered B+tree (src/btree.cuh)                                           */
/* ------------------------------------------------------------------------ */
/* A child reference is either an inner node index or, below a final inner
 * node, the column offset of a leaf slice. */
typedef struct {
    uint32_t count;
    int is_final_inner;
    uint64_t* keys;      /* inner_keys entries, padded with UINT64_MAX (:118-122) */
    uint64_t* children;  /* inner_keys + 1 entries */
} orc_bnode;

struct orc_btree {
    const uint64_t* col;
    uint64_t n;
    uint32_t leaf_keys, inner_keys;
    orc_bnode* nodes;
    uint64_t nnodes, cap;
    uint64_t root;
    uint32_t depth;
};

static uint64_t bt_new_inner(orc_btree* t, int final_inner) {
    if (t->nnodes == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 16;
        t->nodes = (orc_bnode*)realloc(t->nodes, t->cap * sizeof(orc_bnode));
    }
    orc_bnode* nd = &t->nodes[t->nnodes];
    nd->count = 0;
    nd->is_final_inner = final_inner;
    nd->keys = (uint64_t*)malloc(sizeof(uint64_t) * t->inner_keys);
    nd->children = (uint64_t*)calloc(t->inner_keys + 1, sizeof(uint64_t));
    for (uint32_t i = 0; i < t->inner_keys; ++i) nd->keys[i] = UINT64_MAX;
    return t->nnodes++;
}

/* max_key(): src/btree.cuh:156-167 (clustered) */
static uint64_t bt_max_key(const orc_btree* t, uint64_t ref, int is_leaf) {
    while (!is_leaf) {
        const orc_bnode* nd = &t->nodes[ref];
        is_leaf = nd->is_final_inner;
        ref = nd->children[nd->count];
    }
    uint64_t cnt = t->n - ref < t->leaf_keys ? t->n - ref : t->leaf_keys;
    return t->col[ref + cnt - 1];
}

orc_btree* orc_btree_build(const uint64_t* col, uint64_t n, uint32_t leaf_keys, uint32_t inner_keys) {
    if (n == 0 || leaf_keys == 0 || inner_keys == 0) return NULL;
    orc_btree* t = (orc_btree*)calloc(1, sizeof(orc_btree));
    t->col = col; t->n = n; t->leaf_keys = leaf_keys; t->inner_keys = inner_keys;
    /* leaves: every leaf_keys-th column position (:237-243) */
    uint64_t nlower = (n + leaf_keys - 1) / leaf_keys;
    uint64_t* lower = (uint64_t*)malloc(sizeof(uint64_t) * nlower);
    for (uint64_t i = 0; i < nlower; ++i) lower[i] = i * leaf_keys;
    int lower_is_leaf = 1;
    uint32_t inverse_depth = 1;
    /* construct_inner_nodes(): src/btree.cuh:176-206 with load_factor 1.0 */
    for (;;) {
        if (nlower == 1 && inverse_depth > 1) break;
        uint64_t* cur = (uint64_t*)malloc(sizeof(uint64_t) * (nlower / 2 + 2));
        uint64_t ncur = 0, capcur = nlower / 2 + 2;
        uint64_t node = bt_new_inner(t, inverse_depth == 1);
        for (uint64_t i = 0; i + 1 < nlower; ++i) {
            uint64_t child = lower[i];
            uint64_t sep = bt_max_key(t, child, lower_is_leaf);
            orc_bnode* nd = &t->nodes[node];
            if (nd->count >= t->inner_keys) {
                nd->children[nd->count] = child;
                if (ncur == capcur) { capcur *= 2; cur = (uint64_t*)realloc(cur, sizeof(uint64_t) * capcur); }
                cur[ncur++] = node;
                node = bt_new_inner(t, inverse_depth == 1);
            } else {
                nd->keys[nd->count] = sep;
                nd->children[nd->count] = child;
                nd->count += 1;
            }
        }
        t->nodes[node].children[t->nodes[node].count] = lower[nlower - 1];
        if (ncur == capcur) { capcur *= 2; cur = (uint64_t*)realloc(cur, sizeof(uint64_t) * capcur); }
        cur[ncur++] = node;
        free(lower);
        lower = cur; nlower = ncur; lower_is_leaf = 0;
        inverse_depth += 1;
    }
    t->root = lower[0];
    t->depth = inverse_depth - 1;
    free(lower);
    return t;
}

uint32_t orc_btree_depth(const orc_btree* t) { return t->depth; }

uint64_t orc_btree_nodes(const orc_btree* t) { return t->nnodes; }

int64_t orc_btree_write_pages(const orc_btree* t, uint8_t* out, uint64_t page_bytes, uint64_t keys_off,
                              uint64_t children_off, uint64_t pages_base, uint64_t col_base) {
    if (keys_off < 4 || keys_off + 8ull * t->inner_keys > children_off ||
        children_off + 8ull * (t->inner_keys + 1) > page_bytes || (keys_off | children_off) % 8 != 0)
        return -1;
    memset(out, 0, t->nnodes * page_bytes);
    for (uint64_t i = 0; i < t->nnodes; ++i) {
        const orc_bnode* nd = &t->nodes[i];
        uint8_t* pg = out + i * page_bytes;
        const uint16_t count = (uint16_t)nd->count;
        memcpy(pg, &count, 2);
        pg[2] = 0;  /* isLeaf: the clustered tree has no leaf pages */
        pg[3] = (uint8_t)(nd->is_final_inner ? 1 : 0);
        memcpy(pg + keys_off, nd->keys, 8ull * t->inner_keys);
        for (uint32_t c = 0; c <= nd->count; ++c) {
            const uint64_t ptr = nd->is_final_inner ? col_base + 8ull * nd->children[c]
                                                    : pages_base + page_bytes * nd->children[c];
            memcpy(pg + children_off + 8ull * c, &ptr, 8);
        }
    }
    return (int64_t)t->root;
}

/* lookup(): src/btree.cuh:504-531 */
static uint32_t bt_lookup_one(const orc_btree* t, uint64_t key) {
    uint64_t ref = t->root;
    for (;;) {
        const orc_bnode* nd = &t->nodes[ref];
        uint64_t pos = orc_branchy_binary_search(nd->keys, nd->count, key);
        ref = nd->children[pos];
        if (nd->is_final_inner) break;
    }
    uint64_t cnt = t->n - ref < t->leaf_keys ? t->n - ref : t->leaf_keys;
    uint64_t pos = orc_branchy_binary_search(t->col + ref, cnt, key);
    if (pos < cnt && t->col[ref + pos] == key) return (uint32_t)(ref + pos);
    return ORC_INV;
}

typedef struct { const orc_btree* t; const uint64_t* probes; uint32_t* out; } bt_ctx;
static void bt_range(void* p, uint64_t b, uint64_t e) {
    bt_ctx* c = (bt_ctx*)p;
    for (uint64_t i = b; i < e; ++i) c->out[i] = bt_lookup_one(c->t, c->probes[i]);
}
void orc_btree_lookup(const orc_btree* t, const uint64_t* probes, uint64_t m, uint32_t* out, int threads) {
    bt_ctx c = {t, probes, out};
    orc_parallel_for(m, threads, bt_range, &c);
}

/* The global lower bound through the same tree (binary_search_index's
 * semantics, src/indexes.cuh:357-361: position of the first key >= probe,
 * ORC_INV at n).  Separators are the children's maximum keys, so the lower
 * bound over a node's separators names the child holding the lower bound;
 * only the rightmost leaf can come up empty (probe above every key).  A
 * faster restatement of orc_bs_lookup for large checks (tests compare the
 * two). */
static uint32_t bt_lower_bound_one(const orc_btree* t, uint64_t key) {
    uint64_t ref = t->root;
    for (;;) {
        const orc_bnode* nd = &t->nodes[ref];
        uint64_t pos = orc_branchy_binary_search(nd->keys, nd->count, key);
        ref = nd->children[pos];
        if (nd->is_final_inner) break;
    }
    uint64_t cnt = t->n - ref < t->leaf_keys ? t->n - ref : t->leaf_keys;
    uint64_t lb = ref + orc_branchy_binary_search(t->col + ref, cnt, key);
    return lb < t->n ? (uint32_t)lb : ORC_INV;
}
static void bt_lb_range(void* p, uint64_t b, uint64_t e) {
    bt_ctx* c = (bt_ctx*)p;
    for (uint64_t i = b; i < e; ++i) c->out[i] = bt_lower_bound_one(c->t, c->probes[i]);
}
void orc_btree_lower_bound(const orc_btree* t, const uint64_t* probes, uint64_t m, uint32_t* out, int threads) {
    bt_ctx c = {t, probes, out};
    orc_parallel_for(m, threads, bt_lb_range, &c);
}

void orc_btree_free(orc_btree* t) {
    if (!t) return;
    for (uint64_t i = 0; i < t->nnodes; ++i) { free(t->nodes[i].keys); free(t->nodes[i].children); }
    free(t->nodes);
    free(t);
}

/* ------------------------------------------------------------------------ */
/* Harmonia (src/harmonia.cuh)                                                */
/* ------------------------------------------------------------------------ */
typedef struct {
    uint64_t key_count, node_count, node_prefix, key_prefix;
} hm_level;

struct orc_harmonia {
    const uint64_t* col;
    uint64_t n;
    uint64_t K;            /* max_keys per node (fanout - 1) */
    uint64_t* keys;        /* inner key array, K per inner node */
    uint64_t inner_size;   /* K * number of inner nodes */
    uint64_t* children;    /* one entry per node (inner + leaf) */
    uint64_t nchildren;
    hm_level* levels;      /* root first */
    uint32_t depth;
    int err;
};

/* key array with the column appended behind the inner keys (:224-234) */
static uint64_t hm_key_at(const orc_harmonia* h, uint64_t idx) {
    return idx >= h->inner_size ? h->col[idx - h->inner_size] : h->keys[idx];
}

/* get_largest_key(): src/harmonia.cuh:249-264 */
static uint64_t hm_largest(const orc_harmonia* h, uint32_t level, uint64_t node) {
    for (;;) {
        const hm_level* ld = &h->levels[level];
        uint64_t nkc = (node < ld->node_count - 1) ? h->K : (ld->key_count - node * h->K);
        if (level == h->depth - 1) {
            uint64_t start = h->K * (ld->node_prefix + node);
            return hm_key_at(h, start + nkc - 1);
        }
        node = (h->K + 1) * node + nkc;
        level += 1;
    }
}

orc_harmonia* orc_harmonia_build(const uint64_t* col, uint64_t n, uint32_t max_keys, int* err) {
    *err = 0;
    if (max_keys == 0 || n == 0 || n % max_keys != 0) { *err = 1; return NULL; }
    orc_harmonia* h = (orc_harmonia*)calloc(1, sizeof(orc_harmonia));
    h->col = col; h->n = n; h->K = max_keys;
    const uint64_t K = max_keys, F = (uint64_t)max_keys + 1;

    /* gather_tree_info(): src/harmonia.cuh:133-190 (levels are prepended) */
    hm_level tmp[64];
    int nl = 0;
    uint64_t prev_pages = 0, kc = n;
    for (;;) {
        if (nl == 64) { *err = 2; free(h); return NULL; }
        uint64_t pages = (kc + K - 1) / K;
        if (F * pages < prev_pages) pages += 1;
        tmp[nl].key_count = kc;
        tmp[nl].node_count = pages;
        nl++;
        prev_pages = pages;
        kc = (K * pages) / F;
        if (pages == 1) break;
    }
    h->depth = (uint32_t)nl;
    h->levels = (hm_level*)calloc((size_t)nl, sizeof(hm_level));
    for (int i = 0; i < nl; ++i) h->levels[i] = tmp[nl - 1 - i];
    uint64_t tn = 0, tk = 0;
    for (int i = 0; i < nl; ++i) {
        h->levels[i].node_prefix = tn; tn += h->levels[i].node_count;
        h->levels[i].key_prefix = tk; tk += h->levels[i].key_count;
    }
    if (h->depth > 16) { *err = 2; orc_harmonia_free(h); return NULL; }   /* max_depth, :392 */

    const hm_level* leaf = &h->levels[nl - 1];
    h->inner_size = K * leaf->node_prefix;
    h->nchildren = leaf->node_prefix + leaf->node_count;
    h->keys = (uint64_t*)malloc(sizeof(uint64_t) * (h->inner_size ? h->inner_size : 1));
    for (uint64_t i = 0; i < h->inner_size; ++i) h->keys[i] = UINT64_MAX;
    h->children = (uint64_t*)calloc(h->nchildren, sizeof(uint64_t));

    /* store_structure(): src/harmonia.cuh:320-342 */
    uint64_t off = 0, prefix = 1;
    for (int l = 0; l < nl - 1; ++l) {
        const hm_level* lv = &h->levels[l];
        for (uint64_t j = 0; j < lv->node_count; ++j) {
            h->children[off++] = prefix;
            uint64_t nkc = (j < lv->node_count - 1) ? K : (lv->key_count - j * K);
            prefix += nkc + 1;
        }
    }
    /* populate_leaf_nodes(): src/harmonia.cuh:296-313 */
    off = leaf->node_prefix;
    for (uint64_t j = 0; j < leaf->node_count; ++j) h->children[off + j] = j * K;

    /* populate_inner_nodes(): src/harmonia.cuh:266-294, bottom-up */
    for (int l = nl - 2; l >= 0; --l) {
        const hm_level* cur = &h->levels[l];
        const hm_level* low = &h->levels[l + 1];
        uint64_t start = (l > 0 ? cur->node_prefix : 0) * K;
        int skipped = 1;
        uint64_t w = 0;
        for (uint64_t c = 0; c + 1 < low->node_count; ++c) {
            if (!skipped && (w % K) == 0) { skipped = 1; continue; }
            uint64_t sep = hm_largest(h, (uint32_t)(l + 1), c);
            uint64_t idx = start + w;
            if (idx >= h->inner_size) { *err = 3; orc_harmonia_free(h); return NULL; }
            h->keys[idx] = sep;
            w += 1;
            skipped = 0;
        }
    }
    return h;
}

/* host lookup(): src/harmonia.cuh:640-668 */
uint64_t orc_harmonia_lookup_one(const orc_harmonia* h, uint64_t key) {
    const uint64_t K = h->K;
    uint64_t pos = 0, actual = 0;
    int have_actual = 0;
    for (uint32_t d = 1; d <= h->depth; ++d) {
        uint64_t base = K * pos;
        /* lower_bound over the K keys of the node (std::lower_bound) */
        uint64_t lo = 0, cnt = K;
        while (cnt > 0) {
            uint64_t step = cnt / 2, mid = lo + step;
            uint64_t v = (d == h->depth) ? hm_key_at(h, base + mid) : h->keys[base + mid];
            if (v < key) { lo = mid + 1; cnt -= step + 1; } else cnt = step;
        }
        /* actual = node_start[lb]; past the last leaf slot that read is out
         * of range in the reference and can only pair with pos >= size */
        uint64_t aidx = base + lo;
        if (d == h->depth) {
            uint64_t cidx = aidx - h->inner_size;     /* column index of node_start[lb] */
            have_actual = cidx < h->n;
            actual = have_actual ? h->col[cidx] : 0;
        } else {
            actual = aidx < h->inner_size ? h->keys[aidx] : 0;
        }
        pos = h->children[pos] + lo;
    }
    if (pos < h->n && have_actual && key == actual) return pos;
    return UINT64_MAX;
}

typedef struct { const orc_harmonia* h; const uint64_t* probes; uint32_t* out; } hm_ctx;
static void hm_range(void* p, uint64_t b, uint64_t e) {
    hm_ctx* c = (hm_ctx*)p;
    for (uint64_t i = b; i < e; ++i) {
        uint64_t r = orc_harmonia_lookup_one(c->h, c->probes[i]);
        c->out[i] = r == UINT64_MAX ? ORC_INV : (uint32_t)r;
    }
}
void orc_harmonia_lookup(const orc_harmonia* h, const uint64_t* probes, uint64_t m, uint32_t* out, int threads) {
    hm_ctx c = {h, probes, out};
    orc_parallel_for(m, threads, hm_range, &c);
}

void orc_harmonia_arrays(const orc_harmonia* h, const uint64_t** keys, uint64_t* nkeys,
                         const uint64_t** children, uint64_t* nchildren, uint32_t* depth) {
    *keys = h->keys; *nkeys = h->inner_size;
    *children = h->children; *nchildren = h->nchildren;
    *depth = h->depth;
}

void orc_harmonia_free(orc_harmonia* h) {
    if (!h) return;
    free(h->keys); free(h->children); free(h->levels); free(h);
}

/* ------------------------------------------------------------------------ */
/* RadixSpline                                                                */
/* ------------------------------------------------------------------------ */
struct orc_rs {
    uint64_t min_key, max_key, n;
    uint32_t radix_bits, shift_bits, max_error;
    uint32_t* table; uint64_t table_len;
    uint64_t* sx; double* sy; uint64_t npoints, cap;
};

static void rs_push(orc_rs* r, uint64_t x, double y, uint64_t* prev_prefix) {
    /* radix table entry for every prefix up to this point's prefix */
    uint64_t prefix = (x - r->min_key) >> r->shift_bits;
    if (r->npoints == 0) {
        *prev_prefix = 0;
        r->table[0] = 0;
    }
    if (prefix != *prev_prefix) {
        for (uint64_t p = *prev_prefix + 1; p <= prefix; ++p) r->table[p] = (uint32_t)r->npoints;
        *prev_prefix = prefix;
    }
    if (r->npoints == r->cap) {
        r->cap = r->cap ? 2 * r->cap : 1024;
        r->sx = (uint64_t*)realloc(r->sx, sizeof(uint64_t) * r->cap);
        r->sy = (double*)realloc(r->sy, sizeof(double) * r->cap);
    }
    r->sx[r->npoints] = x; r->sy[r->npoints] = y; r->npoints++;
}

/* sign of the cross product (dx1,dy1) x (dx2,dy2): +1 clockwise, -1 counter */
static int rs_orient(double dx1, double dy1, double dx2, double dy2) {
    double e = dy1 * dx2 - dy2 * dx1;
    if (e > 2.220446049250313e-16) return 1;
    if (e < -2.220446049250313e-16) return -1;
    return 0;
}

orc_rs* orc_rs_build(const uint64_t* col, uint64_t n, uint32_t radix_bits, uint32_t max_error) {
    if (n == 0 || radix_bits == 0 || radix_bits > 30) return NULL;
    orc_rs* r = (orc_rs*)calloc(1, sizeof(orc_rs));
    r->min_key = col[0]; r->max_key = col[n - 1]; r->n = n;
    r->radix_bits = radix_bits; r->max_error = max_error;
    uint64_t range = r->max_key - r->min_key;
    unsigned used = range ? 64u - (unsigned)__builtin_clzll(range) : 0u;
    r->shift_bits = used > radix_bits ? used - radix_bits : 0;
    r->table_len = ((uint64_t)1 << radix_bits) + 2;
    r->table = (uint32_t*)calloc(r->table_len, sizeof(uint32_t));

    /* GreedySplineCorridor over the CDF points (key_i, i) */
    uint64_t prev_prefix = 0;
    uint64_t px = 0; double py = 0;          /* previous CDF point */
    uint64_t ux = 0, lx = 0; double uy = 0, ly = 0;   /* corridor limits */
    uint64_t distinct = 0;
    for (uint64_t i = 0; i < n; ++i) {
        uint64_t key = col[i];
        double y = (double)i;
        if (i == 0) {
            rs_push(r, key, y, &prev_prefix);
            distinct = 1; px = key; py = y;
            continue;
        }
        if (key == px) continue;
        distinct += 1;
        double upper_y = y + (double)max_error;
        double lower_y = (double)max_error > y ? 0.0 : y - (double)max_error;
        if (distinct == 2) {
            ux = key; uy = upper_y; lx = key; ly = lower_y;
            px = key; py = y;
            continue;
        }
        uint64_t bx = r->sx[r->npoints - 1]; double by = r->sy[r->npoints - 1];
        double udx = (double)(ux - bx), udy = uy - by;
        double ldx = (double)(lx - bx), ldy = ly - by;
        double dx = (double)(key - bx), dy = y - by;
        if (rs_orient(udx, udy, dx, dy) != 1 || rs_orient(ldx, ldy, dx, dy) != -1) {
            /* the point leaves the corridor: the previous point becomes a knot */
            rs_push(r, px, py, &prev_prefix);
            ux = key; uy = upper_y; lx = key; ly = lower_y;
        } else {
            if (rs_orient(udx, udy, dx, upper_y - by) == 1) { ux = key; uy = upper_y; }
            if (rs_orient(ldx, ldy, dx, lower_y - by) == -1) { lx = key; ly = lower_y; }
        }
        px = key; py = y;
    }
    if (r->sx[r->npoints - 1] != r->max_key) rs_push(r, px, py, &prev_prefix);
    for (uint64_t p = prev_prefix + 1; p < r->table_len; ++p) r->table[p] = (uint32_t)r->npoints;
    return r;
}

/* get_spline_segment() + get_estimate(): src/rs.cuh:118-154 */
double orc_rs_estimate(const orc_rs* r, uint64_t key) {
    if (key <= r->min_key) return 0.0;
    if (key >= r->max_key) return (double)(r->n - 1);
    uint64_t prefix = (key - r->min_key) >> r->shift_bits;
    uint64_t b = r->table[prefix], e = r->table[prefix + 1];
    uint64_t lo = b, cnt = e - b;
    while (cnt > 0) {
        uint64_t step = cnt / 2, mid = lo + step;
        if (r->sx[mid] < key) { lo = mid + 1; cnt -= step + 1; } else cnt = step;
    }
    uint64_t idx = lo;
    double x_diff = (double)(r->sx[idx] - r->sx[idx - 1]);
    double y_diff = r->sy[idx] - r->sy[idx - 1];
    double slope = y_diff / x_diff;
    double key_diff = (double)(key - r->sx[idx - 1]);
    volatile double prod = key_diff * slope;   /* no contraction into an fma */
    return prod + r->sy[idx - 1];
}

typedef struct { const orc_rs* r; const uint64_t* col; const uint64_t* probes; uint32_t* out; } rs_ctx;
static void rs_range(void* p, uint64_t b0, uint64_t e0) {
    rs_ctx* c = (rs_ctx*)p;
    const orc_rs* r = c->r;
    const double err = (double)r->max_error;
    for (uint64_t i = b0; i < e0; ++i) {
        uint64_t key = c->probes[i];
        double est = orc_rs_estimate(r, key);
        /* window arithmetic of src/indexes.cuh:207-214 */
        uint64_t b = est < err ? 0 : (uint64_t)(est - err);
        uint64_t e = (est + err + 2 > (double)r->n) ? r->n : (uint64_t)(est + err + 2);
        if (b > e) b = e;
        uint64_t pos = b + orc_lower_bound(c->col + b, e - b, key);
        /* the window must bracket the lower bound; otherwise search globally */
        if ((pos == b && b > 0 && c->col[b - 1] >= key) || (pos == e && e < r->n && c->col[e] < key))
            pos = orc_lower_bound(c->col, r->n, key);
        c->out[i] = pos < r->n ? (uint32_t)pos : ORC_INV;
    }
}
void orc_rs_lookup(const orc_rs* r, const uint64_t* col, const uint64_t* probes, uint64_t m,
                   uint32_t* out, int threads) {
    rs_ctx c = {r, col, probes, out};
    orc_parallel_for(m, threads, rs_range, &c);
}

void orc_rs_arrays(const orc_rs* r, const uint32_t** radix_table, uint64_t* table_len,
                   const uint64_t** spline_x, const double** spline_y, uint64_t* npoints,
                   uint32_t* shift_bits) {
    *radix_table = r->table; *table_len = r->table_len;
    *spline_x = r->sx; *spline_y = r->sy; *npoints = r->npoints; *shift_bits = r->shift_bits;
}

void orc_rs_free(orc_rs* r) {
    if (!r) return;
    free(r->table); free(r->sx); free(r->sy); free(r);
}

/* ------------------------------------------------------------------------ */
/* stable range partition                                                     */
/* ------------------------------------------------------------------------ */
void orc_range_partition(const uint64_t* keys, uint64_t m, uint64_t min_key, uint32_t shift,
                         uint32_t radix_bits, uint64_t* out_keys, uint32_t* out_rows,
                         uint64_t* offsets) {
    const uint64_t fanout = (uint64_t)1 << radix_bits;
    uint64_t* hist = (uint64_t*)calloc(fanout + 1, sizeof(uint64_t));
    for (uint64_t i = 0; i < m; ++i) {
        uint64_t k = keys[i];
        uint64_t p = k <= min_key ? 0 : (shift >= 64 ? 0 : (k - min_key) >> shift);
        if (p >= fanout) p = fanout - 1;
        hist[p]++;
    }
    uint64_t s = 0;
    for (uint64_t p = 0; p < fanout; ++p) { offsets[p] = s; s += hist[p]; }
    offsets[fanout] = s;
    for (uint64_t p = 0; p < fanout; ++p) hist[p] = offsets[p];
    for (uint64_t i = 0; i < m; ++i) {
        uint64_t k = keys[i];
        uint64_t p = k <= min_key ? 0 : (shift >= 64 ? 0 : (k - min_key) >> shift);
        if (p >= fanout) p = fanout - 1;
        uint64_t d = hist[p]++;
        out_keys[d] = k;
        out_rows[d] = (uint32_t)i;
    }
    free(hist);
}

/* ------------------------------------------------------------------------ */
/* join pairs, star join                                                      */
/* ------------------------------------------------------------------------ */
uint64_t orc_pairs_from_positions(const uint32_t* pos, uint64_t m, uint32_t* out_rows, uint32_t* out_pos) {
    uint64_t c = 0;
    for (uint64_t i = 0; i < m; ++i) {
        if (pos[i] != ORC_INV) {
            out_rows[c] = (uint32_t)i;
            out_pos[c] = pos[i];
            c++;
        }
    }
    return c;
}

/* query_14_part_build(): src/tpch/cpu_only.cpp:230-275 with the PROMO prefix
 * test replaced by a per-row flag and the hash table by an exact lookup */
void orc_star_join(const uint32_t* fk, const uint32_t* date, const int64_t* price,
                   const int64_t* disc, uint64_t nfact, const uint64_t* dim_keys,
                   const uint8_t* dim_flag, uint64_t ndim, uint32_t lo, uint32_t hi,
                   int64_t out[2]) {
    uint64_t num = 0, den = 0;   /* two's-complement wrap, like the GPU atomics */
    for (uint64_t i = 0; i < nfact; ++i) {
        if (date[i] < lo || date[i] >= hi) continue;
        uint64_t key = fk[i];
        uint64_t j = orc_lower_bound(dim_keys, ndim, key);
        if (j >= ndim || dim_keys[j] != key) continue;
        int64_t summand = price[i] * (100 - disc[i]);
        den += (uint64_t)summand;
        if (dim_flag[j]) num += (uint64_t)summand;
    }
    out[0] = (int64_t)num;
    out[1] = (int64_t)den;
}

/* ------------------------------------------------------------------------ */
/* generators                                                                 */
/* ------------------------------------------------------------------------ */
/* SplitMix64 finaliser (Vigna) */
uint64_t orc_mix64(uint64_t x) {
    uint64_t z = x + 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static double u01(uint64_t seed, uint64_t index, uint64_t attempt) {
    uint64_t h = orc_mix64(orc_mix64(seed ^ 0x5851f42d4c957f2dull) + index * 0x2545f4914f6cdd1dull + attempt);
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

/* Rejection-inversion (Hoermann & Derflinger, ACM TOMACS 6(3), 1996), the
 * method of src/zipf.hpp:13-102: hat h(x) = x^-q, H its integral, H^-1. */
static double zf_expm1_over(double t) { return fabs(t) > 1e-8 ? expm1(t) / t : 1.0 + t / 2.0 * (1.0 + t / 3.0 * (1.0 + t / 4.0)); }
static double zf_log1p_over(double t) { return fabs(t) > 1e-8 ? log1p(t) / t : 1.0 - t * (0.5 - t * (1.0 / 3.0 - t * 0.25)); }
static double zf_H(double x, double q) { double lx = log(x); return zf_expm1_over((1.0 - q) * lx) * lx; }
static double zf_Hinv(double u, double q) { double t = u * (1.0 - q); if (t < -1.0) t = -1.0; return exp(zf_log1p_over(t) * u); }
static double zf_h(double x, double q) { return exp(-q * log(x)); }

uint64_t orc_zipf_rank(uint64_t n, double q, uint64_t seed, uint64_t index) {
    if (n <= 1) return 1;
    const double hx1 = zf_H(1.5, q) - 1.0;
    const double hn = zf_H((double)n + 0.5, q);
    for (uint64_t a = 0;; ++a) {
        double u = hx1 + u01(seed, index, a) * (hn - hx1);
        double x = zf_Hinv(u, q);
        double kr = floor(x + 0.5);
        uint64_t k = kr < 1.0 ? 1 : (kr > (double)n ? n : (uint64_t)kr);
        if (u >= zf_H((double)k + 0.5, q) - zf_h((double)k, q)) return k;
        if (a > 1000) return k;   /* bounded retry; never reached in practice */
    }
}

/* four-round Feistel network on 2*half bits, cycle-walked into [0, n) */
uint64_t orc_permute(uint64_t x, uint64_t n, uint64_t seed) {
    if (n <= 1) return 0;
    unsigned bits = 64u - (unsigned)__builtin_clzll(n - 1);
    if (bits < 2) bits = 2;
    if (bits & 1u) bits++;
    const unsigned half = bits / 2;
    const uint64_t mask = ((uint64_t)1 << half) - 1;
    for (;;) {
        uint64_t l = x >> half, r = x & mask;
        for (unsigned round = 0; round < 4; ++round) {
            uint64_t f = orc_mix64(r ^ (seed + 0x632be59bd9b4e019ull * (round + 1))) & mask;
            uint64_t nl = r, nr = l ^ f;
            l = nl; r = nr;
        }
        x = (l << half) | r;
        if (x < n) return x;
    }
}

typedef struct { const uint64_t* col; uint64_t n; uint64_t* out; double q; uint64_t seed; } zp_ctx;
static void zp_range(void* p, uint64_t b, uint64_t e) {
    zp_ctx* c = (zp_ctx*)p;
    const uint64_t perm_seed = orc_mix64(c->seed ^ 0xa0761d6478bd642full);
    for (uint64_t i = b; i < e; ++i) {
        uint64_t rank = c->q == 0.0 ? 1 + (orc_mix64(c->seed + i) % c->n) : orc_zipf_rank(c->n, c->q, c->seed, i);
        c->out[i] = c->col[orc_permute(rank - 1, c->n, perm_seed)];
    }
}
void orc_zipf_probes(const uint64_t* col, uint64_t n, uint64_t* out, uint64_t m, double q, uint64_t seed,
                     int threads) {
    zp_ctx c = {col, n, out, q, seed};
    orc_parallel_for(m, threads, zp_range, &c);
}

/* ------------------------------------------------------------------------ */
/* learned model: MLP 1 -> H -> H -> 1 forward / backward                     */
/* ------------------------------------------------------------------------ */
float orc_mlp_forward(const float* P, int H, float x) {
    const float* W1 = P; const float* b1 = P + H; const float* W2 = P + 2 * H;
    const float* b2 = W2 + H * H; const float* W3 = b2 + H; const float* b3 = W3 + H;
    float h1[256], h2v;
    float out = b3[0];
    for (int j = 0; j < H; ++j) { float a = W1[j] * x + b1[j]; h1[j] = a > 0.f ? a : 0.f; }
    for (int o = 0; o < H; ++o) {
        float a = b2[o];
        for (int j = 0; j < H; ++j) a += W2[o * H + j] * h1[j];
        h2v = a > 0.f ? a : 0.f;
        out += W3[o] * h2v;
    }
    return out;
}

double orc_mlp_loss_grad(const float* P, int H, const float* x, const float* y, uint64_t count, double* g) {
    const float* W1 = P; const float* b1 = P + H; const float* W2 = P + 2 * H;
    const float* b2 = W2 + H * H; const float* W3 = b2 + H; const float* b3 = W3 + H;
    double* gW1 = g; double* gb1 = g + H; double* gW2 = g + 2 * H;
    double* gb2 = gW2 + H * H; double* gW3 = gb2 + H; double* gb3 = gW3 + H;
    double loss = 0;
    double a1[256], h1[256], a2[256], h2[256], d2[256], d1[256];
    for (uint64_t s = 0; s < count; ++s) {
        double xv = x[s];
        for (int j = 0; j < H; ++j) { a1[j] = (double)W1[j] * xv + b1[j]; h1[j] = a1[j] > 0 ? a1[j] : 0; }
        double out = b3[0];
        for (int o = 0; o < H; ++o) {
            double a = b2[o];
            for (int j = 0; j < H; ++j) a += (double)W2[o * H + j] * h1[j];
            a2[o] = a; h2[o] = a > 0 ? a : 0;
            out += (double)W3[o] * h2[o];
        }
        double diff = out - y[s];
        loss += diff * diff;
        double dout = 2.0 * diff;
        gb3[0] += dout;
        for (int o = 0; o < H; ++o) {
            gW3[o] += dout * h2[o];
            d2[o] = a2[o] > 0 ? dout * W3[o] : 0.0;
            gb2[o] += d2[o];
        }
        for (int j = 0; j < H; ++j) {
            double acc = 0;
            for (int o = 0; o < H; ++o) { gW2[o * H + j] += d2[o] * h1[j]; acc += d2[o] * W2[o * H + j]; }
            d1[j] = a1[j] > 0 ? acc : 0.0;
            gW1[j] += d1[j] * xv;
            gb1[j] += d1[j];
        }
    }
    return loss;
}
