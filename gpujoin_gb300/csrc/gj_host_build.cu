// gj_host_build.cpp -- host-side construction of the Harmonia and RadixSpline
// search structures (sequential, O(n); not on the probe path).
//
// Harmonia follows harmonia_tree::construct (src/harmonia.cuh:346-404): the
// same level sizing, children prefix sums and separator placement, so that
// lookups return exactly the reference's positions.  RadixSpline follows the
// published single-pass builder (GreedySplineCorridor + radix table, Kipf et
// al. 2020), whose result the reference consumes in src/rs.cuh:54-64.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "gj_internal.h"

namespace gj {

namespace {
struct level_info {
    uint64_t key_count;
    uint64_t node_count;
    uint64_t node_prefix;  // nodes on the levels above
};
}  // namespace

int build_harmonia_arrays(const uint64_t* col, uint64_t n, harmonia_arrays* out) {
    constexpr uint64_t K = kHarmoniaKeys;  // keys per node
    constexpr uint64_t F = K + 1;          // fanout
    if (n == 0 || n % K != 0) {
        set_error("harmonia: the column size must be a non-zero multiple of %u (got %llu)", (unsigned)K,
                  (unsigned long long)n);
        return GJ_ERR_INVALID_ARGUMENT;
    }
    // level sizes, leaf level first (src/harmonia.cuh:137-176)
    std::vector<level_info> bottom_up;
    uint64_t previous_pages = 0, key_count = n;
    for (;;) {
        uint64_t pages = (key_count + K - 1) / K;
        if (F * pages < previous_pages) pages += 1;  // rightmost node of the level owns one extra child
        bottom_up.push_back({key_count, pages, 0});
        previous_pages = pages;
        key_count = (K * pages) / F;
        if (pages == 1) break;
        if (bottom_up.size() > 16) {
            set_error("harmonia: tree deeper than 16 levels");
            return GJ_ERR_UNSUPPORTED;
        }
    }
    std::vector<level_info> levels(bottom_up.rbegin(), bottom_up.rend());  // root first
    uint64_t total_nodes = 0;
    for (auto& l : levels) {
        l.node_prefix = total_nodes;
        total_nodes += l.node_count;
    }
    const uint32_t depth = static_cast<uint32_t>(levels.size());
    const level_info& leaf = levels.back();
    const uint64_t inner_size = K * leaf.node_prefix;

    out->depth = depth;
    out->level_nodes.clear();
    for (const auto& l : levels) out->level_nodes.push_back(l.node_count);
    out->keys.assign(inner_size, UINT64_MAX);
    out->children.assign(total_nodes, 0);

    // children of inner nodes: running prefix over (node keys + 1), starting at 1
    uint64_t off = 0, prefix = 1;
    for (uint32_t l = 0; l + 1 < depth; ++l) {
        const level_info& lv = levels[l];
        for (uint64_t j = 0; j < lv.node_count; ++j) {
            out->children[off++] = prefix;
            const uint64_t node_keys = (j < lv.node_count - 1) ? K : (lv.key_count - j * K);
            prefix += node_keys + 1;
        }
    }
    // leaf nodes point at their first key position
    for (uint64_t j = 0; j < leaf.node_count; ++j) out->children[leaf.node_prefix + j] = j * K;

    auto key_at = [&](uint64_t idx) -> uint64_t {
        return idx >= inner_size ? col[idx - inner_size] : out->keys[idx];
    };
    // largest key below (level, node): follow the last child down to the leaves
    auto largest = [&](uint32_t level, uint64_t node) -> uint64_t {
        for (;;) {
            const level_info& ld = levels[level];
            const uint64_t node_keys = (node < ld.node_count - 1) ? K : (ld.key_count - node * K);
            if (level == depth - 1) return key_at(K * (ld.node_prefix + node) + node_keys - 1);
            node = F * node + node_keys;
            level += 1;
        }
    };
    // separators, one skipped after every K written (the parent holds it)
    for (int l = static_cast<int>(depth) - 2; l >= 0; --l) {
        const level_info& cur = levels[l];
        const level_info& low = levels[l + 1];
        const uint64_t start = cur.node_prefix * K;
        bool skipped = true;
        uint64_t written = 0;
        for (uint64_t c = 0; c + 1 < low.node_count; ++c) {
            if (!skipped && (written % K) == 0) {
                skipped = true;
                continue;
            }
            const uint64_t idx = start + written;
            if (idx >= inner_size) {
                set_error("harmonia: separator overflow at level %d", l);
                return GJ_ERR_UNSUPPORTED;
            }
            out->keys[idx] = largest(static_cast<uint32_t>(l + 1), c);
            written += 1;
            skipped = false;
        }
    }
    return GJ_OK;
}

namespace {
// orientation of (dx2, dy2) against (dx1, dy1): +1 clockwise, -1 counter-clockwise
int orientation(double dx1, double dy1, double dx2, double dy2) {
    const double e = dy1 * dx2 - dy2 * dx1;
    if (e > 2.220446049250313e-16) return 1;
    if (e < -2.220446049250313e-16) return -1;
    return 0;
}
}  // namespace

int build_radix_spline(const uint64_t* col, uint64_t n, uint32_t radix_bits, uint32_t max_error,
                       radix_spline_arrays* out) {
    if (n == 0 || radix_bits == 0 || radix_bits > 30) {
        set_error("radix spline: invalid size or radix bits");
        return GJ_ERR_INVALID_ARGUMENT;
    }
    out->min_key = col[0];
    out->max_key = col[n - 1];
    const uint64_t range = out->max_key - out->min_key;
    const unsigned used = range ? 64u - static_cast<unsigned>(__builtin_clzll(range)) : 0u;
    out->shift = used > radix_bits ? used - radix_bits : 0;
    out->table.assign((size_t(1) << radix_bits) + 2, 0);
    out->sx.clear();
    out->sy.clear();
    out->sx.reserve(n / 16 + 16);
    out->sy.reserve(n / 16 + 16);

    uint64_t prev_prefix = 0;
    auto push = [&](uint64_t x, double y) {
        const uint64_t prefix = (x - out->min_key) >> out->shift;
        if (out->sx.empty()) {
            prev_prefix = 0;
            out->table[0] = 0;
        }
        if (prefix != prev_prefix) {
            for (uint64_t p = prev_prefix + 1; p <= prefix; ++p) out->table[p] = static_cast<uint32_t>(out->sx.size());
            prev_prefix = prefix;
        }
        out->sx.push_back(x);
        out->sy.push_back(y);
    };

    const double err = static_cast<double>(max_error);
    uint64_t px = 0, ux = 0, lx = 0;
    double py = 0, uy = 0, ly = 0;
    uint64_t distinct = 0;
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t key = col[i];
        const double y = static_cast<double>(i);
        if (i == 0) {
            push(key, y);
            distinct = 1;
            px = key;
            py = y;
            continue;
        }
        if (key == px) continue;
        distinct += 1;
        const double upper_y = y + err;
        const double lower_y = err > y ? 0.0 : y - err;
        if (distinct == 2) {
            ux = lx = key;
            uy = upper_y;
            ly = lower_y;
            px = key;
            py = y;
            continue;
        }
        const uint64_t bx = out->sx.back();
        const double by = out->sy.back();
        const double udx = static_cast<double>(ux - bx), udy = uy - by;
        const double ldx = static_cast<double>(lx - bx), ldy = ly - by;
        const double dx = static_cast<double>(key - bx), dy = y - by;
        if (orientation(udx, udy, dx, dy) != 1 || orientation(ldx, ldy, dx, dy) != -1) {
            push(px, py);  // leaving the corridor: the previous point is a knot
            ux = lx = key;
            uy = upper_y;
            ly = lower_y;
        } else {
            if (orientation(udx, udy, dx, upper_y - by) == 1) {
                ux = key;
                uy = upper_y;
            }
            if (orientation(ldx, ldy, dx, lower_y - by) == -1) {
                lx = key;
                ly = lower_y;
            }
        }
        px = key;
        py = y;
    }
    if (out->sx.back() != out->max_key) push(px, py);
    for (uint64_t p = prev_prefix + 1; p < out->table.size(); ++p) out->table[p] = static_cast<uint32_t>(out->sx.size());
    return GJ_OK;
}

}  // namespace gj
