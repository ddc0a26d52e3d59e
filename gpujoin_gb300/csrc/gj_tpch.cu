// gj_tpch.cu -- TPC-H .tbl loader for the columns of Q14 and the Q14 run on
// the star-join kernel.  The loader is host code only (no GPU needed).
//
// Replaces load_tables_with_aria_parser / load_lineitem_table... /
// load_part_table... (src/tpch/common.cpp:82-220) for the columns the INLJ
// star join reads, and query_14's driver (src/tpch/tpch_14.cu).  Files are
// dbgen's: one row per line, fields separated (and the row ended) by '|'.
// lineitem: l_partkey = field 1, l_extendedprice = 5, l_discount = 6,
// l_shipdate = 10; part: p_partkey = 0, p_type = 4.
//
// Encodings: decimals as integers of their scale-2 value (21168.23 ->
// 2116823, 0.04 -> 4; the reference's numeric<12, 2>); dates as days since
// 1970-01-01 (proleptic Gregorian, the days-from-civil method of H. Hinnant;
// the reference uses Julian day numbers -- any order-preserving day count
// gives the same Q14 window).  The file is split into one chunk per host
// thread at line boundaries and parsed in parallel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "gj_internal.h"

using namespace gj;

namespace {

// days since 1970-01-01 of a proleptic Gregorian date
int64_t days_from_civil(int64_t y, unsigned m, unsigned d) {
    y -= m <= 2;
    const int64_t era = (y >= 0 ? y : y - 399) / 400;
    const unsigned yoe = (unsigned)(y - era * 400);
    const unsigned doy = (153 * (m + (m > 2 ? -3 : 9)) + 2) / 5 + d - 1;
    const unsigned doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
    return era * 146097 + (int64_t)doe - 719468;
}

struct field_cursor {
    const char* p;
    const char* end;
    // next field [b, e) of the current line; false at the line's end
    bool next(const char** b, const char** e) {
        if (p >= end || *p == '\n') return false;
        *b = p;
        while (p < end && *p != '|' && *p != '\n') ++p;
        *e = p;
        if (p < end && *p == '|') ++p;
        return true;
    }
    void skip_line() {
        while (p < end && *p != '\n') ++p;
        if (p < end) ++p;
    }
};

bool parse_uint(const char* b, const char* e, uint64_t* out) {
    if (b == e) return false;
    uint64_t v = 0;
    for (const char* c = b; c < e; ++c) {
        if (*c < '0' || *c > '9') return false;
        v = v * 10 + (uint64_t)(*c - '0');
    }
    *out = v;
    return true;
}

// a decimal with at most 2 fraction digits as its value x 100 (sign allowed)
bool parse_dec2(const char* b, const char* e, int64_t* out) {
    bool neg = false;
    if (b < e && (*b == '-' || *b == '+')) neg = *b++ == '-';
    if (b == e) return false;
    int64_t whole = 0, frac = 0;
    int digits = 0;
    const char* c = b;
    for (; c < e && *c != '.'; ++c) {
        if (*c < '0' || *c > '9') return false;
        whole = whole * 10 + (*c - '0');
    }
    if (c < e) {
        for (++c; c < e; ++c) {
            if (*c < '0' || *c > '9' || digits == 2) return false;
            frac = frac * 10 + (*c - '0');
            ++digits;
        }
    }
    while (digits < 2) frac *= 10, ++digits;
    *out = (neg ? -1 : 1) * (whole * 100 + frac);
    return true;
}

bool parse_date(const char* b, const char* e, uint32_t* out) {
    // YYYY-MM-DD
    if (e - b != 10 || b[4] != '-' || b[7] != '-') return false;
    uint64_t y, m, d;
    if (!parse_uint(b, b + 4, &y) || !parse_uint(b + 5, b + 7, &m) || !parse_uint(b + 8, b + 10, &d)) return false;
    if (m < 1 || m > 12 || d < 1 || d > 31) return false;
    const int64_t days = days_from_civil((int64_t)y, (unsigned)m, (unsigned)d);
    if (days < 0 || days > (int64_t)UINT32_MAX) return false;
    *out = (uint32_t)days;
    return true;
}

bool read_file(const char* path, std::string* out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    out->resize(size > 0 ? (size_t)size : 0);
    const size_t got = size > 0 ? std::fread(&(*out)[0], 1, (size_t)size, f) : 0;
    std::fclose(f);
    return got == out->size();
}

// line-aligned chunks of text for `parts` threads
std::vector<std::pair<size_t, size_t>> chunks(const std::string& text, unsigned parts) {
    std::vector<std::pair<size_t, size_t>> out;
    size_t begin = 0;
    for (unsigned t = 0; t < parts && begin < text.size(); ++t) {
        size_t end = t + 1 == parts ? text.size() : std::max(begin, text.size() * (t + 1) / parts);
        while (end < text.size() && text[end - 1] != '\n') ++end;
        if (end > begin) out.push_back({begin, end});
        begin = end;
    }
    return out;
}

struct lineitem_cols {
    std::vector<uint32_t> partkey, shipdate;
    std::vector<int64_t> price, discount;
    long bad_line = -1;  // first malformed line of the chunk (0-based in the chunk)
};

struct part_cols {
    std::vector<uint64_t> partkey;
    std::vector<uint8_t> promo;
    long bad_line = -1;
};

void parse_lineitem(const char* p, const char* end, lineitem_cols* out) {
    field_cursor cur{p, end};
    long line = 0;
    while (cur.p < cur.end) {
        const char *b, *e;
        uint64_t partkey = 0;
        int64_t price = 0, disc = 0;
        uint32_t ship = 0;
        bool ok = true;
        for (int f = 0; f <= 10 && ok; ++f) {
            if (!cur.next(&b, &e)) {
                ok = false;
                break;
            }
            if (f == 1) ok = parse_uint(b, e, &partkey) && partkey <= UINT32_MAX;
            else if (f == 5) ok = parse_dec2(b, e, &price);
            else if (f == 6) ok = parse_dec2(b, e, &disc);
            else if (f == 10) ok = parse_date(b, e, &ship);
        }
        if (!ok) {
            if (out->bad_line < 0) out->bad_line = line;
            return;
        }
        out->partkey.push_back((uint32_t)partkey);
        out->price.push_back(price);
        out->discount.push_back(disc);
        out->shipdate.push_back(ship);
        cur.skip_line();
        ++line;
    }
}

void parse_part(const char* p, const char* end, part_cols* out) {
    field_cursor cur{p, end};
    long line = 0;
    while (cur.p < cur.end) {
        const char *b, *e;
        uint64_t partkey = 0;
        uint8_t promo = 0;
        bool ok = true;
        for (int f = 0; f <= 4 && ok; ++f) {
            if (!cur.next(&b, &e)) {
                ok = false;
                break;
            }
            if (f == 0) ok = parse_uint(b, e, &partkey);
            else if (f == 4) promo = (e - b >= 5 && std::memcmp(b, "PROMO", 5) == 0) ? 1 : 0;  // p_type LIKE 'PROMO%'
        }
        if (!ok) {
            if (out->bad_line < 0) out->bad_line = line;
            return;
        }
        out->partkey.push_back(partkey);
        out->promo.push_back(promo);
        cur.skip_line();
        ++line;
    }
}

template <class T>
T* copy_out(const std::vector<T>& v) {
    T* p = static_cast<T*>(std::malloc(std::max<size_t>(v.size(), 1) * sizeof(T)));
    if (p && !v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

}  // namespace

extern "C" {

int gj_tpch_day(int year, int month, int day, uint32_t* out_day) {
    GJ_CHECK_ARG(out_day, "gj_tpch_day: null output");
    GJ_CHECK_ARG(month >= 1 && month <= 12 && day >= 1 && day <= 31 && year >= 1970 && year <= 9999,
                 "gj_tpch_day: date out of range");
    *out_day = (uint32_t)days_from_civil(year, (unsigned)month, (unsigned)day);
    return GJ_OK;
}

int gj_tpch_load_q14(const char* lineitem_tbl, const char* part_tbl, gj_q14_tables* out) {
    GJ_CHECK_ARG(lineitem_tbl && part_tbl && out, "gj_tpch_load_q14: null argument");
    std::memset(out, 0, sizeof(*out));
    std::string li, pa;
    if (!read_file(lineitem_tbl, &li)) {
        set_error("gj_tpch_load_q14: cannot read %s", lineitem_tbl);
        return GJ_ERR_INVALID_ARGUMENT;
    }
    if (!read_file(part_tbl, &pa)) {
        set_error("gj_tpch_load_q14: cannot read %s", part_tbl);
        return GJ_ERR_INVALID_ARGUMENT;
    }
    const unsigned threads = std::max(1u, std::thread::hardware_concurrency());
    const auto lc = chunks(li, threads);
    const auto pc = chunks(pa, threads);
    std::vector<lineitem_cols> lcols(lc.size());
    std::vector<part_cols> pcols(pc.size());
    {
        std::vector<std::thread> pool;
        for (size_t t = 0; t < lc.size(); ++t)
            pool.emplace_back(parse_lineitem, li.data() + lc[t].first, li.data() + lc[t].second, &lcols[t]);
        for (size_t t = 0; t < pc.size(); ++t)
            pool.emplace_back(parse_part, pa.data() + pc[t].first, pa.data() + pc[t].second, &pcols[t]);
        for (auto& th : pool) th.join();
    }
    lineitem_cols L;
    long line = 0;
    for (const auto& c : lcols) {
        if (c.bad_line >= 0) {
            set_error("gj_tpch_load_q14: malformed lineitem row %ld", line + c.bad_line + 1);
            return GJ_ERR_INVALID_ARGUMENT;
        }
        L.partkey.insert(L.partkey.end(), c.partkey.begin(), c.partkey.end());
        L.price.insert(L.price.end(), c.price.begin(), c.price.end());
        L.discount.insert(L.discount.end(), c.discount.begin(), c.discount.end());
        L.shipdate.insert(L.shipdate.end(), c.shipdate.begin(), c.shipdate.end());
        line += (long)c.partkey.size();
    }
    part_cols P;
    line = 0;
    for (const auto& c : pcols) {
        if (c.bad_line >= 0) {
            set_error("gj_tpch_load_q14: malformed part row %ld", line + c.bad_line + 1);
            return GJ_ERR_INVALID_ARGUMENT;
        }
        P.partkey.insert(P.partkey.end(), c.partkey.begin(), c.partkey.end());
        P.promo.insert(P.promo.end(), c.promo.begin(), c.promo.end());
        line += (long)c.partkey.size();
    }
    // the B+tree over p_partkey needs the part rows sorted by key (dbgen
    // writes them so): checked, not sorted here
    for (size_t i = 1; i < P.partkey.size(); ++i) {
        if (P.partkey[i] <= P.partkey[i - 1]) {
            set_error("gj_tpch_load_q14: part keys are not strictly increasing (row %zu)", i + 1);
            return GJ_ERR_UNSORTED;
        }
    }
    out->n_lineitem = L.partkey.size();
    out->n_part = P.partkey.size();
    out->l_partkey = copy_out(L.partkey);
    out->l_shipdate = copy_out(L.shipdate);
    out->l_extendedprice = copy_out(L.price);
    out->l_discount = copy_out(L.discount);
    out->p_partkey = copy_out(P.partkey);
    out->p_promo = copy_out(P.promo);
    if (!out->l_partkey || !out->l_shipdate || !out->l_extendedprice || !out->l_discount || !out->p_partkey ||
        !out->p_promo) {
        gj_tpch_free_q14(out);
        set_error("gj_tpch_load_q14: out of host memory");
        return GJ_ERR_OUT_OF_MEMORY;
    }
    return GJ_OK;
}

void gj_tpch_free_q14(gj_q14_tables* t) {
    if (!t) return;
    std::free(t->l_partkey);
    std::free(t->l_shipdate);
    std::free(t->l_extendedprice);
    std::free(t->l_discount);
    std::free(t->p_partkey);
    std::free(t->p_promo);
    std::memset(t, 0, sizeof(*t));
}

int gj_tpch_q14(const gj_q14_tables* t, void* stream, int64_t sums[2], double* promo_revenue) {
    GJ_CHECK_ARG(t && sums, "gj_tpch_q14: null argument");
    GJ_CHECK_ARG(t->n_part > 0, "gj_tpch_q14: no part rows");
    cudaStream_t s = as_stream(stream);
    const uint64_t nl = t->n_lineitem, np = t->n_part;
    struct buffers {
        void* p[7] = {};
        ~buffers() {
            for (void* x : p) cudaFree(x);
        }
    } b;
    const size_t bytes[7] = {np * 8, np, nl * 4, nl * 4, nl * 8, nl * 8, 16};
    for (int i = 0; i < 7; ++i) {
        if (cudaMalloc(&b.p[i], bytes[i] ? bytes[i] : 16) != cudaSuccess) {
            set_error("gj_tpch_q14: device allocation of %zu bytes failed", bytes[i]);
            return GJ_ERR_OUT_OF_MEMORY;
        }
    }
    const void* src[6] = {t->p_partkey, t->p_promo, t->l_partkey, t->l_shipdate, t->l_extendedprice, t->l_discount};
    for (int i = 0; i < 6; ++i)
        if (bytes[i]) GJ_CUDA_TRY(cudaMemcpyAsync(b.p[i], src[i], bytes[i], cudaMemcpyHostToDevice, s));
    gj_index* ix = nullptr;
    GJ_TRY(gj_index_build(GJ_INDEX_BTREE, static_cast<const uint64_t*>(b.p[0]), nullptr, np, nullptr, stream, &ix));
    uint32_t lo = 0, hi = 0;
    gj_tpch_day(1995, 9, 1, &lo);
    gj_tpch_day(1995, 10, 1, &hi);
    int rc = gj_star_join_sum(ix, static_cast<const uint32_t*>(b.p[2]), static_cast<const uint32_t*>(b.p[3]),
                              static_cast<const int64_t*>(b.p[4]), static_cast<const int64_t*>(b.p[5]), nl,
                              static_cast<const uint8_t*>(b.p[1]), lo, hi, static_cast<int64_t*>(b.p[6]), stream);
    if (rc == GJ_OK) {
        int64_t h[2] = {0, 0};
        if (cudaMemcpyAsync(h, b.p[6], sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess) {
            set_error("gj_tpch_q14: %s", cudaGetErrorString(cudaGetLastError()));
            rc = GJ_ERR_CUDA;
        } else {
            sums[0] = h[0];
            sums[1] = h[1];
            if (promo_revenue) *promo_revenue = h[1] ? 100.0 * (double)h[0] / (double)h[1] : 0.0;
        }
    }
    gj_index_free(ix);
    return rc;
}

}  // extern "C"
