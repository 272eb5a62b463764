// Dataset ingest: text log -> (train, test) partition with query-document
// parameter indices, bit-exact with the reference's Dataset::parse_dataset for
// one worker (data/dataset.cpp:421-455).
//
// Steps and the reference code they follow:
//   parse      dataset.cpp:224-305, search.cu:93-122
//   split      dataset.cpp:385-397   n_train = int(n * (1 - t) - 0.5) + 1, tail = test
//   sort       dataset.cpp:17-43     std::sort by query id (unstable; the same
//                                    libstdc++ algorithm on the same key sequence
//                                    gives the same permutation, so an index
//                                    array is sorted with the query comparator)
//   index      dataset.cpp:314-339   qd index in order of first appearance
//                                    while scanning the sorted train set
//   filter     dataset.cpp:349-374   drop a test session whose query is unseen
//                                    or none of whose docs is seen; unseen docs
//                                    keep index -1
//
// Deliberate differences on malformed input, where the reference has
// undefined behaviour or terminates: an empty line, or a field that std::stoi
// rejects inside a query or click line, is reported and skipped; a click line
// before the first query line starts an empty session whose doc ids are 0
// (the reference keeps an uninitialised one); a split that would keep more
// training sessions than exist keeps them all.
#include <algorithm>
#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "host_internal.h"

namespace mch {

// std::stoi semantics on one token: optional sign then decimal digits; stops
// at the first non-digit.  Returns false where std::stoi would throw.
static bool parse_int(const char* b, const char* e, int32_t* out) {
    const char* p = b;
    while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\v' || *p == '\f' || *p == '\r')) p++;
    bool neg = false;
    if (p < e && (*p == '+' || *p == '-')) { neg = (*p == '-'); p++; }
    if (p >= e || *p < '0' || *p > '9') return false;
    long long v = 0;
    while (p < e && *p >= '0' && *p <= '9') {
        v = v * 10 + (*p - '0');
        if (v > 2147483648LL) return false;
        p++;
    }
    v = neg ? -v : v;
    if (v > INT_MAX || v < INT_MIN) return false;
    *out = (int32_t)v;
    return true;
}

struct RawSession {
    int32_t query = -1;
    int32_t docs[MC_MAX_SERP] = {0};
    uint16_t click = 0;
};

// Number of training sessions kept by the split (dataset.cpp:390): the
// product is formed in float (int * float), the 0.5 subtracted in double.
static int64_t train_count(int64_t n, float test_share) {
    float prod = (float)n * (1.0f - test_share);
    int64_t n_train = (int64_t)((double)prod - 0.5) + 1;
    if (n_train > n) n_train = n;
    if (n_train < 0) n_train = 0;
    return n_train;
}

// Builds the partition from sessions in arrival order.
static void build_partition(const std::vector<int32_t>& query, const std::vector<int32_t>& docs,
                            const std::vector<uint16_t>& click, float test_share, mc_dataset* d) {
    int64_t n = (int64_t)query.size();
    int64_t n_train = train_count(n, test_share);
    int64_t n_test = n - n_train;

    // Sort the training sessions by query with the reference's comparator.
    std::vector<int32_t> order((size_t)n_train);
    std::iota(order.begin(), order.end(), 0);
    const int32_t* q = query.data();
    std::sort(order.begin(), order.end(), [q](int32_t a, int32_t b) { return q[a] < q[b]; });

    SessionSet& tr = d->train;
    tr.query.resize((size_t)n_train);
    tr.docs.resize((size_t)n_train * MC_MAX_SERP);
    tr.pidx.assign((size_t)n_train * MC_MAX_SERP, -1);
    tr.click.resize((size_t)n_train);
    for (int64_t i = 0; i < n_train; i++) {
        int32_t src = order[(size_t)i];
        tr.query[(size_t)i] = query[(size_t)src];
        std::memcpy(&tr.docs[(size_t)i * MC_MAX_SERP], &docs[(size_t)src * MC_MAX_SERP], MC_MAX_SERP * sizeof(int32_t));
        tr.click[(size_t)i] = click[(size_t)src];
    }

    // Query segments of the sorted training set.
    std::vector<int64_t> seg_begin;
    for (int64_t i = 0; i < n_train; i++)
        if (i == 0 || tr.query[(size_t)i] != tr.query[(size_t)i - 1]) seg_begin.push_back(i);
    size_t n_seg = seg_begin.size();
    seg_begin.push_back(n_train);

    // Per segment: distinct docs in order of first appearance get local
    // indices 0..k-1; the lookup table keeps (doc, local index) sorted by doc.
    std::vector<int64_t> seg_ndocs(n_seg, 0);
    std::vector<std::vector<std::pair<int32_t, int32_t>>> seg_lookup(n_seg);
    auto index_segment = [&](size_t s) {
        int64_t b = seg_begin[s], e = seg_begin[s + 1];
        size_t m = (size_t)(e - b) * MC_MAX_SERP;
        std::vector<uint64_t> keys(m);
        for (size_t k = 0; k < m; k++) {
            uint32_t doc = (uint32_t)tr.docs[(size_t)b * MC_MAX_SERP + k];
            keys[k] = ((uint64_t)(doc ^ 0x80000000u) << 32) | (uint64_t)k;  // signed doc order
        }
        std::sort(keys.begin(), keys.end());
        // Groups of equal doc: first element carries the first appearance.
        std::vector<std::pair<uint32_t, uint32_t>> firsts;  // (first position, group start)
        for (size_t k = 0; k < m; k++)
            if (k == 0 || (keys[k] >> 32) != (keys[k - 1] >> 32)) firsts.push_back({(uint32_t)(keys[k] & 0xffffffffu), (uint32_t)k});
        std::vector<uint32_t> by_first(firsts.size());
        std::iota(by_first.begin(), by_first.end(), 0);
        std::sort(by_first.begin(), by_first.end(), [&](uint32_t x, uint32_t y) { return firsts[x].first < firsts[y].first; });
        std::vector<int32_t> local(firsts.size());
        for (size_t r = 0; r < by_first.size(); r++) local[by_first[r]] = (int32_t)r;
        auto& lk = seg_lookup[s];
        lk.resize(firsts.size());
        for (size_t g = 0; g < firsts.size(); g++) {
            size_t k0 = firsts[g].second, k1 = (g + 1 < firsts.size()) ? firsts[g + 1].second : m;
            int32_t doc = (int32_t)((uint32_t)(keys[k0] >> 32) ^ 0x80000000u);
            lk[g] = {doc, local[g]};
            for (size_t k = k0; k < k1; k++)
                tr.pidx[(size_t)b * MC_MAX_SERP + (keys[k] & 0xffffffffu)] = local[g];
        }
        seg_ndocs[s] = (int64_t)firsts.size();
    };
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    size_t n_threads = std::min<size_t>(hw, std::max<size_t>(1, n_seg / 64));
    {
        std::vector<std::thread> pool;
        for (size_t t = 0; t < n_threads; t++)
            pool.emplace_back([&, t]() { for (size_t s = t; s < n_seg; s += n_threads) index_segment(s); });
        for (auto& th : pool) th.join();
    }
    std::vector<int64_t> seg_base(n_seg + 1, 0);
    for (size_t s = 0; s < n_seg; s++) seg_base[s + 1] = seg_base[s] + seg_ndocs[s];
    {
        std::vector<std::thread> pool;
        for (size_t t = 0; t < n_threads; t++)
            pool.emplace_back([&, t]() {
                for (size_t s = t; s < n_seg; s += n_threads) {
                    int32_t base = (int32_t)seg_base[s];
                    for (int64_t k = seg_begin[s] * MC_MAX_SERP; k < seg_begin[s + 1] * MC_MAX_SERP; k++)
                        tr.pidx[(size_t)k] += base;
                }
            });
        for (auto& th : pool) th.join();
    }
    d->n_qd = seg_base[n_seg];

    // Test set: the tail in arrival order, filtered.
    SessionSet& te = d->test;
    for (int64_t i = n_train; i < n; i++) {
        int32_t qi = query[(size_t)i];
        size_t lo = 0, hi = n_seg;
        while (lo < hi) {  // first segment with query >= qi
            size_t mid = (lo + hi) / 2;
            if (tr.query[(size_t)seg_begin[mid]] < qi) lo = mid + 1; else hi = mid;
        }
        if (lo == n_seg || tr.query[(size_t)seg_begin[lo]] != qi) continue;
        const auto& lk = seg_lookup[lo];
        int32_t p[MC_MAX_SERP];
        bool any = false;
        for (int r = 0; r < MC_MAX_SERP; r++) {
            int32_t doc = docs[(size_t)i * MC_MAX_SERP + r];
            auto it = std::lower_bound(lk.begin(), lk.end(), std::make_pair(doc, INT_MIN));
            if (it != lk.end() && it->first == doc) { p[r] = (int32_t)seg_base[lo] + it->second; any = true; }
            else p[r] = -1;
        }
        if (!any) continue;
        te.query.push_back(qi);
        for (int r = 0; r < MC_MAX_SERP; r++) {
            te.docs.push_back(docs[(size_t)i * MC_MAX_SERP + r]);
            te.pidx.push_back(p[r]);
        }
        te.click.push_back(click[(size_t)i]);
    }
    (void)n_test;
}

static void tokenize(const std::string& line, std::vector<std::pair<const char*, const char*>>& tok) {
    tok.clear();
    const char* p = line.data();
    const char* e = p + line.size();
    while (p < e) {
        while (p < e && std::isspace((unsigned char)*p)) p++;
        if (p >= e) break;
        const char* s = p;
        while (p < e && !std::isspace((unsigned char)*p)) p++;
        tok.push_back({s, p});
    }
}

}  // namespace mch

using namespace mch;

extern "C" int mc_dataset_parse(const char* path, int32_t max_sessions, float test_share, mc_dataset** out) {
    if (!path || !out) return set_error(MC_ERR_INVALID, "dataset_parse: null argument");
    *out = nullptr;
    if (!(test_share >= 0.0f && test_share <= 1.0f))
        return set_error(MC_ERR_INVALID, "dataset_parse: test_share must be in [0, 1]");
    std::ifstream f(path);
    if (!f.is_open()) return set_error(MC_ERR_IO, std::string("Unable to open the raw dataset: ") + path);

    std::vector<int32_t> query, docs;
    std::vector<uint16_t> click;
    std::string line;
    std::vector<std::pair<const char*, const char*>> tok;
    RawSession cur;
    int64_t n_queries = 0;
    long long session_prev = -1;
    bool have_prev = false;
    while ((n_queries < max_sessions || max_sessions == -1) && std::getline(f, line)) {
        tokenize(line, tok);
        int32_t sid;
        if (tok.empty() || !parse_int(tok[0].first, tok[0].second, &sid)) {
            std::cout << "\nInvalid data: " << line << std::endl;
            continue;
        }
        if (tok.size() == 15) {
            RawSession next;
            bool ok = parse_int(tok[3].first, tok[3].second, &next.query);
            for (int r = 0; r < MC_MAX_SERP && ok; r++) ok = parse_int(tok[5 + r].first, tok[5 + r].second, &next.docs[r]);
            if (!ok) { std::cout << "\nInvalid data: " << line << std::endl; continue; }
            if (have_prev && session_prev != -1) {
                query.push_back(cur.query);
                docs.insert(docs.end(), cur.docs, cur.docs + MC_MAX_SERP);
                click.push_back(cur.click);
                n_queries++;
            }
            cur = next;
        } else if (tok.size() == 4) {
            int32_t doc;
            if (!parse_int(tok[3].first, tok[3].second, &doc)) { std::cout << "\nInvalid data: " << line << std::endl; continue; }
            for (int r = 0; r < MC_MAX_SERP; r++)
                if (cur.docs[r] == doc) { cur.click |= (uint16_t)(1u << r); break; }
        } else {
            std::cout << "\nInvalid data: " << line << std::endl;
        }
        session_prev = sid;
        have_prev = true;
    }
    mc_dataset* d = new (std::nothrow) mc_dataset();
    if (!d) return set_error(MC_ERR_NOMEM, "dataset_parse: out of host memory");
    build_partition(query, docs, click, test_share, d);
    *out = d;
    return MC_OK;
}

extern "C" int mc_dataset_from_sessions(int64_t n, const int32_t* query, const int32_t* docs,
                                        const uint16_t* click_mask, float test_share, mc_dataset** out) {
    if (!out) return set_error(MC_ERR_INVALID, "dataset_from_sessions: null output");
    *out = nullptr;
    if (n < 0 || n > INT_MAX) return set_error(MC_ERR_INVALID, "dataset_from_sessions: n out of range");
    if (n > 0 && (!query || !docs || !click_mask)) return set_error(MC_ERR_INVALID, "dataset_from_sessions: null input");
    if (!(test_share >= 0.0f && test_share <= 1.0f))
        return set_error(MC_ERR_INVALID, "dataset_from_sessions: test_share must be in [0, 1]");
    std::vector<int32_t> q(query, query + n), dd(docs, docs + n * MC_MAX_SERP);
    std::vector<uint16_t> c(click_mask, click_mask + n);
    mc_dataset* d = new (std::nothrow) mc_dataset();
    if (!d) return set_error(MC_ERR_NOMEM, "dataset_from_sessions: out of host memory");
    build_partition(q, dd, c, test_share, d);
    *out = d;
    return MC_OK;
}

extern "C" int mc_dataset_info(const mc_dataset* d, int64_t* n_train, int64_t* n_test, int64_t* n_qd) {
    if (!d) return set_error(MC_ERR_INVALID, "dataset_info: null dataset");
    if (n_train) *n_train = d->train.size();
    if (n_test) *n_test = d->test.size();
    if (n_qd) *n_qd = d->n_qd;
    return MC_OK;
}

extern "C" int mc_dataset_copy(const mc_dataset* d, int which, int32_t* query, int32_t* docs,
                               int32_t* pidx, uint16_t* click_mask) {
    if (!d) return set_error(MC_ERR_INVALID, "dataset_copy: null dataset");
    if (which != 0 && which != 1) return set_error(MC_ERR_INVALID, "dataset_copy: which must be 0 (train) or 1 (test)");
    const SessionSet& s = which == 0 ? d->train : d->test;
    if (query) std::copy(s.query.begin(), s.query.end(), query);
    if (docs) std::copy(s.docs.begin(), s.docs.end(), docs);
    if (pidx) std::copy(s.pidx.begin(), s.pidx.end(), pidx);
    if (click_mask) std::copy(s.click.begin(), s.click.end(), click_mask);
    return MC_OK;
}

extern "C" void mc_dataset_free(mc_dataset* d) { delete d; }
