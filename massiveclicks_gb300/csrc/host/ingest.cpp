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
#include <atomic>
#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <future>
#include <iostream>
#include <memory>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "host_internal.h"
#include "pool.h"

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

// Builds the partition from n sessions in arrival order (query[n],
// docs[n * 10], click[n]).
static void build_partition(int64_t n, const int32_t* query, const int32_t* docs, const uint16_t* click,
                            float test_share, mc_dataset* d) {
    int64_t n_train = train_count(n, test_share);
    int64_t n_test = n - n_train;

    // Sort the training sessions by query with the reference's comparator.
    // The elements are (query, index) pairs compared by query alone: std::sort
    // then makes the same comparisons with the same outcomes and the same
    // moves as on the sessions themselves, so it leaves the indices in the
    // reference's (unstable) order, without a random load per comparison.
    struct KV {
        int32_t first, second;  // query, session index
    };
    RawVec<KV> kv((size_t)n_train);
    const int64_t kFill = 1 << 20;
    parallel_for((size_t)((n_train + kFill - 1) / kFill), [&](size_t c) {
        const int64_t i1 = std::min<int64_t>(n_train, (int64_t)(c + 1) * kFill);
        for (int64_t i = (int64_t)c * kFill; i < i1; i++) kv[(size_t)i] = KV{query[i], (int32_t)i};
    });
    std::sort(kv.begin(), kv.end(), [](const KV& a, const KV& b) { return a.first < b.first; });
    SessionSet& tr = d->train;
    tr.query.resize((size_t)n_train);
    tr.docs.resize((size_t)n_train * MC_MAX_SERP);
    tr.pidx.resize((size_t)n_train * MC_MAX_SERP);  // every entry is written by the indexing below
    tr.click.resize((size_t)n_train);
    const int64_t kGather = 65536;
    parallel_for((size_t)((n_train + kGather - 1) / kGather), [&](size_t c) {
        const int64_t i1 = std::min<int64_t>(n_train, (int64_t)(c + 1) * kGather);
        for (int64_t i = (int64_t)c * kGather; i < i1; i++) {
            const int64_t src = kv[(size_t)i].second;
            tr.query[(size_t)i] = query[src];
            std::memcpy(&tr.docs[(size_t)i * MC_MAX_SERP], &docs[src * MC_MAX_SERP], MC_MAX_SERP * sizeof(int32_t));
            tr.click[(size_t)i] = click[src];
        }
    });
    RawVec<KV>().swap(kv);

    // Query segments of the sorted training set.
    std::vector<int64_t> seg_begin;
    for (int64_t i = 0; i < n_train; i++)
        if (i == 0 || tr.query[(size_t)i] != tr.query[(size_t)i - 1]) seg_begin.push_back(i);
    size_t n_seg = seg_begin.size();
    seg_begin.push_back(n_train);

    // Per segment: distinct docs in order of first appearance get local
    // indices 0..k-1 (one scan with an open-addressing table of doc -> local
    // index); the lookup table keeps (doc, local index) sorted by doc.
    std::vector<int64_t> seg_ndocs(n_seg, 0);
    std::vector<std::vector<std::pair<int32_t, int32_t>>> seg_lookup(n_seg);
    struct Scratch {
        std::vector<int32_t> slot_doc, slot_local;  // slot_local -1 = empty
    };
    auto index_segment = [&](size_t s, Scratch& sc) {
        const int64_t b = seg_begin[s], e = seg_begin[s + 1];
        const size_t m = (size_t)(e - b) * MC_MAX_SERP;
        // The table starts small and doubles when half full (rehashed from
        // lk, which holds every (doc, local index) so far): a query's
        // distinct docs are few even when its sessions are many.
        size_t cap = 64;
        auto clear_table = [&]() {
            if (sc.slot_doc.size() < cap) {
                sc.slot_doc.resize(cap);
                sc.slot_local.resize(cap);
            }
            std::fill(sc.slot_local.begin(), sc.slot_local.begin() + (long)cap, -1);
        };
        clear_table();
        uint32_t mask = (uint32_t)cap - 1;
        auto& lk = seg_lookup[s];
        lk.clear();
        auto slot_of = [&](int32_t doc) {
            uint32_t h = ((uint32_t)doc * 0x9E3779B1u) & mask;
            while (sc.slot_local[h] >= 0 && sc.slot_doc[h] != doc) h = (h + 1) & mask;
            return h;
        };
        int32_t* const pidx = &tr.pidx[(size_t)b * MC_MAX_SERP];
        const int32_t* const dk = &tr.docs[(size_t)b * MC_MAX_SERP];
        for (size_t k = 0; k < m; k++) {
            const int32_t doc = dk[k];
            uint32_t h = slot_of(doc);
            if (sc.slot_local[h] < 0) {
                if (2 * (lk.size() + 1) > cap) {
                    cap *= 2;
                    mask = (uint32_t)cap - 1;
                    clear_table();
                    for (const auto& kv2 : lk) {
                        const uint32_t h2 = slot_of(kv2.first);
                        sc.slot_doc[h2] = kv2.first;
                        sc.slot_local[h2] = kv2.second;
                    }
                    h = slot_of(doc);
                }
                sc.slot_doc[h] = doc;
                sc.slot_local[h] = (int32_t)lk.size();
                lk.push_back({doc, (int32_t)lk.size()});
            }
            pidx[k] = sc.slot_local[h];
        }
        seg_ndocs[s] = (int64_t)lk.size();
        std::sort(lk.begin(), lk.end());
    };
    // Segments in tasks of 64, taken dynamically: one head query can hold a
    // large share of all sessions.
    const size_t kSegTask = 64;
    parallel_for((n_seg + kSegTask - 1) / kSegTask, [&](size_t c) {
        Scratch sc;  // per task: its tables grow to the task's largest segment
        const size_t s1 = std::min(n_seg, (c + 1) * kSegTask);
        for (size_t s = c * kSegTask; s < s1; s++) index_segment(s, sc);
    });
    std::vector<int64_t> seg_base(n_seg + 1, 0);
    for (size_t s = 0; s < n_seg; s++) seg_base[s + 1] = seg_base[s] + seg_ndocs[s];
    parallel_for((n_seg + kSegTask - 1) / kSegTask, [&](size_t c) {
        const size_t s1 = std::min(n_seg, (c + 1) * kSegTask);
        for (size_t s = c * kSegTask; s < s1; s++) {
            const int32_t base = (int32_t)seg_base[s];
            for (int64_t k = seg_begin[s] * MC_MAX_SERP; k < seg_begin[s + 1] * MC_MAX_SERP; k++)
                tr.pidx[(size_t)k] += base;
        }
    });
    d->n_qd = seg_base[n_seg];

    // Test set: the tail in arrival order, filtered; contiguous ranges on
    // several threads, joined in order.  The segments' queries, in one small
    // array, are binary-searched per test session.
    std::vector<int32_t> seg_query(n_seg);
    for (size_t g = 0; g < n_seg; g++) seg_query[g] = tr.query[(size_t)seg_begin[g]];
    auto filter_range = [&](int64_t i0, int64_t i1, SessionSet& out) {
        out.query.reserve((size_t)(i1 - i0));
        out.docs.reserve((size_t)(i1 - i0) * MC_MAX_SERP);
        out.pidx.reserve((size_t)(i1 - i0) * MC_MAX_SERP);
        out.click.reserve((size_t)(i1 - i0));
        for (int64_t i = i0; i < i1; i++) {
            const int32_t qi = query[i];
            const size_t lo = (size_t)(std::lower_bound(seg_query.begin(), seg_query.end(), qi) - seg_query.begin());
            if (lo == n_seg || seg_query[lo] != qi) continue;
            const auto& lk = seg_lookup[lo];
            int32_t p[MC_MAX_SERP];
            bool any = false;
            for (int r = 0; r < MC_MAX_SERP; r++) {
                int32_t doc = docs[i * MC_MAX_SERP + r];
                auto it = std::lower_bound(lk.begin(), lk.end(), std::make_pair(doc, INT_MIN));
                if (it != lk.end() && it->first == doc) { p[r] = (int32_t)seg_base[lo] + it->second; any = true; }
                else p[r] = -1;
            }
            if (!any) continue;
            out.query.push_back(qi);
            for (int r = 0; r < MC_MAX_SERP; r++) {
                out.docs.push_back(docs[i * MC_MAX_SERP + r]);
                out.pidx.push_back(p[r]);
            }
            out.click.push_back(click[i]);
        }
    };
    const int64_t kTestPart = 16384;
    const int64_t n_tparts = std::max<int64_t>(1, (n_test + kTestPart - 1) / kTestPart);
    std::vector<SessionSet> tparts((size_t)n_tparts);
    parallel_for((size_t)n_tparts, [&](size_t t) {
        filter_range(n_train + (int64_t)t * kTestPart, std::min<int64_t>(n, n_train + ((int64_t)t + 1) * kTestPart),
                     tparts[t]);
    });
    SessionSet& te = d->test;
    std::vector<size_t> at(tparts.size() + 1, 0);
    for (size_t t = 0; t < tparts.size(); t++) at[t + 1] = at[t] + tparts[t].query.size();
    te.query.resize(at.back());
    te.docs.resize(at.back() * MC_MAX_SERP);
    te.pidx.resize(at.back() * MC_MAX_SERP);
    te.click.resize(at.back());
    parallel_for(tparts.size(), [&](size_t t) {
        const SessionSet& part = tparts[t];
        std::copy(part.query.begin(), part.query.end(), te.query.begin() + (long)at[t]);
        std::copy(part.docs.begin(), part.docs.end(), te.docs.begin() + (long)(at[t] * MC_MAX_SERP));
        std::copy(part.pidx.begin(), part.pidx.end(), te.pidx.begin() + (long)(at[t] * MC_MAX_SERP));
        std::copy(part.click.begin(), part.click.end(), te.click.begin() + (long)at[t]);
    });
    (void)n_test;
}

// One parsed line.  kind: 1 query line (15 tokens), 2 click line (4 tokens),
// 3 other token count (reported, but its session id still becomes the last
// one seen), 0 rejected (bad session id or field: reported, no state change).
struct ParsedLine {
    const char* b;  // the line's text, for the report
    const char* e;
    int32_t sid;
    int32_t query;
    int32_t v[MC_MAX_SERP];  // query line: docs; click line: v[0] = doc
    uint8_t kind;
};

// The six characters std::isspace accepts in the "C" locale, as a table
// indexed by the byte (one load per character instead of six compares).
struct SpaceTable {
    bool t[256] = {};
    SpaceTable() {
        for (unsigned char c : {' ', '\t', '\n', '\v', '\f', '\r'}) t[c] = true;
    }
};
static const SpaceTable kSpace;
static inline bool is_space(char c) { return kSpace.t[(unsigned char)c]; }

// Tokens as the reference's std::istringstream >> splits them (whitespace).
static ParsedLine parse_line(const char* b, const char* e) {
    ParsedLine pl;
    pl.b = b;
    pl.e = e;
    pl.kind = 0;
    pl.sid = 0;
    pl.query = 0;
    const char* tb[16];
    const char* te[16];
    int nt = 0;
    const char* p = b;
    while (p < e) {
        while (p < e && is_space(*p)) p++;
        if (p >= e) break;
        const char* s0 = p;
        while (p < e && !is_space(*p)) p++;
        if (nt < 16) { tb[nt] = s0; te[nt] = p; }
        nt++;
    }
    if (nt == 0 || !parse_int(tb[0], te[0], &pl.sid)) return pl;
    if (nt == 15) {
        bool ok = parse_int(tb[3], te[3], &pl.query);
        for (int r = 0; r < MC_MAX_SERP && ok; r++) ok = parse_int(tb[5 + r], te[5 + r], &pl.v[r]);
        if (ok) pl.kind = 1;
    } else if (nt == 4) {
        if (parse_int(tb[3], te[3], &pl.v[0])) pl.kind = 2;
    } else {
        pl.kind = 3;
    }
    return pl;
}

// One contiguous run of lines replayed on its own.  Everything a line needs
// from the lines before the run -- the open session and the last session id
// -- is recorded at the run's boundary and settled when the runs are joined
// in order (join_part); the sessions the run both opens and closes are
// complete here.
struct PartReplay {
    int64_t n_lines = 0;
    // Before the first query line: click docs for the incoming open session,
    // and the session id of the last non-rejected line, if any.
    std::vector<int32_t> prefix_clicks;
    bool prefix_sid = false;
    int32_t prefix_last_sid = 0;
    int64_t first_query = -1;  // line index of the first query line, -1 if none
    // Sessions opened and closed in the run, in order, and the index of the
    // query line that closed each (a query line closes the open session when
    // the previous non-rejected line's session id is not -1).
    std::vector<int32_t> q, d;
    std::vector<uint16_t> c;
    std::vector<int64_t> closed_at;
    RawSession open;               // opened by the last query line
    bool any_sid = false;          // a non-rejected line in the run
    int32_t last_sid = 0;          // the last one's session id
    std::vector<std::pair<int64_t, std::string>> invalid;  // reported lines
};

static void replay_part(const char* base, size_t p, size_t e, PartReplay& out) {
    out = PartReplay();
    bool seen_query = false;
    RawSession cur;
    int64_t li = 0;
    while (p < e) {
        const char* nl = static_cast<const char*>(std::memchr(base + p, '\n', e - p));
        const size_t q = nl ? (size_t)(nl - base) : e;
        const ParsedLine pl = parse_line(base + p, base + q);
        if (pl.kind == 0 || pl.kind == 3) out.invalid.push_back({li, std::string(pl.b, pl.e)});
        if (pl.kind != 0) {
            if (pl.kind == 1) {
                if (!seen_query) {
                    out.first_query = li;  // whether it closes the incoming session is settled at the join
                    seen_query = true;
                } else if (out.last_sid != -1) {
                    out.q.push_back(cur.query);
                    out.d.insert(out.d.end(), cur.docs, cur.docs + MC_MAX_SERP);
                    out.c.push_back(cur.click);
                    out.closed_at.push_back(li);
                }
                cur = RawSession();
                cur.query = pl.query;
                std::memcpy(cur.docs, pl.v, sizeof(cur.docs));
            } else if (pl.kind == 2) {
                if (!seen_query) out.prefix_clicks.push_back(pl.v[0]);
                else
                    for (int r = 0; r < MC_MAX_SERP; r++)
                        if (cur.docs[r] == pl.v[0]) { cur.click |= (uint16_t)(1u << r); break; }
            }
            if (!seen_query) {
                out.prefix_sid = true;
                out.prefix_last_sid = pl.sid;
            }
            out.any_sid = true;
            out.last_sid = pl.sid;
        }
        li++;
        p = q + 1;
    }
    out.open = cur;
    out.n_lines = li;
}

}  // namespace mch

using namespace mch;

// Read size and run count of mc_dataset_parse; 0 = the defaults (64 MB
// blocks, one run of lines per hardware thread).
static std::atomic<int64_t> g_block_bytes{0};
static std::atomic<int32_t> g_parse_runs{0};

extern "C" int mc_ingest_configure(int64_t block_bytes, int32_t runs) {
    if (block_bytes < 0 || runs < 0) return set_error(MC_ERR_INVALID, "ingest_configure: negative size");
    g_block_bytes.store(block_bytes);
    g_parse_runs.store(runs);
    return MC_OK;
}

// The text log is read in blocks; the lines of a block are parsed by several
// threads (each a contiguous run of lines) and then replayed in order through
// the reference's session state machine (dataset.cpp:224-305): the session
// count is checked before every line, a query line closes the open session
// when a previous line set a session id other than -1, a click line marks the
// first matching doc, and the open session at the stop is dropped.
extern "C" int mc_dataset_parse(const char* path, int32_t max_sessions, float test_share, mc_dataset** out) {
    if (!path || !out) return set_error(MC_ERR_INVALID, "dataset_parse: null argument");
    *out = nullptr;
    if (!(test_share >= 0.0f && test_share <= 1.0f))
        return set_error(MC_ERR_INVALID, "dataset_parse: test_share must be in [0, 1]");
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_error(MC_ERR_IO, std::string("Unable to open the raw dataset: ") + path);

    // Sessions kept, in order, as a list of chunks: a run's own sessions are
    // moved in whole, boundary sessions appended one by one to a tail chunk;
    // the chunks are concatenated once at the end.
    struct Chunk {
        std::vector<int32_t> q, d;
        std::vector<uint16_t> c;
        bool whole = false;  // a run's sessions (no appends)
    };
    std::vector<Chunk> chunks;
    RawSession cur;
    int64_t n_queries = 0;
    long long session_prev = -1;
    bool have_prev = false;
    bool done = false;

    const size_t kBlock = g_block_bytes.load() > 0 ? (size_t)g_block_bytes.load() : (size_t)64 << 20;
    const unsigned n_threads = g_parse_runs.load() > 0 ? (unsigned)g_parse_runs.load()
                                                       : std::max(1u, std::thread::hardware_concurrency());
    // Blocks are read into two buffers (left uninitialised: no zero fill of
    // 64 MB per block): the next block is read on another thread while the
    // current one is parsed and replayed.
    struct Block {
        std::unique_ptr<char[]> data;
        size_t cap = 0, size = 0;
        bool eof = false;
    };
    Block blocks[2];
    auto read_block = [&](Block& b, const std::string& carry) {
        const size_t need = carry.size() + kBlock;
        if (b.cap < need) {
            b.data.reset(new char[need]);
            b.cap = need;
        }
        std::memcpy(b.data.get(), carry.data(), carry.size());
        const size_t got = std::fread(b.data.get() + carry.size(), 1, kBlock, f);
        b.size = carry.size() + got;
        b.eof = got < kBlock;
    };
    std::string carry;  // the unfinished last line of the previous block
    std::vector<PartReplay> parts(n_threads);
    // Joins a replayed run to the state of the lines before it, in order: the
    // session count is checked before every line (it changes only at query
    // lines, so the stop falls on the line after the closing query line that
    // reached the limit), reported lines are printed up to the stop, and the
    // run's boundary facts are applied to the open session.
    const auto limit_reached = [&]() { return !(n_queries < max_sessions || max_sessions == -1); };
    auto push = [&](int32_t q, const int32_t* dd, uint16_t c) {
        if (chunks.empty() || chunks.back().whole) chunks.emplace_back();
        Chunk& t = chunks.back();
        t.q.push_back(q);
        t.d.insert(t.d.end(), dd, dd + MC_MAX_SERP);
        t.c.push_back(c);
        n_queries++;
    };
    auto report = [&](const PartReplay& P, int64_t upto) {  // lines with index < upto
        for (const auto& m : P.invalid)
            if (m.first < upto) std::cout << "\nInvalid data: " << m.second << std::endl;
    };
    auto join_part = [&](PartReplay& P) {
        if (P.n_lines == 0) return;
        if (limit_reached()) { done = true; return; }  // stops before the run's first line
        // The prefix: clicks on the incoming open session.
        for (int32_t doc : P.prefix_clicks)
            for (int r = 0; r < MC_MAX_SERP; r++)
                if (cur.docs[r] == doc) { cur.click |= (uint16_t)(1u << r); break; }
        if (P.prefix_sid) {
            session_prev = P.prefix_last_sid;
            have_prev = true;
        }
        if (P.first_query < 0) {  // no query line: the prefix is the whole run
            report(P, P.n_lines);
            return;
        }
        // The first query line closes the incoming session, then the run's own.
        if (have_prev && session_prev != -1) {
            push(cur.query, cur.docs, cur.click);
            if (limit_reached() && P.first_query + 1 < P.n_lines) {
                report(P, P.first_query + 1);
                done = true;
                return;
            }
        }
        const size_t n_closed = P.closed_at.size();
        if (max_sessions == -1 || n_queries + (int64_t)n_closed < (int64_t)max_sessions) {
            // The limit cannot fall inside the run: its sessions in one move.
            if (n_closed) {
                chunks.emplace_back();
                Chunk& t = chunks.back();
                t.q = std::move(P.q);
                t.d = std::move(P.d);
                t.c = std::move(P.c);
                t.whole = true;
            }
            n_queries += (int64_t)n_closed;
        } else for (size_t k = 0; k < n_closed; k++) {
            push(P.q[k], &P.d[k * MC_MAX_SERP], P.c[k]);
            if (limit_reached() && P.closed_at[k] + 1 < P.n_lines) {
                report(P, P.closed_at[k] + 1);
                done = true;
                return;
            }
        }
        report(P, P.n_lines);
        cur = P.open;
        session_prev = P.last_sid;
        have_prev = true;
    };
    int cur_b = 0;
    read_block(blocks[0], carry);
    std::future<void> pending;
    bool eof = false;
    while (!done && !eof) {
        if (pending.valid()) pending.get();  // blocks[cur_b] is read
        Block& blk = blocks[cur_b];
        eof = blk.eof;
        const char* const bufp = blk.data.get();
        // Complete lines of this block: up to the last newline (all of it at EOF).
        size_t end = blk.size;
        if (!eof) {
            size_t nl = end;
            while (nl > 0 && bufp[nl - 1] != '\n') nl--;
            if (nl == 0) {  // a line longer than the block: keep reading
                carry.assign(bufp, bufp + blk.size);
                read_block(blk, carry);
                continue;
            }
            end = nl;
        }
        carry.assign(bufp + end, bufp + blk.size);
        if (!eof) {
            Block& next = blocks[cur_b ^ 1];
            const std::string next_carry = carry;
            pending = std::async(std::launch::async, [&read_block, &next, next_carry]() { read_block(next, next_carry); });
        }
        if (end == 0) break;
        const char* base = bufp;
        // Thread ranges start at line boundaries.
        std::vector<size_t> cut(n_threads + 1, end);
        cut[0] = 0;
        for (unsigned t = 1; t < n_threads; t++) {
            size_t c = std::max(cut[t - 1], end * t / n_threads);
            while (c < end && c > 0 && base[c - 1] != '\n') c++;
            cut[t] = c;
        }
        parallel_for(n_threads, [&](size_t t) { replay_part(base, cut[t], cut[t + 1], parts[t]); });
        for (unsigned t = 0; t < n_threads && !done; t++) join_part(parts[t]);
        cur_b ^= 1;  // the next block (being read) becomes current
    }
    if (pending.valid()) pending.get();  // a read still in flight when the session limit stopped us
    std::fclose(f);
    mc_dataset* d = new (std::nothrow) mc_dataset();
    if (!d) return set_error(MC_ERR_NOMEM, "dataset_parse: out of host memory");
    std::vector<size_t> at(chunks.size() + 1, 0);
    for (size_t k = 0; k < chunks.size(); k++) at[k + 1] = at[k] + chunks[k].q.size();
    RawVec<int32_t> query(at.back()), docs(at.back() * MC_MAX_SERP);
    RawVec<uint16_t> click(at.back());
    parallel_for(chunks.size(), [&](size_t k) {
        const Chunk& t = chunks[k];
        std::copy(t.q.begin(), t.q.end(), query.begin() + (long)at[k]);
        std::copy(t.d.begin(), t.d.end(), docs.begin() + (long)(at[k] * MC_MAX_SERP));
        std::copy(t.c.begin(), t.c.end(), click.begin() + (long)at[k]);
    });
    std::vector<Chunk>().swap(chunks);
    build_partition((int64_t)query.size(), query.data(), docs.data(), click.data(), test_share, d);
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
    mc_dataset* d = new (std::nothrow) mc_dataset();
    if (!d) return set_error(MC_ERR_NOMEM, "dataset_from_sessions: out of host memory");
    build_partition(n, query, docs, click_mask, test_share, d);  // reads the caller's arrays
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
    // In chunks on the host threads (the caller's fresh arrays are first
    // touched in parallel too).
    const int64_t n = s.size(), kCopy = 1 << 18;
    parallel_for((size_t)((n + kCopy - 1) / kCopy), [&](size_t c) {
        const int64_t i0 = (int64_t)c * kCopy, i1 = std::min<int64_t>(n, i0 + kCopy);
        if (query) std::copy(s.query.begin() + i0, s.query.begin() + i1, query + i0);
        if (docs) std::copy(s.docs.begin() + i0 * MC_MAX_SERP, s.docs.begin() + i1 * MC_MAX_SERP, docs + i0 * MC_MAX_SERP);
        if (pidx) std::copy(s.pidx.begin() + i0 * MC_MAX_SERP, s.pidx.begin() + i1 * MC_MAX_SERP, pidx + i0 * MC_MAX_SERP);
        if (click_mask) std::copy(s.click.begin() + i0, s.click.begin() + i1, click_mask + i0);
    });
    return MC_OK;
}

extern "C" void mc_dataset_free(mc_dataset* d) { delete d; }
