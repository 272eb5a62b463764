// Seeded synthetic click logs in the reference's input shape.
//
// A session is a query id, the ten doc ids shown and a click per rank.  The
// reference reads such sessions from a text log (README.md:39-52: a 15-token
// "Q" line "sid time Q qid region d0..d9" followed by 4-token "C" lines
// "sid time C doc"); mc_synth_write_log writes exactly that format, and
// mc_synth_generate produces the same sessions straight into arrays.
//
// Every random draw is a pure function of (seed, session index) or
// (seed, query, pool slot), so any chunk of sessions can be produced
// independently and in parallel, with the same result for any thread count.
//
//   queries      Zipf(s) over [0, n_queries), drawn by inverse CDF
//   shown list   a random 10-subset of the query's pool, in random order;
//                doc id = query * pool + slot (unique per (query, slot))
//   clicks       from a ground-truth PBM, CCM or DBN (mc_synth_config)
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "mclicks.h"
#include "host_internal.h"

namespace mch {

static inline uint64_t mix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// Small sequential generator seeded from a mixed 64-bit key.
struct Rng {
    uint64_t s;
    explicit Rng(uint64_t key) : s(mix64(key)) {}
    uint64_t next() { s += 0x9e3779b97f4a7c15ULL; return mix64(s); }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    uint32_t below(uint32_t n) { return (uint32_t)((next() >> 32) * (uint64_t)n >> 32); }
};

static inline double hash_uniform(uint64_t seed, uint64_t a, uint64_t b, uint64_t kind) {
    uint64_t h = mix64(seed ^ mix64(a * 0x100000001b3ULL + kind));
    h = mix64(h ^ (b + 0x632be59bd9b4e019ULL * kind));
    return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// Beta(1, b) by inversion: 1 - U^(1/b).
static inline double beta1(double u, double b) { return 1.0 - std::pow(u, 1.0 / b); }

struct Generator {
    mc_synth_config cfg;
    std::vector<double> cdf;  // cumulative Zipf weights, normalised

    explicit Generator(const mc_synth_config& c) : cfg(c) {
        cdf.resize((size_t)c.n_queries);
        double acc = 0.0;
        for (int32_t k = 0; k < c.n_queries; k++) {
            double w = (c.zipf_s == 1.0) ? 1.0 / (double)(k + 1) : std::pow((double)(k + 1), -c.zipf_s);
            acc += w;
            cdf[(size_t)k] = acc;
        }
        for (auto& v : cdf) v /= acc;
    }

    double attractiveness(int32_t q, int32_t slot) const {
        return beta1(hash_uniform(cfg.seed, (uint64_t)q, (uint64_t)slot, 1), cfg.atr_beta_b);
    }
    double satisfaction(int32_t q, int32_t slot) const {
        return beta1(hash_uniform(cfg.seed, (uint64_t)q, (uint64_t)slot, 2), cfg.sat_beta_b);
    }

    void session(int64_t i, int32_t* query, int32_t* docs, uint16_t* mask) const {
        Rng rng((cfg.seed * 0x2545f4914f6cdd1dULL) ^ (uint64_t)i);
        double u = rng.uniform();
        int32_t q = (int32_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        if (q >= cfg.n_queries) q = cfg.n_queries - 1;
        // Partial Fisher-Yates over the pool: the first ten picks, in order.
        int32_t pool = cfg.pool;
        int32_t perm[256];
        for (int32_t k = 0; k < pool; k++) perm[k] = k;
        int32_t slots[MC_MAX_SERP];
        for (int r = 0; r < MC_MAX_SERP; r++) {
            int32_t j = r + (int32_t)rng.below((uint32_t)(pool - r));
            std::swap(perm[r], perm[j]);
            slots[r] = perm[r];
        }
        uint16_t m = 0;
        if (cfg.click_model == 0) {  // PBM: P(click_r) = alpha_qd * 0.9 / sqrt(r + 1)
            for (int r = 0; r < MC_MAX_SERP; r++) {
                double p = attractiveness(q, slots[r]) * cfg.pbm_exam_scale / std::sqrt((double)(r + 1));
                if (rng.uniform() < p) m |= (uint16_t)(1u << r);
            }
        } else if (cfg.click_model == 1) {  // CCM with relevance ~ Beta(1, b)
            bool examined = true;
            for (int r = 0; r < MC_MAX_SERP && examined; r++) {
                double rel = attractiveness(q, slots[r]);
                if (rng.uniform() < rel) {
                    m |= (uint16_t)(1u << r);
                    double cont = cfg.tau2 * (1.0 - rel) + cfg.tau3 * rel;
                    examined = rng.uniform() < cont;
                } else {
                    examined = rng.uniform() < cfg.tau1;
                }
            }
        } else {  // DBN
            bool examined = true;
            for (int r = 0; r < MC_MAX_SERP && examined; r++) {
                if (rng.uniform() < attractiveness(q, slots[r])) {
                    m |= (uint16_t)(1u << r);
                    if (rng.uniform() < satisfaction(q, slots[r])) { examined = false; break; }
                }
                examined = rng.uniform() < cfg.gamma;
            }
        }
        *query = q;
        for (int r = 0; r < MC_MAX_SERP; r++) docs[r] = q * pool + slots[r];
        *mask = m;
    }
};

static int check_config(const mc_synth_config* c) {
    if (!c) return set_error(MC_ERR_INVALID, "synth: null config");
    if (c->n_queries <= 0) return set_error(MC_ERR_INVALID, "synth: n_queries must be positive");
    if (c->pool < MC_MAX_SERP || c->pool > 256)
        return set_error(MC_ERR_INVALID, "synth: pool must be in [10, 256]");
    if ((int64_t)c->n_queries * (int64_t)c->pool > 2147483647LL)
        return set_error(MC_ERR_INVALID, "synth: n_queries * pool overflows int32 doc ids");
    if (c->click_model < 0 || c->click_model > 2)
        return set_error(MC_ERR_INVALID, "synth: click_model must be 0 (PBM), 1 (CCM) or 2 (DBN)");
    return MC_OK;
}

}  // namespace mch

using namespace mch;

extern "C" void mc_synth_config_default(mc_synth_config* c, int preset) {
    std::memset(c, 0, sizeof(*c));
    c->atr_beta_b = 3.0;
    c->sat_beta_b = 4.0;
    c->gamma = 0.9;
    c->tau1 = 0.6; c->tau2 = 0.3; c->tau3 = 0.2;
    c->pbm_exam_scale = 0.9;
    switch (preset) {
        case 1:  // 2M sessions, 100k queries, Zipf 1.0, 30-doc pools, DBN clicks
            c->n_sessions = 2000000; c->n_queries = 100000; c->zipf_s = 1.0; c->pool = 30;
            c->click_model = 2; c->seed = 20240002; break;
        case 2:  // 20M sessions, 1M queries, Zipf 1.0, 50-doc pools, CCM clicks
            c->n_sessions = 20000000; c->n_queries = 1000000; c->zipf_s = 1.0; c->pool = 50;
            c->click_model = 1; c->seed = 20240003; break;
        default:  // 40k sessions, 1k queries, Zipf 1.1, 20-doc pools, PBM clicks
            c->n_sessions = 40000; c->n_queries = 1000; c->zipf_s = 1.1; c->pool = 20;
            c->click_model = 0; c->seed = 20240001; break;
    }
}

extern "C" int mc_synth_generate(const mc_synth_config* cfg, int64_t first, int64_t count,
                                 int32_t* query, int32_t* docs, uint16_t* click_mask) {
    int rc = check_config(cfg);
    if (rc) return rc;
    if (count < 0 || first < 0) return set_error(MC_ERR_INVALID, "synth: negative range");
    if (count > 0 && (!query || !docs || !click_mask)) return set_error(MC_ERR_INVALID, "synth: null output");
    Generator gen(*cfg);
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int64_t n_threads = std::min<int64_t>((int64_t)hw, std::max<int64_t>(1, count / 65536));
    std::vector<std::thread> pool;
    for (int64_t t = 0; t < n_threads; t++) {
        int64_t b = count * t / n_threads, e = count * (t + 1) / n_threads;
        pool.emplace_back([&, b, e]() {
            for (int64_t i = b; i < e; i++)
                gen.session(first + i, &query[i], &docs[i * MC_MAX_SERP], &click_mask[i]);
        });
    }
    for (auto& th : pool) th.join();
    return MC_OK;
}

extern "C" int mc_synth_write_log(const mc_synth_config* cfg, const char* path) {
    int rc = check_config(cfg);
    if (rc) return rc;
    FILE* f = std::fopen(path, "w");
    if (!f) return set_error(MC_ERR_IO, std::string("synth: cannot open ") + path);
    Generator gen(*cfg);
    // One session more than requested: the reference's parser keeps a session
    // only when the next query line arrives, so the last one is never kept.
    for (int64_t i = 0; i <= cfg->n_sessions; i++) {
        int32_t q, docs[MC_MAX_SERP];
        uint16_t m;
        gen.session(i, &q, docs, &m);
        std::fprintf(f, "%lld 0 Q %d 0", (long long)i, q);
        for (int r = 0; r < MC_MAX_SERP; r++) std::fprintf(f, " %d", docs[r]);
        std::fputc('\n', f);
        for (int r = 0; r < MC_MAX_SERP; r++)
            if (m & (1u << r)) std::fprintf(f, "%lld %d C %d\n", (long long)i, r + 1, docs[r]);
    }
    if (std::fclose(f) != 0) return set_error(MC_ERR_IO, std::string("synth: write failed for ") + path);
    return MC_OK;
}
