// ORACLE — test infrastructure, not product code.
//
// A CPU restatement of the reference's (skip-th/MassiveClicks) CPU training
// path: session ingest, the E-step of PBM / UBM / DBN / CCM, the parameter
// reset and update, and the test-set evaluation.  Only tests, the smoke check
// and the benchmark's CPU-baseline leg use it, to check results or as the timed
// CPU baseline; the product never links it.
//
// Templated on the arithmetic type T.  With T = float and one thread it
// evaluates every expression in the reference's order and precision, so its
// parameters match the compiled reference bit for bit (pinned by the golden
// vectors under tests/golden, produced by oracle/ref).  With T = double it is
// the FP64 oracle the GPU results are measured against.
//
// Reference files followed (paths within the reference project):
//   param        click_models/param.cu:116-128 (value(), clamp 1 - 1e-6)
//   PBM          click_models/pbm.cu:191-253 (E), 376-439 (eval)
//   UBM          click_models/ubm.cu:185-247 (E), 376-468 (eval)
//   DBN          click_models/dbn.cu:207-467 (E), 611-683 (eval)
//   CCM          click_models/ccm.cu:185-478 (E), 600-660 (eval)
//   factor       click_models/factor.cu:73-142 (CCM), 206-274 (DBN), host branches
//   update       click_models/common.cu:71-82 (reset), 114-192 (update)
//   session      data/search.cu:160-198 (last / previous clicked rank)
//   evaluation   click_models/evaluation.cpp:25-66, parallel_em/parallel_em.cu:697-723
//   ingest       data/dataset.cpp:224-410, data/search.cu:93-122
//
// The per-thread copy of the whole training set that the reference's DBN and
// CCM E-step threads receive (dbn.cu:244, ccm.cu:223: std::thread copies its
// by-value argument) is reproduced in multi-threaded runs, since it is part of
// what the CPU baseline costs; copy_sessions = false leaves it out where
// only the results matter (the copies do not change them).
#ifndef MCLICKS_ORACLE_HPP
#define MCLICKS_ORACLE_HPP

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <mutex>
#include <numeric>
#include <sstream>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace oracle {

constexpr int R = 10;  // MAX_SERP

enum { PBM = 0, CCM = 1, DBN = 2, UBM = 3 };
enum { PARITY = 0, CLEAN = 1 };

// One search result and one session, in the reference's host layout
// (search.cuh:24-55: click, doc id, parameter index; query first).
struct Result { int32_t click, doc, pidx; };
struct Session {
    int32_t query;
    Result r[R];
    int last_click_rank() const {  // search.cu:160-173; 10 when nothing is clicked
        for (int k = R - 1; k >= 0; --k)
            if (r[k].click == 1) return k;
        return R;
    }
    void prev_clicked_rank(int (&prev)[R]) const {  // search.cu:184-198; 9 when none
        int last = R - 1;
        for (int k = 0; k < R; k++) {
            prev[k] = last;
            if (r[k].click == 1) last = k;
        }
    }
};

template <typename T>
struct Param {
    T num = T(1), den = T(2);
    T value() const {
        const T top = T(1) - T(0.000001);
        return (num / den) < top ? (num / den) : top;
    }
    void add(T n, T d) { num += n; den += d; }
};

template <typename T>
inline T def_value() { return T(1) / T(2); }  // PARAM_DEF_NUM / PARAM_DEF_DENOM

// ---------------------------------------------------------------------------
// Factors of the DBN / CCM gamma and tau updates, host branch of factor.cu.
// ---------------------------------------------------------------------------
template <typename T>
struct Tail {
    T click_probs[R][R];
    T exam_probs[R + 1];
};

template <typename T>
T dbn_factor(const Tail<T>& t, int click, int last, int rank, T a, T s, T g, int x, int y, int z) {
    using std::exp;
    using std::log;
    T lp = T(0);
    if (click == 0) {
        if (y == 1) return T(0);
        lp += log(T(1) - a);
        if (x == 1) {
            if (z == 1) lp += log(g);
            else lp += log(T(1) - g);
        } else if (z == 1) {
            return T(0);
        }
    } else {
        if (x == 0) return T(0);
        lp += log(a);
        if (y == 0) {
            lp += log(T(1) - s);
            if (z == 1) lp += log(g);
            else lp += log(T(1) - g);
        } else {
            if (z == 1) return T(0);
            lp += log(s);
        }
    }
    if (z == 0) {
        if (last >= rank + 1) return T(0);
    } else if (rank + 1 < R) {
        for (int j = 0; j < R - rank - 1; j++) lp += log(t.click_probs[rank + 1][j]);
    }
    T e = t.exam_probs[rank];
    if (x == 1) lp += log(e);
    else lp += log(T(1) - e);
    return exp(lp);
}

template <typename T>
T ccm_factor(const Tail<T>& t, int click, int last, int rank, T a, T t1, T t2, T t3, int x, int y, int z) {
    using std::exp;
    using std::log;
    T lp = T(0);
    if (click == 0) {
        if (y == 1) return T(0);
        lp += log(T(1) - a);
        if (x == 1) {
            if (z == 1) lp += log(t1);
            else lp += log(T(1) - t1);
        } else if (z == 1) {
            return T(0);
        }
    } else {
        if (x == 0) return T(0);
        lp += log(a);
        if (y == 0) {
            lp += log(T(1) - a);
            if (z == 1) lp += log(t2);
            else lp += log(T(1) - t2);
        } else {
            lp += log(a);
            if (z == 1) lp += log(t3);
            else lp += log(T(1) - t3);
        }
    }
    if (z == 0) {
        if (last >= rank + 1) return T(0);
    } else if (rank + 1 < R) {
        for (int j = 0; j < R - rank - 1; j++) lp += log(t.click_probs[rank + 1][j]);
    }
    if (x == 1) lp += log(t.exam_probs[rank]);
    else lp += log(T(1) - t.exam_probs[rank]);
    return exp(lp);
}

static const int kFactorInputs[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 1, 0}, {0, 1, 1},
                                        {1, 0, 0}, {1, 0, 1}, {1, 1, 0}, {1, 1, 1}};

// ---------------------------------------------------------------------------
// One click model fit.
// ---------------------------------------------------------------------------
template <typename T>
struct Fit {
    int type = PBM, mode = PARITY;
    bool copy_sessions = true;  // per-thread dataset copies of DBN/CCM (baseline timing only)
    int64_t n = 0, n_qd = 0;
    std::vector<Param<T>> atr, sat, pub;          // pub: exm (10 / 55), gamma (1), tau (3)
    std::vector<Param<T>> atr_tmp, sat_tmp, pub_tmp;

    int n_public() const { return type == PBM ? R : type == UBM ? R * (R - 1) / 2 + R : type == DBN ? 1 : 3; }

    // init_parameters (common.cu:31-61): values and temporaries start at the
    // default Param (1, 2); CLEAN starts temporaries at (0, 0) so slots the
    // E-step never writes add nothing.
    void init(int type_, int mode_, int64_t n_, int64_t n_qd_) {
        type = type_; mode = mode_; n = n_; n_qd = n_qd_;
        Param<T> tmp_default;
        if (mode == CLEAN) { tmp_default.num = T(0); tmp_default.den = T(0); }
        atr.assign((size_t)n_qd, Param<T>());
        atr_tmp.assign((size_t)(n * R), tmp_default);
        if (type == DBN) {
            sat.assign((size_t)n_qd, Param<T>());
            sat_tmp.assign((size_t)(n * R), tmp_default);
        }
        pub.assign((size_t)n_public(), Param<T>());
        pub_tmp.assign((size_t)(n * n_public()), tmp_default);
    }

    // ---- E-step of one session -------------------------------------------
    void estep_pbm(const Session& ses, int64_t q) {
        for (int r = 0; r < R; r++) {
            const Result& sr = ses.r[r];
            T a = atr[(size_t)sr.pidx].value();
            T e = pub[(size_t)r].value();
            T na = T(1), ne = T(1);
            if (sr.click == 0) {
                T ae = a * e;
                na = (a - ae) / (T(1) - ae);
                ne = (e - ae) / (T(1) - ae);
            }
            atr_tmp[(size_t)(r * n + q)] = Param<T>{na, T(1)};
            pub_tmp[(size_t)(r * n + q)] = Param<T>{ne, T(1)};
        }
    }

    void estep_ubm(const Session& ses, int64_t q) {
        int prev[R];
        ses.prev_clicked_rank(prev);
        for (int r = 0; r < R; r++) {
            const Result& sr = ses.r[r];
            int slot = r * (r + 1) / 2 + prev[r];
            T a = atr[(size_t)sr.pidx].value();
            T e = pub[(size_t)slot].value();
            T na = T(1), ne = T(1);
            if (sr.click == 0) {
                T ae = a * e;
                na = (a - ae) / (T(1) - ae);
                ne = (e - ae) / (T(1) - ae);
            }
            atr_tmp[(size_t)(r * n + q)] = Param<T>{na, T(1)};
            pub_tmp[(size_t)(slot * n + q)] = Param<T>{ne, T(1)};
        }
    }

    // Conditional click probabilities of the tail starting at each rank
    // (dbn.cu:390-423 / ccm.cu:338-380).  As in the reference, the tail that
    // starts at rank s reads the parameters of the documents at ranks
    // 0, 1, ... and the clicks at ranks s, s + 1, ...
    template <bool IsDbn>
    void tail(const Session& ses, Tail<T>& t) {
        for (int s = 0; s < R; s++)
            for (int j = 0; j < R; j++) t.click_probs[s][j] = T(0);
        t.exam_probs[0] = T(1);
        for (int s = 0; s < R; s++) {
            T ex = T(1);
            int j = 0;
            for (int res = s; res < R; res++) {
                const Result& doc = ses.r[j];
                T a = atr[(size_t)doc.pidx].value();
                T cp;
                if (IsDbn) {
                    T sv = sat[(size_t)doc.pidx].value();
                    T g = pub[0].value();
                    if (ses.r[res].click == 1) {
                        cp = a * ex;
                        ex = g * (T(1) - sv);
                    } else {
                        cp = T(1) - a * ex;
                        ex *= g * (T(1) - a) / cp;
                    }
                } else {
                    T t1 = pub[0].value(), t2 = pub[1].value(), t3 = pub[2].value();
                    if (ses.r[res].click == 1) {
                        cp = a * ex;
                        ex = t2 * (T(1) - a) + t3 * a;
                    } else {
                        cp = T(1) - a * ex;
                        ex *= t1 * (T(1) - a) / cp;
                    }
                }
                t.click_probs[s][j] = cp;
                if (s == 0) t.exam_probs[j + 1] = ex;
                j++;
            }
        }
    }

    void estep_dbn(const Session& ses, int64_t q) {
        int last = ses.last_click_rank();
        T exam[R + 1], car[R + 1], h_a[R], h_t[R];
        for (int k = 0; k <= R; k++) car[k] = T(0);
        pub_tmp[(size_t)q] = Param<T>{T(0), T(0)};
        // compute_exm_car (dbn.cu:266-296)
        exam[0] = T(1);
        for (int r = 0; r < R; r++) {
            const Result& sr = ses.r[r];
            T a = atr[(size_t)sr.pidx].value();
            T s = sat[(size_t)sr.pidx].value();
            T g = pub[0].value();
            T ex = exam[r];
            T tmp = g * (T(1) - a);
            ex *= tmp + g * a * (T(1) - s);
            h_a[r] = a; h_t[r] = tmp;
            exam[r + 1] = ex;
        }
        for (int r = R - 1; r >= 0; r--) car[r] = h_a[r] + h_t[r] * car[r + 1];
        // compute_dbn_atr (dbn.cu:312-336)
        for (int r = 0; r < R; r++) {
            const Result& sr = ses.r[r];
            T num = T(0), den = T(1);
            if (sr.click == 1) {
                num += T(1);
            } else if (r >= last) {
                T a = atr[(size_t)sr.pidx].value();
                T e = exam[r], c = car[r];
                num += (a * (T(1) - e)) / (T(1) - e * c);
            }
            atr_tmp[(size_t)(r * n + q)] = Param<T>{num, den};
        }
        // compute_dbn_sat (dbn.cu:350-378): unclicked ranks are not written
        for (int r = 0; r < R; r++) {
            const Result& sr = ses.r[r];
            if (sr.click == 1) {
                T num = T(0), den = T(1);
                if (r == last) {
                    T s = sat[(size_t)sr.pidx].value();
                    T g = pub[0].value();
                    T c = r < R - 1 ? car[r + 1] : T(0);
                    num += s / (T(1) - (T(1) - s) * g * c);
                }
                sat_tmp[(size_t)(r * n + q)] = Param<T>{num, den};
            }
        }
        Tail<T> t;
        tail<true>(ses, t);
        // compute_gamma (dbn.cu:436-467)
        for (int r = 0; r < R; r++) {
            const Result& sr = ses.r[r];
            T a = atr[(size_t)sr.pidx].value(), s = sat[(size_t)sr.pidx].value(), g = pub[0].value();
            T f[8];
            T sum = T(0);
            for (int k = 0; k < 8; k++) {
                f[k] = dbn_factor<T>(t, sr.click, last, r, a, s, g, kFactorInputs[k][0], kFactorInputs[k][1], kFactorInputs[k][2]);
                sum += f[k];
            }
            T num = f[5] / sum;
            T den = (f[4] + f[5]) / sum;
            pub_tmp[(size_t)q].add(num, den);
        }
    }

    void estep_ccm(const Session& ses, int64_t q) {
        int last = ses.last_click_rank();
        T exam[R + 1], car[R + 1], h_a[R], h_t[R];
        for (int k = 0; k <= R; k++) car[k] = T(0);
        for (int k = 0; k < 3; k++) pub_tmp[(size_t)(k * n + q)] = Param<T>{T(0), T(0)};
        // compute_exm_car (ccm.cu:245-286)
        exam[0] = T(1);
        for (int r = 0; r < R; r++) {
            const Result& sr = ses.r[r];
            T a = atr[(size_t)sr.pidx].value();
            T t1 = pub[0].value(), t2 = pub[1].value(), t3 = pub[2].value();
            T ex = exam[r];
            T tmp = (T(1) - a) * t1;
            ex *= tmp + a * ((T(1) - a) * t2 + a * t3);
            h_a[r] = a; h_t[r] = tmp;
            exam[r + 1] = ex;
        }
        for (int r = R - 1; r >= 0; r--) car[r] = h_a[r] + h_t[r] * car[r + 1];
        // compute_ccm_atr (ccm.cu:295-331)
        for (int r = 0; r < R; r++) {
            const Result& sr = ses.r[r];
            T num = T(0), den = T(1);
            T a = atr[(size_t)sr.pidx].value();
            T e = exam[r];
            if (sr.click == 1) {
                num += T(1);
                den += T(1);
            } else if (r >= last) {
                T c = car[r];
                num += ((T(1) - e) * a) / (T(1) - e * c);
            }
            if (sr.click == 1 && r == last) {
                T c = car[r + 1];
                num += a / (T(1) - (pub[1].value() * (T(1) - a) + pub[2].value() * a) * c);
            }
            atr_tmp[(size_t)(r * n + q)] = Param<T>{num, den};
        }
        Tail<T> t;
        tail<false>(ses, t);
        // compute_taus (ccm.cu:387-476): quotients in T, accumulated through
        // double temporaries and added back as T.
        for (int r = 0; r < R; r++) {
            const Result& sr = ses.r[r];
            T a = atr[(size_t)sr.pidx].value();
            T t1 = pub[0].value(), t2 = pub[1].value(), t3 = pub[2].value();
            T f[8];
            T sum = T(0);
            for (int k = 0; k < 8; k++) {
                f[k] = ccm_factor<T>(t, sr.click, last, r, a, t1, t2, t3, kFactorInputs[k][0], kFactorInputs[k][1], kFactorInputs[k][2]);
                sum += f[k];
            }
            if (sr.click == 0) {
                double nu = (f[5] + f[7]) / sum;
                double de = nu + ((f[4] + f[6]) / sum);
                pub_tmp[(size_t)q].add((T)nu, (T)de);
            } else {
                double nu2 = f[5] / sum;
                double de2 = nu2 + (f[4] / sum);
                pub_tmp[(size_t)(n + q)].add((T)nu2, (T)de2);
                double nu3 = f[7] / sum;
                double de3 = nu3 + (f[6] / sum);
                pub_tmp[(size_t)(2 * n + q)].add((T)nu3, (T)de3);
            }
        }
    }

    void estep_range(const std::vector<Session>& data, int64_t b, int64_t e) {
        for (int64_t q = b; q < e; q++) {
            const Session ses = data[(size_t)q];
            switch (type) {
                case PBM: estep_pbm(ses, q); break;
                case UBM: estep_ubm(ses, q); break;
                case DBN: estep_dbn(ses, q); break;
                default: estep_ccm(ses, q); break;
            }
        }
    }

    // process_session: an even split over threads (pbm.cu:233-252).
    void process_sessions(const std::vector<Session>& data, int threads) {
        if (threads <= 1) { estep_range(data, 0, n); return; }
        int64_t part = n / threads, left = n % threads, b = 0;
        std::vector<std::thread> pool;
        for (int t = 0; t < threads; t++) {
            int64_t e = b + (t < left ? part + 1 : part);
            if ((type == DBN || type == CCM) && copy_sessions) {
                // The reference hands each thread its own copy of the sessions.
                pool.emplace_back([this, b, e](std::vector<Session> copy) { estep_range(copy, b, e); }, data);
            } else {
                pool.emplace_back([this, &data, b, e]() { estep_range(data, b, e); });
            }
            b = e;
        }
        for (auto& th : pool) th.join();
    }

    // reset_parameters (common.cu:71-82).
    void reset() {
        for (auto& p : atr) p = Param<T>();
        for (auto& p : sat) p = Param<T>();
        for (auto& p : pub) p = Param<T>();
    }

    // update_unique_parameters_hst (common.cu:114-141).
    void update_unique(std::vector<Param<T>>& src, std::vector<Param<T>>& dst, const std::vector<Session>& data,
                       int64_t b, int64_t e) {
        for (int64_t q = b; q < e; q++)
            for (int r = 0; r < R; r++) {
                const Param<T>& u = src[(size_t)(r * n + q)];
                Param<T>& d = dst[(size_t)data[(size_t)q].r[r].pidx];
                d.num += u.num;
                d.den += u.den;
            }
    }

    // update_shared_parameters_hst (common.cu:153-192): per-thread partials
    // from (0, 0), then added under a mutex per slot.
    void update_shared_part(int tid, int64_t b, int64_t e, std::vector<std::mutex>& mtx) {
        size_t k_n = pub.size();
        std::vector<Param<T>> local(k_n, Param<T>{T(0), T(0)});
        for (int64_t q = b; q < e; q++)
            for (size_t k = 0; k < k_n; k++) {
                const Param<T>& u = pub_tmp[(size_t)((int64_t)k * n + q)];
                local[k].num += u.num;
                local[k].den += u.den;
            }
        int off = tid % (int)k_n;
        for (size_t k = 0; k < k_n; k++) {
            size_t idx = (k + (size_t)off) % k_n;
            std::lock_guard<std::mutex> lock(mtx[idx]);
            pub[idx].num += local[idx].num;
            pub[idx].den += local[idx].den;
        }
    }

    // update_parameters over query-aligned thread ranges.
    void update_parameters(const std::vector<Session>& data, const std::vector<int64_t>& starts) {
        size_t n_threads = starts.size();
        std::vector<std::mutex> mtx(pub.size());
        auto run = [&](std::vector<Param<T>>& src, std::vector<Param<T>>& dst) {
            std::vector<std::thread> pool;
            for (size_t t = 0; t < n_threads; t++) {
                int64_t b = starts[t], e = t + 1 < n_threads ? starts[t + 1] : n;
                pool.emplace_back([&, b, e]() { update_unique(src, dst, data, b, e); });
            }
            for (auto& th : pool) th.join();
        };
        if (n_threads <= 1) {
            update_unique(atr_tmp, atr, data, 0, n);
            if (type == DBN) update_unique(sat_tmp, sat, data, 0, n);
            update_shared_part(0, 0, n, mtx);
            return;
        }
        run(atr_tmp, atr);
        if (type == DBN) run(sat_tmp, sat);
        std::vector<std::thread> pool;
        for (size_t t = 0; t < n_threads; t++) {
            int64_t b = starts[t], e = t + 1 < n_threads ? starts[t + 1] : n;
            pool.emplace_back([&, t, b, e]() { update_shared_part((int)t, b, e, mtx); });
        }
        for (auto& th : pool) th.join();
    }

    // One EM iteration of the CPU path (parallel_em.cu:462-609, exec_mode 1).
    void iterate(const std::vector<Session>& data, int threads, const std::vector<int64_t>& starts) {
        process_sessions(data, threads);
        reset();
        update_parameters(data, starts);
    }

    // ---- evaluation (host) ------------------------------------------------
    T atr_or_default(int32_t p) const { return p != -1 ? atr[(size_t)p].value() : def_value<T>(); }
    T sat_or_default(int32_t p) const { return p != -1 ? sat[(size_t)p].value() : def_value<T>(); }

    void log_conditional(const Session& ses, T (&out)[R]) const {
        using std::log;
        if (type == PBM || type == UBM) {
            int prev[R];
            ses.prev_clicked_rank(prev);
            for (int r = 0; r < R; r++) {
                T a = atr_or_default(ses.r[r].pidx);
                T e = type == PBM ? pub[(size_t)r].value() : pub[(size_t)(r * (r + 1) / 2 + prev[r])].value();
                T ae = a * e;
                out[r] = ses.r[r].click == 1 ? log(ae) : log(T(1) - ae);
            }
        } else {
            T ex = T(1), cp;
            for (int r = 0; r < R; r++) {
                T a = atr_or_default(ses.r[r].pidx);
                if (type == DBN) {
                    T s = sat_or_default(ses.r[r].pidx);
                    T g = pub[0].value();
                    if (ses.r[r].click == 1) { cp = a * ex; ex = g * (T(1) - s); }
                    else { cp = T(1) - a * ex; ex *= g * (T(1) - a) / cp; }
                } else {
                    T t1 = pub[0].value(), t2 = pub[1].value(), t3 = pub[2].value();
                    if (ses.r[r].click == 1) { cp = a * ex; ex = t2 * (T(1) - a) + t3 * a; }
                    else { cp = T(1) - a * ex; ex *= t1 * (T(1) - a) / cp; }
                }
                out[r] = log(cp);
            }
        }
    }

    void full_click_probs(const Session& ses, T (&out)[R]) const {
        if (type == PBM) {
            for (int r = 0; r < R; r++) {
                T ae = atr_or_default(ses.r[r].pidx) * pub[(size_t)r].value();
                out[r] = ses.r[r].click == 1 ? ae : T(1) - ae;
            }
        } else if (type == UBM) {  // ubm.cu:412-468: marginal over the previous click
            T marg[R];
            for (int r = 0; r < R; r++) {
                T cp = T(0);
                for (int pc = -1; pc < r; pc++) {
                    T none_between = T(1);
                    int pcc = pc == -1 ? 9 : pc;
                    for (int b = pc + 1; b < r; b++) {
                        T ab = atr_or_default(ses.r[b].pidx);
                        T eb = pub[(size_t)(b * (b + 1) / 2 + pcc)].value();
                        none_between *= T(1) - ab * eb;
                    }
                    T a = atr_or_default(ses.r[r].pidx);
                    T e = pub[(size_t)(r * (r + 1) / 2 + pcc)].value();
                    T tmp = none_between * (a * e);
                    if (pc >= 0) cp += marg[pc] * tmp;
                    else cp += tmp;
                }
                marg[r] = cp;
                out[r] = ses.r[r].click == 1 ? cp : T(1) - cp;
            }
        } else {
            T ex = T(1);
            for (int r = 0; r < R; r++) {
                T a = atr_or_default(ses.r[r].pidx);
                T ae = a * ex;
                out[r] = ses.r[r].click == 1 ? ae : T(1) - ae;
                if (type == DBN) {
                    T s = sat_or_default(ses.r[r].pidx), g = pub[0].value();
                    ex *= g * (T(1) - a) + g * a * (T(1) - s);
                } else {
                    T t1 = pub[0].value(), t2 = pub[1].value(), t3 = pub[2].value();
                    ex *= (T(1) - a) * t1 + a * ((T(1) - a) * t2 + a * t3);
                }
            }
        }
    }

    // LogLikelihood::evaluate and Perplexity::evaluate (evaluation.cpp:25-66).
    void evaluate(const std::vector<Session>& test, T* llh_sum, T (&log2_sums)[R]) const {
        using std::log2;
        std::vector<T> per_session;
        for (int r = 0; r < R; r++) log2_sums[r] = T(0);
        for (const Session& ses : test) {
            T lp[R], fp[R];
            log_conditional(ses, lp);
            T acc = T(0);
            for (int r = 0; r < R; r++) acc += lp[r];
            per_session.push_back(acc / R);
            full_click_probs(ses, fp);
            for (int r = 0; r < R; r++) log2_sums[r] += log2(fp[r]);
        }
        T tot = T(0);
        for (T v : per_session) tot += v;
        *llh_sum = tot;
    }
};

// ---------------------------------------------------------------------------
// Ingest, restated literally: the reference's parser, split, std::sort of the
// session records and a map of maps for the query-document indices.
// ---------------------------------------------------------------------------
struct Partition {
    std::vector<Session> train, test;
    int64_t n_qd = 0;
};

inline bool stoi_ok(const std::string& s, int32_t* v) {
    try {
        size_t pos = 0;
        *v = std::stoi(s, &pos);
        return true;
    } catch (...) {
        return false;
    }
}

inline bool parse_log(const std::string& path, int max_sessions, std::vector<Session>& out) {
    std::ifstream f(path);
    if (!f.is_open()) return false;
    std::string line, tok;
    Session cur{};
    cur.query = -1;
    for (auto& x : cur.r) x = Result{0, 0, -1};
    int n_queries = 0;
    int prev_sid = -1;
    while ((n_queries < max_sessions || max_sessions == -1) && std::getline(f, line)) {
        std::istringstream ss(line);
        std::vector<std::string> v;
        while (ss >> tok) v.push_back(tok);
        int32_t sid;
        if (v.empty() || !stoi_ok(v[0], &sid)) continue;
        if (v.size() == 15) {
            Session nx{};
            bool ok = stoi_ok(v[3], &nx.query);
            for (int k = 0; k < R && ok; k++) {
                int32_t d;
                ok = stoi_ok(v[5 + k], &d);
                nx.r[k] = Result{0, d, -1};
            }
            if (!ok) continue;
            if (prev_sid != -1) {
                out.push_back(cur);
                n_queries++;
            }
            cur = nx;
        } else if (v.size() == 4) {
            int32_t d;
            if (!stoi_ok(v[3], &d)) continue;
            for (int k = 0; k < R; k++)
                if (cur.r[k].doc == d) { cur.r[k].click = 1; break; }
        }
        prev_sid = sid;
    }
    return true;
}

inline void prepare(std::vector<Session> sessions, float test_share, Partition& p) {
    int n = (int)sessions.size();
    int n_train = static_cast<int>(n * (1 - test_share) - 0.5) + 1;
    if (n_train > n) n_train = n;
    p.test.assign(sessions.begin() + n_train, sessions.end());
    sessions.erase(sessions.begin() + n_train, sessions.end());
    std::sort(sessions.begin(), sessions.end(), [](const Session& a, const Session& b) { return a.query < b.query; });
    std::unordered_map<int, std::unordered_map<int, int>> qd;
    int64_t idx = 0;
    for (Session& s : sessions) {
        auto qit = qd.emplace(s.query, std::unordered_map<int, int>{}).first;
        for (int k = 0; k < R; k++) {
            auto ins = qit->second.emplace(s.r[k].doc, (int)idx);
            s.r[k].pidx = ins.first->second;
            if (ins.second) idx++;
        }
    }
    p.n_qd = idx;
    p.train = std::move(sessions);
    p.test.erase(std::remove_if(p.test.begin(), p.test.end(), [&](Session& s) {
        auto qit = qd.find(s.query);
        if (qit == qd.end()) return true;
        bool found = false;
        for (int k = 0; k < R; k++) {
            auto dit = qit->second.find(s.r[k].doc);
            if (dit != qit->second.end()) { found = true; s.r[k].pidx = dit->second; }
        }
        return !found;
    }), p.test.end());
}

}  // namespace oracle

#endif  // MCLICKS_ORACLE_HPP
