// ORACLE — test infrastructure, not product code.  C entry points over
// oracle.hpp for the Python tests and the benchmark's CPU-baseline leg.
#include <cstring>
#include <memory>

#include "oracle.hpp"

using namespace oracle;

namespace {

struct FitBox {
    int dtype = 1;  // 0 float, 1 double
    Fit<float> f32;
    Fit<double> f64;
    std::vector<Session> data;
    std::vector<int64_t> starts;
};

std::vector<Session> make_sessions(int64_t n, const int32_t* query, const int32_t* pidx, const uint16_t* click) {
    std::vector<Session> v((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        v[(size_t)i].query = query ? query[i] : 0;
        for (int r = 0; r < R; r++)
            v[(size_t)i].r[r] = Result{(click[i] >> r) & 1, 0, pidx[i * R + r]};
    }
    return v;
}

// Query-aligned thread ranges for the update step: an even split with each
// start moved forward to the next query boundary.
std::vector<int64_t> query_aligned_starts(const std::vector<Session>& d, int threads) {
    int64_t n = (int64_t)d.size();
    std::vector<int64_t> s;
    if (threads <= 1 || n == 0) return {0};
    for (int t = 0; t < threads; t++) {
        int64_t b = n * t / threads;
        while (b > 0 && b < n && d[(size_t)b].query == d[(size_t)b - 1].query) b++;
        if (b >= n) break;
        if (s.empty() || b > s.back()) s.push_back(b);
    }
    if (s.empty() || s[0] != 0) s.insert(s.begin(), 0);
    return s;
}

template <typename T>
void flat_params(const Fit<T>& f, double* num, double* den, double* val) {
    std::vector<const std::vector<Param<T>>*> order;
    if (f.type == PBM || f.type == UBM) order = {&f.pub, &f.atr};
    else if (f.type == DBN) order = {&f.atr, &f.sat, &f.pub};
    else order = {&f.atr, &f.pub};
    size_t k = 0;
    for (auto* v : order)
        for (const auto& p : *v) {
            if (num) num[k] = (double)p.num;
            if (den) den[k] = (double)p.den;
            if (val) val[k] = (double)p.value();
            k++;
        }
}

template <typename T>
void set_values(Fit<T>& f, const double* val) {
    std::vector<std::vector<Param<T>>*> order;
    if (f.type == PBM || f.type == UBM) order = {&f.pub, &f.atr};
    else if (f.type == DBN) order = {&f.atr, &f.sat, &f.pub};
    else order = {&f.atr, &f.pub};
    size_t k = 0;
    for (auto* v : order)
        for (auto& p : *v) { p.num = (T)val[k++]; p.den = T(1); }
}

template <typename T>
void eval(const Fit<T>& f, int64_t n_test, const int32_t* pidx, const uint16_t* click, double* llh_sum,
          double* log2_sums, double* llh, double* ppl) {
    std::vector<Session> test = make_sessions(n_test, nullptr, pidx, click);
    T ls, l2[R];
    f.evaluate(test, &ls, l2);
    T n = (T)n_test;
    if (llh_sum) *llh_sum = (double)ls;
    for (int r = 0; r < R; r++) if (log2_sums) log2_sums[r] = (double)l2[r];
    if (llh) *llh = (double)(ls / n);
    double acc = 0.0;
    for (int r = 0; r < R; r++) {
        T pr = (T)std::pow(2.0, (double)((-1 * l2[r]) / n));
        acc += (double)pr;
    }
    if (ppl) *ppl = (double)(T)(acc / 10.0);
}

}  // namespace

extern "C" {

void* orc_parse(const char* path, int max_sessions, float test_share) {
    std::vector<Session> raw;
    if (!parse_log(path, max_sessions, raw)) return nullptr;
    Partition* p = new Partition();
    prepare(std::move(raw), test_share, *p);
    return p;
}

int64_t orc_part_info(void* h, int64_t* n_train, int64_t* n_test) {
    Partition* p = (Partition*)h;
    *n_train = (int64_t)p->train.size();
    *n_test = (int64_t)p->test.size();
    return p->n_qd;
}

void orc_part_copy(void* h, int which, int32_t* query, int32_t* docs, int32_t* pidx, uint16_t* click) {
    Partition* p = (Partition*)h;
    const std::vector<Session>& s = which == 0 ? p->train : p->test;
    for (size_t i = 0; i < s.size(); i++) {
        if (query) query[i] = s[i].query;
        uint16_t m = 0;
        for (int r = 0; r < R; r++) {
            if (docs) docs[i * R + r] = s[i].r[r].doc;
            if (pidx) pidx[i * R + r] = s[i].r[r].pidx;
            if (s[i].r[r].click == 1) m |= (uint16_t)(1u << r);
        }
        if (click) click[i] = m;
    }
}

void orc_part_free(void* h) { delete (Partition*)h; }

void* orc_fit_new(int dtype, int model, int mode, int64_t n, const int32_t* query, const int32_t* pidx,
                  const uint16_t* click, int64_t n_qd) {
    FitBox* b = new FitBox();
    b->dtype = dtype;
    b->data = make_sessions(n, query, pidx, click);
    if (dtype == 0) b->f32.init(model, mode, n, n_qd);
    else b->f64.init(model, mode, n, n_qd);
    return b;
}

int orc_fit_run(void* h, int iterations, int threads) {
    FitBox* b = (FitBox*)h;
    std::vector<int64_t> starts = threads > 1 ? query_aligned_starts(b->data, threads) : std::vector<int64_t>{0};
    for (int it = 0; it < iterations; it++) {
        if (b->dtype == 0) b->f32.iterate(b->data, threads, starts);
        else b->f64.iterate(b->data, threads, starts);
    }
    return 0;
}

int64_t orc_fit_n_params(void* h) {
    FitBox* b = (FitBox*)h;
    if (b->dtype == 0) return (int64_t)(b->f32.atr.size() + b->f32.sat.size() + b->f32.pub.size());
    return (int64_t)(b->f64.atr.size() + b->f64.sat.size() + b->f64.pub.size());
}

void orc_fit_get(void* h, double* num, double* den, double* val) {
    FitBox* b = (FitBox*)h;
    if (b->dtype == 0) flat_params(b->f32, num, den, val);
    else flat_params(b->f64, num, den, val);
}

void orc_fit_set_values(void* h, const double* val) {
    FitBox* b = (FitBox*)h;
    if (b->dtype == 0) set_values(b->f32, val);
    else set_values(b->f64, val);
}

void orc_fit_eval(void* h, int64_t n_test, const int32_t* pidx, const uint16_t* click, double* llh_sum,
                  double* log2_sums, double* llh, double* ppl) {
    FitBox* b = (FitBox*)h;
    if (b->dtype == 0) eval(b->f32, n_test, pidx, click, llh_sum, log2_sums, llh, ppl);
    else eval(b->f64, n_test, pidx, click, llh_sum, log2_sums, llh, ppl);
}

void orc_fit_free(void* h) { delete (FitBox*)h; }

}  // extern "C"
