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

// DBN log-likelihood of the reference's conditional model (dbn.cu:611-639)
// in FP64, with a = sigmoid(alpha), s = sigmoid(beta), g = sigmoid(gamma).
double dbn_loglik(int64_t n, const int32_t* pidx, const uint16_t* click, const double* alpha, const double* beta,
                  double gamma) {
    auto sg = [](double x) { return 1.0 / (1.0 + std::exp(-x)); };
    double g = sg(gamma), ll = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double ex = 1.0;
        for (int r = 0; r < R; r++) {
            int32_t p = pidx[i * R + r];
            double a = sg(alpha[p]), s = sg(beta[p]), pr;
            if ((click[i] >> r) & 1) { pr = a * ex; ex = g * (1.0 - s); }
            else { pr = 1.0 - a * ex; ex = ex * g * (1.0 - a) / pr; }
            ll += std::log(pr);
        }
    }
    return ll;
}

// Fisher-identity scores of the same likelihood: the expected complete-data
// score under the exact DBN posterior (a textbook forward-backward over the
// examination chain, not the reference's E-step), with respect to the logits.
//   alpha: clicked occurrence (1 - a); unclicked -a P(E_r = 1 | clicks)
//   beta:  clicked before the last click -s; last click P(S = 1 | clicks) - s
//   gamma: per transition r -> r+1 (r <= 8) from an examined state that may
//          continue: P(E_{r+1} = 1, eligible) - g P(eligible)
void dbn_fisher(int64_t n, const int32_t* pidx, const uint16_t* click, const double* alpha, const double* beta,
                double gamma, double* s_alpha, double* s_beta, double* s_gamma) {
    auto sg = [](double x) { return 1.0 / (1.0 + std::exp(-x)); };
    double g = sg(gamma);
    *s_gamma = 0.0;
    for (int64_t i = 0; i < n; i++) {
        unsigned m = click[i];
        double a[R], s[R];
        int p[R];
        for (int r = 0; r < R; r++) { p[r] = pidx[i * R + r]; a[r] = sg(alpha[p[r]]); s[r] = sg(beta[p[r]]); }
        int l = -1;
        for (int r = R - 1; r >= 0; r--) if ((m >> r) & 1u) { l = r; break; }
        // backward: b[r] = P(no clicks at r..9 | E_r = 1), for ranks after l
        double b[R + 1];
        b[R] = 1.0;
        for (int r = R - 1; r > l; r--) b[r] = (1.0 - a[r]) * (g * b[r + 1] + (1.0 - g));
        // forward after l: f[r] = P(E_r = 1, no clicks in (l, r) | history)
        double f[R + 1] = {0};
        int first = l + 1;
        double start = l >= 0 ? (1.0 - s[l]) * g : 1.0;  // P(E_{l+1} = 1 | click at l) or E_0 = 1
        if (first < R) f[first] = start;
        for (int r = first; r < R - 1; r++) f[r + 1] = f[r] * (1.0 - a[r]) * g;
        // Z = P(no clicks after l | history)
        double Z = l >= 0 ? (s[l] + (1.0 - s[l]) * ((1.0 - g) + g * (l + 1 < R ? b[l + 1] : 1.0))) : b[0];
        if (l >= 0 && l + 1 >= R) Z = 1.0;
        auto pe = [&](int r) {  // P(E_r = 1 | clicks)
            if (r <= l) return 1.0;
            if (r >= R) return 0.0;
            return f[r] * b[r] / Z;
        };
        for (int r = 0; r < R; r++) {
            if ((m >> r) & 1u) s_alpha[p[r]] += 1.0 - a[r];
            else s_alpha[p[r]] += -a[r] * pe(r);
            if ((m >> r) & 1u) {
                if (r < l) s_beta[p[r]] += -s[r];
                else if (l + 1 < R) s_beta[p[r]] += s[r] / Z - s[r];
                else s_beta[p[r]] += 0.0;  // last rank: satisfaction does not affect the likelihood
            }
        }
        for (int r = 0; r < R - 1; r++) {
            if (r < l) {
                *s_gamma += 1.0 - g;
            } else if (r == l) {
                double p_cont = f[l + 1] * b[l + 1] / Z;       // P(S_l = 0, E_{l+1} = 1 | clicks)
                double p_elig = 1.0 - s[l] / Z;                 // P(S_l = 0 | clicks)
                *s_gamma += p_cont - g * p_elig;
            } else {
                *s_gamma += pe(r + 1) - g * pe(r);
            }
        }
    }
}

extern "C" {

double orc_dbn_loglik(int64_t n, const int32_t* pidx, const uint16_t* click, const double* alpha, const double* beta,
                      double gamma) {
    return dbn_loglik(n, pidx, click, alpha, beta, gamma);
}

void orc_dbn_fisher(int64_t n, const int32_t* pidx, const uint16_t* click, const double* alpha, const double* beta,
                    double gamma, double* s_alpha, double* s_beta, double* s_gamma) {
    dbn_fisher(n, pidx, click, alpha, beta, gamma, s_alpha, s_beta, s_gamma);
}

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

void orc_fit_set_copies(void* h, int copy_sessions) {
    FitBox* b = (FitBox*)h;
    b->f32.copy_sessions = copy_sessions != 0;
    b->f64.copy_sessions = copy_sessions != 0;
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
