// Drives the per-session probability virtuals of include/mclicks_host.hpp on
// the host, with no GPU: parses a log, gives a model the parameter values of a
// file (float32, in get_parameters(ALL) order), and evaluates the test set
// through LogLikelihood and Perplexity, which reach the model only through
// its virtuals (evaluation.cpp:25-66).  A subclass counts the calls, so the
// dispatch itself is checked.  Prints:
//   LLH <sum>            LogLikelihood::evaluate
//   L2 <r> <sum>         Perplexity task_rank_perplexities[r]
//   TASK <n>             Perplexity task_size
//   CALLS <n>            overridden get_log_conditional_click_probs calls
//   SERP_DEV <x>         max |exp(log p_r) - the same probability from
//                        get_serp_probability| over the test set
//   FOOTPRINT <bytes>    compute_memory_footprint(n_train, n_qd)
//
//   virtuals_check LOG MAX_SESSIONS TEST_SHARE MODEL PARAMS.f32
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "mclicks_host.hpp"

using namespace mclicks;

template <typename Base>
struct Counting : Base {
    long calls = 0;
    void get_log_conditional_click_probs(SERP_Hst& s, std::vector<float>& out) override {
        calls++;
        Base::get_log_conditional_click_probs(s, out);
    }
};

static ClickModel_Hst* make(int model, long** calls) {
    switch (model) {
        case MC_CCM: { auto* m = new Counting<CCM_Hst>(); *calls = &m->calls; return m; }
        case MC_DBN: { auto* m = new Counting<DBN_Hst>(); *calls = &m->calls; return m; }
        case MC_UBM: { auto* m = new Counting<UBM_Hst>(); *calls = &m->calls; return m; }
        default: { auto* m = new Counting<PBM_Hst>(); *calls = &m->calls; return m; }
    }
}

int main(int argc, char** argv) {
    if (argc != 6) {
        std::cerr << "usage: virtuals_check LOG MAX_SESSIONS TEST_SHARE MODEL PARAMS.f32" << std::endl;
        return 2;
    }
    ProcessingConfig config;
    config.dataset_path = argv[1];
    config.max_sessions = std::stoi(argv[2]);
    config.test_share = std::stof(argv[3]);
    const int model = std::stoi(argv[4]);
    LocalPartitions parts;
    if (Dataset::parse_dataset(config, parts)) return 1;
    TestSet& test = std::get<1>(parts[0]);
    const int n_qd = std::get<2>(parts[0]);

    std::ifstream f(argv[5], std::ios::binary);
    std::vector<float> flat;
    float v;
    while (f.read(reinterpret_cast<char*>(&v), sizeof v)) flat.push_back(v);

    long* calls = nullptr;
    ClickModel_Hst* cm = make(model, &calls);
    // Sizes in get_parameters(ALL) order (pbm.cu:305-321, ccm.cu:531-533,
    // dbn.cu:535-538, ubm.cu:299-315).
    std::vector<size_t> sizes;
    if (model == MC_PBM) sizes = {10, (size_t)n_qd};
    else if (model == MC_UBM) sizes = {55, (size_t)n_qd};
    else if (model == MC_DBN) sizes = {(size_t)n_qd, (size_t)n_qd, 1};
    else sizes = {(size_t)n_qd, 3};
    std::vector<std::vector<Param>> all;
    size_t off = 0;
    for (size_t k : sizes) {
        std::vector<Param> a(k);
        for (size_t j = 0; j < k; j++) a[j] = Param(flat.at(off + j), 1.f);
        off += k;
        all.push_back(a);
    }
    if (off != flat.size()) {
        std::cerr << "parameter file holds " << flat.size() << " values, expected " << off << std::endl;
        return 3;
    }
    cm->set_parameters(all, ALL);

    LogLikelihood llh(cm);
    const float ll = llh.evaluate(test);
    const long calls_by_llh = *calls;
    Perplexity ppl;
    ppl.evaluate(cm, test);

    double dev = 0;
    for (SERP_Hst s : test) {
        float sp[MAX_SERP];
        std::vector<float> lp;
        cm->get_serp_probability(s, sp);
        cm->get_log_conditional_click_probs(s, lp);
        for (int r = 0; r < MAX_SERP; r++) {
            const bool cascade = model == MC_DBN || model == MC_CCM;
            const float expect = cascade || s[r].get_click() == 1 ? sp[r] : 1 - sp[r];
            dev = std::max(dev, (double)std::fabs(std::exp((double)lp[(size_t)r]) - (double)expect));
        }
    }
    std::printf("LLH %.9g\n", (double)ll);
    for (int r = 0; r < MAX_SERP; r++) std::printf("L2 %d %.9g\n", r, (double)ppl.task_rank_perplexities[(size_t)r]);
    std::printf("TASK %.9g\n", (double)ppl.task_size);
    std::printf("CALLS %ld\n", calls_by_llh);
    std::printf("SERP_DEV %.9g\n", dev);
    std::printf("FOOTPRINT %zu\n", cm->compute_memory_footprint((int)std::get<0>(parts[0]).size(), n_qd));
    std::printf("MEMORY %zu\n", cm->get_memory_usage());
    delete cm;
    return 0;
}
