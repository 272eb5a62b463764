// The reference's C++ host API (include/mclicks_host.hpp) over the C-ABI.
#include <charconv>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <numeric>
#include <stdexcept>
#include <string>

#include "mclicks_host.hpp"
#include "host_internal.h"
#include "pool.h"

namespace mclicks {

// ---------------------------------------------------------------------------
// Sessions
// ---------------------------------------------------------------------------
int SERP_Hst::last_click_rank() const {
    for (int r = MAX_SERP - 1; r >= 0; --r)
        if (session_[r].get_click() == 1) return r;
    return MAX_SERP;
}

void SERP_Hst::prev_clicked_rank(int (&prev)[MAX_SERP]) const {
    int last = MAX_SERP - 1;
    for (int r = 0; r < MAX_SERP; r++) {
        prev[r] = last;
        if (session_[r].get_click() == 1) last = r;
    }
}

uint16_t SERP_Hst::click_mask() const {
    uint16_t m = 0;
    for (int r = 0; r < MAX_SERP; r++)
        if (session_[r].get_click() == 1) m |= (uint16_t)(1u << r);
    return m;
}

static void to_serps(const mc_dataset* d, int which, std::vector<SERP_Hst>& out) {
    const mch::SessionSet& s = which == 0 ? d->train : d->test;
    out.resize((size_t)s.size());
    for (int64_t i = 0; i < s.size(); i++) {
        SERP_Hst& serp = out[(size_t)i];
        serp.set_query(s.query[(size_t)i]);
        for (int r = 0; r < MAX_SERP; r++)
            serp.access_sr(r) = SearchResult_Hst(s.docs[(size_t)(i * MAX_SERP + r)], (s.click[(size_t)i] >> r) & 1,
                                                 s.pidx[(size_t)(i * MAX_SERP + r)]);
    }
}

namespace Dataset {
int parse_dataset(const ProcessingConfig& config, LocalPartitions& partitions) {
    mc_dataset* d = nullptr;
    if (mc_dataset_parse(config.dataset_path.c_str(), config.max_sessions, config.test_share, &d) != MC_OK) return 1;
    partitions.resize(1);
    to_serps(d, 0, std::get<0>(partitions[0]));
    to_serps(d, 1, std::get<1>(partitions[0]));
    std::get<2>(partitions[0]) = (int)d->n_qd;
    mc_dataset_free(d);
    return 0;
}
}  // namespace Dataset

static void session_arrays(const std::vector<SERP_Hst>& set, std::vector<int32_t>& query, std::vector<int32_t>& pidx,
                           std::vector<uint16_t>& click) {
    size_t n = set.size();
    query.resize(n);
    pidx.resize(n * MAX_SERP);
    click.resize(n);
    for (size_t i = 0; i < n; i++) {
        query[i] = set[i].get_query();
        click[i] = set[i].click_mask();
        for (int r = 0; r < MAX_SERP; r++) pidx[i * MAX_SERP + r] = set[i][r].get_param_index();
    }
}

// ---------------------------------------------------------------------------
// Click models
// ---------------------------------------------------------------------------
ClickModel_Hst::ClickModel_Hst(int model_type) : model_type_(model_type) {
    switch (model_type) {
        case MC_PBM:
        case MC_UBM: public_names_ = {"examination"}; private_names_ = {"attractiveness"}; break;
        case MC_DBN: public_names_ = {"continuation"}; private_names_ = {"attractiveness", "satisfaction"}; break;
        default: public_names_ = {"continuation"}; private_names_ = {"attractiveness"}; break;
    }
    public_.resize(public_names_.size());
    private_.resize(private_names_.size());
}

ClickModel_Hst::~ClickModel_Hst() { destroy_parameters(); }

void ClickModel_Hst::check(int rc) const {
    if (rc != MC_OK) {
        char msg[1024];
        mc_last_error(msg, sizeof msg);
        throw std::runtime_error(std::string("mclicks: ") + msg);
    }
}

void ClickModel_Hst::ensure_created() {
    if (!m_) check(mc_model_create(model_type_, mode_, device_, &m_));
}

size_t ClickModel_Hst::get_memory_usage() {
    int64_t b = 0;
    if (m_) check(mc_model_memory(m_, &b));
    return (size_t)b;
}

void ClickModel_Hst::get_parameter_information(
    std::pair<std::vector<std::string>, std::vector<std::string>>& headers,
    std::pair<std::vector<std::vector<Param>*>, std::vector<std::vector<Param>*>>& parameters) {
    headers = std::make_pair(public_names_, private_names_);
    std::vector<std::vector<Param>*> pub, prv;
    for (auto& v : public_) pub.push_back(&v);
    for (auto& v : private_) prv.push_back(&v);
    parameters = std::make_pair(pub, prv);
}

void ClickModel_Hst::init_parameters(const Partition& dataset, size_t, bool) {
    ensure_created();
    std::vector<int32_t> q, p;
    std::vector<uint16_t> c;
    session_arrays(std::get<0>(dataset), q, p, c);
    check(mc_model_upload(m_, (int64_t)q.size(), q.data(), p.data(), c.data(), std::get<2>(dataset), nullptr));
    upload_test(std::get<1>(dataset));
    int n_params = mc_model_param_count(m_);
    for (int i = 0; i < n_params; i++) {
        char name[64];
        int64_t size = 0;
        int pub = 0;
        check(mc_model_param_info(m_, i, name, sizeof name, &size, &pub));
        for (size_t k = 0; k < (pub ? public_names_ : private_names_).size(); k++)
            if ((pub ? public_names_ : private_names_)[k] == name) (pub ? public_ : private_)[k].assign((size_t)size, Param());
    }
}

void ClickModel_Hst::upload_test(const TestSet& test) {
    ensure_created();
    std::vector<int32_t> q, p;
    std::vector<uint16_t> c;
    session_arrays(test, q, p, c);
    check(mc_model_upload_test(m_, (int64_t)q.size(), p.data(), c.data(), nullptr));
}

void ClickModel_Hst::process_session(const TrainSet&, const std::vector<int>&) { check(mc_model_process_sessions(m_, nullptr)); }
void ClickModel_Hst::update_parameters(TrainSet&, const std::vector<int>&) { check(mc_model_update_parameters(m_, nullptr)); }
void ClickModel_Hst::reset_parameters(bool) {}

void ClickModel_Hst::transfer_parameters(int parameter_type, int transfer_direction, bool) {
    int n_params = mc_model_param_count(m_);
    for (int i = 0; i < n_params; i++) {
        char name[64];
        int64_t size = 0;
        int pub = 0;
        check(mc_model_param_info(m_, i, name, sizeof name, &size, &pub));
        if (!(parameter_type == ALL || (parameter_type == PUBLIC) == (pub != 0))) continue;
        auto& names = pub ? public_names_ : private_names_;
        auto& store = pub ? public_ : private_;
        for (size_t k = 0; k < names.size(); k++) {
            if (names[k] != name) continue;
            std::vector<float> v((size_t)size);
            if (transfer_direction == D2H) {
                check(mc_model_get_param(m_, i, v.data(), nullptr));
                store[k].resize((size_t)size);
                for (int64_t j = 0; j < size; j++) store[k][(size_t)j].set_values(v[(size_t)j], 1.f);
            } else {
                for (int64_t j = 0; j < size; j++) v[(size_t)j] = store[k][(size_t)j].value();
                check(mc_model_set_param(m_, i, v.data(), nullptr));
            }
        }
    }
}

void ClickModel_Hst::get_parameters(std::vector<std::vector<Param>>& destination, int parameter_type) {
    // Order of get_parameters(ALL) in the reference: PBM/UBM public first;
    // DBN/CCM private first (pbm.cu:305-321, dbn.cu:535-538, ccm.cu:531-533).
    destination.clear();
    bool pub_first = model_type_ == MC_PBM || model_type_ == MC_UBM;
    if (parameter_type == PUBLIC || (parameter_type == ALL && pub_first))
        for (auto& v : public_) destination.push_back(v);
    if (parameter_type == PRIVATE || parameter_type == ALL)
        for (auto& v : private_) destination.push_back(v);
    if (parameter_type == ALL && !pub_first)
        for (auto& v : public_) destination.push_back(v);
}

void ClickModel_Hst::set_parameters(std::vector<std::vector<Param>>& source, int parameter_type) {
    bool pub_first = model_type_ == MC_PBM || model_type_ == MC_UBM;
    size_t k = 0;
    if (parameter_type == PUBLIC || (parameter_type == ALL && pub_first))
        for (auto& v : public_) v = source.at(k++);
    if (parameter_type == PRIVATE || parameter_type == ALL)
        for (auto& v : private_) v = source.at(k++);
    if (parameter_type == ALL && !pub_first)
        for (auto& v : public_) v = source.at(k++);
}

void ClickModel_Hst::destroy_parameters() {
    if (m_) mc_model_destroy(m_);
    m_ = nullptr;
}

void ClickModel_Hst::em(int iterations, int impl) { check(mc_model_em(m_, iterations, impl, nullptr)); }

void ClickModel_Hst::evaluate_device(int which, double& ll_sum, std::array<double, MAX_SERP>& log2_sums, int64_t& n) {
    check(mc_model_evaluate(m_, which, &ll_sum, log2_sums.data(), &n, nullptr));
}

void PBM_Hst::say_hello() { std::cout << "Host-side PBM says hello!" << std::endl; }
void CCM_Hst::say_hello() { std::cout << "Host-side CCM says hello!" << std::endl; }
void DBN_Hst::say_hello() { std::cout << "Host-side DBN says hello!" << std::endl; }
void UBM_Hst::say_hello() { std::cout << "Host-side UBM says hello!" << std::endl; }

ClickModel_Hst* create_cm_host(int model_type) {
    switch (model_type) {
        case MC_CCM: return new CCM_Hst();
        case MC_DBN: return new DBN_Hst();
        case MC_UBM: return new UBM_Hst();
        default: return new PBM_Hst();
    }
}

// ---------------------------------------------------------------------------
// Evaluation
// ---------------------------------------------------------------------------
float LogLikelihood::evaluate(TestSet& testing_queries) {
    cm_->upload_test(testing_queries);
    double ll = 0;
    std::array<double, MAX_SERP> l2{};
    int64_t n = 0;
    cm_->evaluate_device(1, ll, l2, n);
    return (float)ll;
}

void Perplexity::evaluate(ClickModel_Hst* cm, TestSet& testing_queries) {
    cm->upload_test(testing_queries);
    double ll = 0;
    std::array<double, MAX_SERP> l2{};
    int64_t n = 0;
    cm->evaluate_device(1, ll, l2, n);
    task_size = (float)n;
    for (int r = 0; r < MAX_SERP; r++) task_rank_perplexities[(size_t)r] = (float)l2[(size_t)r];
}

// ---------------------------------------------------------------------------
// Parameter CSVs (communicator.cpp:423-516, one worker): public parameters
// as "rank, value" under a header line; private ones as "query, document,
// value", one line per training session and rank, 0.5 for an index of -1.
// ---------------------------------------------------------------------------
void output_parameters(const std::string& file_path, const Partition& partition, ClickModel_Hst* cm) {
    std::pair<std::vector<std::string>, std::vector<std::string>> headers;
    std::pair<std::vector<std::vector<Param>*>, std::vector<std::vector<Param>*>> params;
    cm->get_parameter_information(headers, params);
    for (size_t k = 0; k < headers.first.size(); k++) {
        std::string path = file_path + "_" + headers.first[k] + ".csv";
        std::cout << "  Writing parameter " << headers.first[k] << " to " << path << std::endl;
        std::ofstream f(path);
        f << "rank, " << headers.first[k] << std::endl;
        for (size_t r = 0; r < params.first[k]->size(); r++) f << r << ", " << (*params.first[k])[r].value() << std::endl;
    }
    for (size_t k = 0; k < headers.second.size(); k++) {
        std::string path = file_path + "_" + headers.second[k] + ".csv";
        std::cout << "  Writing parameter " << headers.second[k] << " to " << path << std::endl;
        // The reference writes this header, then writes the data from offset
        // 0 of the same file (MPI_File_write_at_all), which overwrites it: its
        // files hold the data lines only, and so do these.
        // Lines are formatted on the host threads in chunks of sessions,
        // a bounded group of chunks at a time, and written in order.
        // std::to_chars (fixed, 6 digits; decimal for the ids) gives the text
        // of std::to_string, which the reference writes.
        std::ofstream f(path, std::ios::binary);
        const std::vector<Param>& v = *params.second[k];
        const TrainSet& train = std::get<0>(partition);
        const size_t kChunk = 65536;
        const size_t n_chunks = (train.size() + kChunk - 1) / kChunk;
        const size_t group = 4 * mch::pool_threads();
        std::vector<std::string> text(group);
        for (size_t g0 = 0; g0 < n_chunks; g0 += group) {
            const size_t g1 = std::min(n_chunks, g0 + group);
            mch::parallel_for(g1 - g0, [&](size_t j) {
                std::string& out = text[j];
                out.clear();
                const size_t s0 = (g0 + j) * kChunk, s1 = std::min(train.size(), s0 + kChunk);
                out.reserve((s1 - s0) * MAX_SERP * 28);
                char line[96];
                for (size_t si = s0; si < s1; si++) {
                    const SERP_Hst& sess = train[si];
                    for (int r = 0; r < MAX_SERP; r++) {
                        const SearchResult_Hst sr = sess[r];
                        const float val = sr.get_param_index() != -1 ? v[(size_t)sr.get_param_index()].value() : 0.5f;
                        char* p = std::to_chars(line, line + sizeof line, sess.get_query()).ptr;
                        *p++ = ',';
                        *p++ = ' ';
                        p = std::to_chars(p, line + sizeof line, sr.get_doc_id()).ptr;
                        *p++ = ',';
                        *p++ = ' ';
                        p = std::to_chars(p, line + sizeof line, val, std::chars_format::fixed, 6).ptr;
                        *p++ = '\n';
                        out.append(line, (size_t)(p - line));
                    }
                }
            });
            for (size_t j = 0; j < g1 - g0; j++) f.write(text[j].data(), (std::streamsize)text[j].size());
        }
    }
}

// ---------------------------------------------------------------------------
// em_parallel
// ---------------------------------------------------------------------------
void em_parallel(const ProcessingConfig& config, LocalPartitions& device_partitions) {
    using clock = std::chrono::steady_clock;
    std::cout << "\nExpectation Maximization (EM) in parallel ..." << std::endl;
    ClickModel_Hst* cm = create_cm_host(config.model_type);
    cm->say_hello();
    Partition& part = device_partitions.at(0);

    auto t0 = clock::now();
    cm->init_parameters(part, 0, true);
    double h2d_init = std::chrono::duration<double>(clock::now() - t0).count();

    std::cout << "\nStarting " << config.iterations << " EM parameter estimation iterations..." << std::endl;
    auto t1 = clock::now();
    cm->em(config.iterations);
    double total = std::chrono::duration<double>(clock::now() - t1).count();

    auto t2 = clock::now();
    double ll = 0;
    std::array<double, MAX_SERP> l2{};
    int64_t n_test = 0;
    cm->evaluate_device(1, ll, l2, n_test);
    double eval_s = std::chrono::duration<double>(clock::now() - t2).count();

    if (!config.output_path.empty()) {
        std::cout << "\nWriting output to file..." << std::endl;
        cm->transfer_parameters(ALL, D2H);
        output_parameters(config.output_path, part, cm);
    }

    double it = config.iterations > 0 ? total / config.iterations : 0.0;
    std::cout << "\nTotal Log likelihood is: " << (n_test ? ll / (double)n_test : 0.0) << std::endl;
    double ppl_sum = 0.0;
    for (int r = 0; r < MAX_SERP; r++) {
        double p = n_test ? std::pow(2.0, -l2[(size_t)r] / (double)n_test) : 0.0;
        std::cout << "Perplexity at rank " << r << " is: " << p << std::endl;
        ppl_sum += p;
    }
    std::cout << "Perplexity is: " << ppl_sum / MAX_SERP << std::endl;
    std::cout << "\nHost to Device dataset transfer time: " << h2d_init
              << "\nAverage Host to Device parameter transfer time: " << 0.0
              << "\nAverage Device to Host parameter transfer time: " << 0.0 << std::endl;
    std::cout << "\nAverage time per iteration: " << it
              << "\nAverage time per computation in each iteration: " << it
              << "\nAverage time per update in each iteration: " << 0.0
              << "\nAverage time per synchronization in each iteration: " << 0.0
              << "\nTotal time of training: " << total
              << "\nEvaluation time: " << eval_s << std::endl;
    delete cm;
}

}  // namespace mclicks
