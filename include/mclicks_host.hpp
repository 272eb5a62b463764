// mclicks_host.hpp — the reference's C++ host API over the GB300 C-ABI.
//
// Same class and function names as the reference's host side, so host code
// written against it keeps compiling:
//   SearchResult_Hst / SERP_Hst / TrainSet / TestSet / Partition /
//   LocalPartitions                               (data/search.cuh:24-55, utils/types.h:26-30)
//   Param                                         (click_models/param.cuh:18-39)
//   ProcessingConfig                              (utils/types.h:81-100)
//   ClickModel_Hst, PBM_Hst, CCM_Hst, DBN_Hst,
//   UBM_Hst, create_cm_host                       (click_models/base.cuh:30-53, base.cu:19-49)
//   LogLikelihood, Perplexity                     (click_models/evaluation.h:21-39)
//   Dataset::parse_dataset                        (data/dataset.h:63)
//   em_parallel                                   (parallel_em/parallel_em.cuh:39-42)
// Everything lives in namespace mclicks.  Device work goes through
// include/mclicks.h; parameters on the host side are held as Param(value, 1).
#ifndef MCLICKS_HOST_HPP
#define MCLICKS_HOST_HPP

#include <array>
#include <cstddef>
#include <cstdint>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "mclicks.h"

namespace mclicks {

constexpr int MAX_SERP = MC_MAX_SERP;
enum { PUBLIC = 0, PRIVATE = 1, ALL = -1 };   // utils/definitions.h:36-38
enum { D2H = 0, H2D = 1 };                    // utils/definitions.h:32-33

class SearchResult_Hst {
public:
    SearchResult_Hst() = default;
    SearchResult_Hst(int doc_id, int click, int param) : click_(click), doc_id_(doc_id), param_index_(param) {}
    void update_click(int click_val) { click_ = click_val; }
    void set_param_index(int index) { param_index_ = index; }
    int get_doc_id() const { return doc_id_; }
    int get_click() const { return click_; }
    int get_param_index() const { return param_index_; }

private:
    int click_ = 0, doc_id_ = 0, param_index_ = -1;
};

class SERP_Hst {
public:
    SERP_Hst() = default;
    SearchResult_Hst operator[](int rank) const { return session_[rank]; }
    SearchResult_Hst& access_sr(int rank) { return session_[rank]; }
    int get_query() const { return query_; }
    void set_query(int q) { query_ = q; }
    // Last clicked rank, MAX_SERP when nothing is clicked (search.cu:160-173).
    int last_click_rank() const;
    // Previous clicked rank per rank, 9 when none (search.cu:184-198).
    void prev_clicked_rank(int (&prev)[MAX_SERP]) const;
    uint16_t click_mask() const;

private:
    int query_ = -1;
    SearchResult_Hst session_[MAX_SERP]{};
};

using TrainSet = std::vector<SERP_Hst>;
using TestSet = std::vector<SERP_Hst>;
using Partition = std::tuple<TrainSet, TestSet, int>;
using LocalPartitions = std::vector<Partition>;

class Param {
public:
    Param() = default;
    Param(float numerator, float denominator) : num_(numerator), den_(denominator) {}
    float value() const {
        float v = num_ / den_;
        return v < 1.f - 0.000001f ? v : 1.f - 0.000001f;
    }
    float numerator_val() const { return num_; }
    float denominator_val() const { return den_; }
    void set_values(float n, float d) { num_ = n; den_ = d; }
    void add_to_values(float n, float d) { num_ += n; den_ += d; }

private:
    float num_ = 1.f, den_ = 2.f;
};

struct ProcessingConfig {
    std::string dataset_path = "YandexRelPredChallenge100k.txt";
    std::string output_path;
    int job_id = 0;
    int max_sessions = 40000;
    int model_type = 0;
    int partitioning_type = 0;
    int node_id = 0;
    int total_nodes = 1;
    int thread_count = 1;
    int iterations = 50;
    int exec_mode = 0;          // 0 = GPU (the only mode here)
    float test_share = 0.2f;
    int device_count = 1;
    int max_gpus = 1;
    int worker_count = 1;
    int device = 0;             // CUDA device to use
    int mode = MC_MODE_PARITY;  // statistics mode
    bool help = false;
};

namespace Dataset {
// Dataset::parse_dataset (data/dataset.cpp:421-455) for one worker; returns 1
// if the file cannot be read.
int parse_dataset(const ProcessingConfig& config, LocalPartitions& partitions);
}  // namespace Dataset

class ClickModel_Hst {
public:
    explicit ClickModel_Hst(int model_type);
    virtual ~ClickModel_Hst();
    ClickModel_Hst(const ClickModel_Hst&) = delete;
    ClickModel_Hst& operator=(const ClickModel_Hst&) = delete;

    virtual ClickModel_Hst* clone() = 0;
    virtual void say_hello() = 0;

    int model_type() const { return model_type_; }
    size_t get_memory_usage();
    void get_parameter_information(std::pair<std::vector<std::string>, std::vector<std::string>>& headers,
                                   std::pair<std::vector<std::vector<Param>*>, std::vector<std::vector<Param>*>>& parameters);

    // init_parameters: uploads the partition (training and test sessions) to
    // the device and sets every parameter to 1/2; fmem is accepted and unused.
    void init_parameters(const Partition& dataset, size_t fmem, bool device);
    // The two halves of one plain iteration (E-step; reset + update).
    void process_session(const TrainSet& dataset, const std::vector<int>& thread_start_idx);
    void update_parameters(TrainSet& dataset, const std::vector<int>& thread_start_idx);
    // The prior (1, 2) is part of the device M-step; kept for callers that call it.
    void reset_parameters(bool device);
    // D2H fills the host-side Param vectors from the device, H2D sends them.
    void transfer_parameters(int parameter_type, int transfer_direction, bool tmp = false);
    void get_parameters(std::vector<std::vector<Param>>& destination, int parameter_type);
    void set_parameters(std::vector<std::vector<Param>>& source, int parameter_type);
    void destroy_parameters();

    // GB300 additions: the fused loop and the device evaluation.
    void em(int iterations, int impl = MC_IMPL_FUSED);
    void evaluate_device(int which, double& ll_sum, std::array<double, MAX_SERP>& log2_sums, int64_t& n);
    void upload_test(const TestSet& test);
    mc_model* handle() { return m_; }

protected:
    void ensure_created();
    void check(int rc) const;
    int model_type_;
    int mode_ = MC_MODE_PARITY;
    int device_ = 0;
    mc_model* m_ = nullptr;
    std::vector<std::string> public_names_, private_names_;
    std::vector<std::vector<Param>> public_, private_;
};

class PBM_Hst : public ClickModel_Hst {
public:
    PBM_Hst() : ClickModel_Hst(MC_PBM) {}
    ClickModel_Hst* clone() override { return new PBM_Hst(); }
    void say_hello() override;
};
class CCM_Hst : public ClickModel_Hst {
public:
    CCM_Hst() : ClickModel_Hst(MC_CCM) {}
    ClickModel_Hst* clone() override { return new CCM_Hst(); }
    void say_hello() override;
};
class DBN_Hst : public ClickModel_Hst {
public:
    DBN_Hst() : ClickModel_Hst(MC_DBN) {}
    ClickModel_Hst* clone() override { return new DBN_Hst(); }
    void say_hello() override;
};
class UBM_Hst : public ClickModel_Hst {
public:
    UBM_Hst() : ClickModel_Hst(MC_UBM) {}
    ClickModel_Hst* clone() override { return new UBM_Hst(); }
    void say_hello() override;
};

// create_cm_host (click_models/base.cu:19-49): unknown ids give a PBM.
ClickModel_Hst* create_cm_host(int model_type);

class LogLikelihood {
public:
    explicit LogLikelihood(ClickModel_Hst* cm) : cm_(cm) {}
    // Sum over sessions of (sum_r log p_r) / 10 (evaluation.cpp:25-40).
    float evaluate(TestSet& testing_queries);

private:
    ClickModel_Hst* cm_;
};

class Perplexity {
public:
    std::array<float, MAX_SERP> task_rank_perplexities{{0}};
    float task_size = 0;
    // Sums of log2 of the full click probability per rank (evaluation.cpp:49-66).
    void evaluate(ClickModel_Hst* cm, TestSet& testing_queries);
};

// em_parallel (parallel_em/parallel_em.cu:349-746) on one GPU: creates the
// model, uploads, runs config.iterations fused iterations, evaluates the test
// set, writes the parameter CSVs when config.output_path is set, and prints
// the reference's result lines.
void em_parallel(const ProcessingConfig& config, LocalPartitions& device_partitions);

// The parameter CSVs of communicator.cpp:423-516 for one worker (private
// parameter files carry no header line, as the reference's do).
void output_parameters(const std::string& file_path, const Partition& partition, ClickModel_Hst* cm);

}  // namespace mclicks

#endif  // MCLICKS_HOST_HPP
