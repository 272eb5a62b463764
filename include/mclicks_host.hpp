// mclicks_host.hpp — the reference's C++ host API over the GB300 C-ABI.
//
// Same class, member and function names and signatures as the reference's
// host side, so host code written against it keeps compiling:
//   SearchResult_Hst / SERP_Hst                   (data/search.cuh:24-55)
//   TrainSet / TestSet / Partition / LocalPartitions,
//   DeviceProperties / HostProperties / NodeProperties / ClusterProperties,
//   ProcessingConfig                              (utils/types.h:17-100)
//   Param                                         (click_models/param.cuh:18-39)
//   ClickModel_Hst (every member virtual, as in click_models/base.cuh:30-53),
//   PBM_Hst, CCM_Hst, DBN_Hst, UBM_Hst,
//   create_cm_host                                (click_models/base.cu:19-49)
//   LogLikelihood, Perplexity                     (click_models/evaluation.h:21-39)
//   Dataset::parse_dataset                        (data/dataset.h:63)
//   em_parallel                                   (parallel_em/parallel_em.cuh:39-42)
// Everything lives in namespace mclicks.  Device work goes through
// include/mclicks.h; parameters on the host side are held as Param(value, 1).
//
// Not carried over: the MPI communicator (parallel_em/communicator.h), the
// device-property scoring of utils/utils.cuh and the hash-ring partitioner of
// data/dataset.h; this API drives one GPU of one node.
#ifndef MCLICKS_HOST_HPP
#define MCLICKS_HOST_HPP

#include <array>
#include <climits>
#include <cstddef>
#include <cstdint>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "mclicks.h"

#ifndef HOST_NAME_MAX
#define HOST_NAME_MAX 64
#endif

namespace mclicks {

constexpr int MAX_SERP = MC_MAX_SERP;
enum { PUBLIC = 0, PRIVATE = 1, ALL = -1 };   // utils/definitions.h:36-38
enum { D2H = 0, H2D = 1 };                    // utils/definitions.h:32-33

class SearchResult_Hst {
public:
    SearchResult_Hst() = default;
    SearchResult_Hst(const int& doc_id, const int& click, const int& param)
        : click_(click), doc_id_(doc_id), param_index_(param) {}
    void update_click(const int& click_val) { click_ = click_val; }
    void set_param_index(const int& index) { param_index_ = index; }
    int get_doc_id() const { return doc_id_; }
    int get_click() const { return click_; }
    int get_param_index() const { return param_index_; }

private:
    int click_ = 0, doc_id_ = 0, param_index_ = -1;
};

class SERP_Hst {
public:
    SERP_Hst() = default;
    // A query line of the text log, split into its 15 tokens
    // "session time Q query region d0 .. d9" (search.cu:93-108).
    explicit SERP_Hst(const std::vector<std::string>& line);
    SearchResult_Hst operator[](const int& rank) const { return session_[rank]; }
    // A click line "session time C doc": marks the first rank showing doc;
    // false when no rank shows it (search.cu:110-122).
    bool update_click_res(const std::vector<std::string>& line);
    SearchResult_Hst& access_sr(const int& rank) { return session_[rank]; }
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

using UnassignedSet = std::vector<SERP_Hst>;
using TrainSet = UnassignedSet;
using TestSet = UnassignedSet;
using Partition = std::tuple<TrainSet, TestSet, int>;
using LocalPartitions = std::vector<Partition>;

// Cluster description of utils/types.h:32-79.  One node with one device is
// the only layout this API trains on; local_cluster_properties() fills it.
struct DeviceProperties {
    int device_id = 0;
    int compute_capability = 0;
    int registers_per_block = 0;
    int registers_per_sm = 0;
    int threads_per_block = 0;
    int threads_per_sm = 0;
    int warp_size = 0;
    int memory_clock_rate = 0;
    int memory_bus_width = 0;
    int cores_per_sm = 0;
    int clock_rate = 0;
    int multiprocessor_count = 0;
    size_t total_global_memory = 0;
    size_t available_memory = 0;
    size_t shared_memory_per_block = 0;
    size_t total_constant_memory = 0;
    size_t peak_performance = 0;
    char device_name[256] = {0};
};

struct HostProperties {
    int node_id = 0;
    int device_count = 0;
    int thread_count = 0;
    size_t free_memory = 0;
    size_t total_memory = 0;
    char host_name[HOST_NAME_MAX] = {0};
};

struct NodeProperties {
    HostProperties host;
    std::vector<DeviceProperties> devices;
};

struct ClusterProperties {
    int node_count = 0;
    int device_count = 0;
    std::vector<NodeProperties> nodes;
};

class Param {
public:
    Param() = default;
    Param(const float& numerator, const float& denominator) : num_(numerator), den_(denominator) {}
    Param operator+(const Param& other) const { return Param(num_ + other.num_, den_ + other.den_); }
    Param& operator+=(const Param& value) {
        num_ += value.num_;
        den_ += value.den_;
        return *this;
    }
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

// The fields of utils/types.h:81-100, with the reference's defaults of
// main.cpp:189-201, plus `device` (the CUDA device to use) and `mode` (the
// statistics mode of include/mclicks.h).
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
    int* devices_per_node = nullptr;
    int iterations = 50;
    int exec_mode = 0;          // 0 = GPU (the only mode here)
    float test_share = 0.2f;
    int device_count = 1;
    int max_gpus = 1;
    int worker_count = 1;
    bool help = false;
    char host_name[HOST_NAME_MAX] = {0};
    int device = 0;             // CUDA device to use
    int mode = MC_MODE_PARITY;  // statistics mode
};

// A one-node cluster holding the CUDA devices this process sees (name,
// compute capability, SM count, memory), with config.host_name and
// config.thread_count; stands in for Communicate::gather_properties
// (parallel_em/communicator.cpp) in a single-node run.
ClusterProperties local_cluster_properties(const ProcessingConfig& config);

namespace Dataset {
// Dataset::parse_dataset (data/dataset.cpp:421-455) for one worker: the whole
// log goes to my_partitions[0] (resized to at least one partition; further
// partitions are left empty).  Returns 1, as the reference does, when the
// file cannot be read, and also when cluster_properties or config describe
// more than one node, which this API does not partition for.
int parse_dataset(const ClusterProperties& cluster_properties, const ProcessingConfig& config,
                  LocalPartitions& my_partitions);
// The same with the local one-node cluster.
int parse_dataset(const ProcessingConfig& config, LocalPartitions& partitions);
}  // namespace Dataset

class ClickModel_Hst {
public:
    explicit ClickModel_Hst(int model_type);
    virtual ~ClickModel_Hst();
    ClickModel_Hst(const ClickModel_Hst&) = delete;
    ClickModel_Hst& operator=(const ClickModel_Hst&) = delete;

    // ---- the virtual interface of click_models/base.cuh:30-53 -------------
    virtual ClickModel_Hst* clone() = 0;
    virtual void say_hello() = 0;

    // Device bytes the model holds (sessions, tiles, parameters, statistics).
    virtual size_t get_memory_usage(void);
    // Device bytes of the parameter and statistic arrays for n_qd
    // query-document pairs: FP32 values per private parameter, the per-pair
    // occurrence counts, the public values and their FP64 bins.  This design
    // keeps no per-session temporaries, so n_queries (sessions) does not enter,
    // where the reference counts n_queries * MAX_SERP temporary Params
    // (pbm.cu:64-71 etc.).
    virtual size_t compute_memory_footprint(int n_queries, int n_qd);
    virtual void get_parameter_information(
        std::pair<std::vector<std::string>, std::vector<std::string>>& headers,
        std::pair<std::vector<std::vector<Param>*>, std::vector<std::vector<Param>*>>& parameters);
    // Device arrays in the reference's Param layout (numerator, denominator as
    // two floats) holding the current values as (value, 1), one per parameter
    // array in get_parameters(ALL) order: param_refs is a device array of
    // device pointers, param_sizes a device array of their lengths, as in
    // dbn.cu:152-186.  They are a snapshot taken by this call (the fused
    // kernels keep FP32 values, not Params, and do not read them back), owned
    // by the model and freed by destroy_parameters or the next call.
    virtual void get_device_references(Param**& param_refs, int*& param_sizes);

    // The two halves of one plain iteration (E-step; reset + update).
    virtual void process_session(const TrainSet& dataset, const std::vector<int>& thread_start_idx);
    virtual void update_parameters(TrainSet& dataset, const std::vector<int>& thread_start_idx);

    // Uploads the partition (training and test sessions) to the device and
    // sets every parameter to 1/2; fmem and device are accepted and unused.
    virtual void init_parameters(const Partition& dataset, const size_t fmem, const bool device);
    // D2H fills the host-side Param vectors from the device, H2D sends them.
    virtual void transfer_parameters(int parameter_type, int transfer_direction, bool tmp = false);
    virtual void get_parameters(std::vector<std::vector<Param>>& destination, int parameter_type);
    virtual void set_parameters(std::vector<std::vector<Param>>& source, int parameter_type);
    // The prior (1, 2) is part of the device M-step; kept for callers that call it.
    virtual void reset_parameters(bool device);
    virtual void destroy_parameters(void);

    // Per-session probabilities from the host-side parameters (call
    // transfer_parameters(ALL, D2H) first, as the reference's evaluation
    // does); an index of -1 takes the prior value 1/2.
    //   get_serp_probability: PBM/UBM a_r * e_r; DBN/CCM the conditional
    //     click-or-skip probability of each rank (dbn.cu:572-600 etc.);
    //   get_log_conditional_click_probs: appends log of the conditional
    //     probability of what happened at each rank (dbn.cu:611-639 etc.);
    //   get_full_click_probs: appends the unconditional probability of what
    //     happened at each rank (dbn.cu:650-683; UBM: the marginal over the
    //     previous click, ubm.cu:412-468).
    virtual void get_serp_probability(SERP_Hst& query_session, float (&probablities)[MAX_SERP]) = 0;
    virtual void get_log_conditional_click_probs(SERP_Hst& query_session, std::vector<float>& log_click_probs) = 0;
    virtual void get_full_click_probs(SERP_Hst& query_session, std::vector<float>& full_click_probs) = 0;

    // ---- GB300 additions: the fused loop and the device evaluation --------
    int model_type() const { return model_type_; }
    // CUDA device and statistics mode (MC_MODE_PARITY / MC_MODE_CLEAN) of the
    // device model; call before init_parameters.  Defaults: device 0, parity.
    void set_device(int device, int mode = MC_MODE_PARITY);
    void em(int iterations, int impl = MC_IMPL_FUSED);
    void evaluate_device(int which, double& ll_sum, std::array<double, MAX_SERP>& log2_sums, int64_t& n);
    void upload_test(const TestSet& test);
    mc_model* handle() { return m_; }

protected:
    void ensure_created();
    void check(int rc) const;
    void free_device_references();
    // The host-side value of a private parameter array k (0 attractiveness,
    // 1 satisfaction) at index p, 1/2 for p = -1; of public array 0 at i.
    float private_value(size_t k, int p) const;
    float public_value(size_t i) const { return public_[0][i].value(); }
    int model_type_;
    int mode_ = MC_MODE_PARITY;
    int device_ = 0;
    mc_model* m_ = nullptr;
    std::vector<std::string> public_names_, private_names_;
    std::vector<std::vector<Param>> public_, private_;
    void* dev_refs_ = nullptr;                 // device Param* [n] (get_device_references)
    std::vector<void*> dev_ref_arrays_;        // device Param arrays behind it
    void* dev_sizes_ = nullptr;                // device int [n]
};

class PBM_Hst : public ClickModel_Hst {
public:
    PBM_Hst() : ClickModel_Hst(MC_PBM) {}
    ClickModel_Hst* clone() override { return new PBM_Hst(); }
    void say_hello() override;
    void get_serp_probability(SERP_Hst& query_session, float (&probablities)[MAX_SERP]) override;
    void get_log_conditional_click_probs(SERP_Hst& query_session, std::vector<float>& log_click_probs) override;
    void get_full_click_probs(SERP_Hst& query_session, std::vector<float>& full_click_probs) override;
};
class CCM_Hst : public ClickModel_Hst {
public:
    CCM_Hst() : ClickModel_Hst(MC_CCM) {}
    ClickModel_Hst* clone() override { return new CCM_Hst(); }
    void say_hello() override;
    void get_serp_probability(SERP_Hst& query_session, float (&probablities)[MAX_SERP]) override;
    void get_log_conditional_click_probs(SERP_Hst& query_session, std::vector<float>& log_click_probs) override;
    void get_full_click_probs(SERP_Hst& query_session, std::vector<float>& full_click_probs) override;
};
class DBN_Hst : public ClickModel_Hst {
public:
    DBN_Hst() : ClickModel_Hst(MC_DBN) {}
    ClickModel_Hst* clone() override { return new DBN_Hst(); }
    void say_hello() override;
    void get_serp_probability(SERP_Hst& query_session, float (&probablities)[MAX_SERP]) override;
    void get_log_conditional_click_probs(SERP_Hst& query_session, std::vector<float>& log_click_probs) override;
    void get_full_click_probs(SERP_Hst& query_session, std::vector<float>& full_click_probs) override;
};
class UBM_Hst : public ClickModel_Hst {
public:
    UBM_Hst() : ClickModel_Hst(MC_UBM) {}
    ClickModel_Hst* clone() override { return new UBM_Hst(); }
    void say_hello() override;
    void get_serp_probability(SERP_Hst& query_session, float (&probablities)[MAX_SERP]) override;
    void get_log_conditional_click_probs(SERP_Hst& query_session, std::vector<float>& log_click_probs) override;
    void get_full_click_probs(SERP_Hst& query_session, std::vector<float>& full_click_probs) override;
};

// create_cm_host (click_models/base.cu:19-49): unknown ids give a PBM.
ClickModel_Hst* create_cm_host(int model_type);

// evaluation.cpp:25-66, on the host through the model's virtuals.
class LogLikelihood {
public:
    explicit LogLikelihood(ClickModel_Hst* cm) : cm_(cm) {}
    // Appends (sum_r log p_r) / 10 of every test session to the values kept
    // by this object and returns the FP32 sum of all values kept so far.
    float evaluate(TestSet& testing_queries);

private:
    std::vector<float> llh_values_;
    ClickModel_Hst* cm_;
};

class Perplexity {
public:
    std::array<float, MAX_SERP> task_rank_perplexities{{0}};
    float task_size{0};
    Perplexity() = default;
    Perplexity(Perplexity const& ppl_obj) = default;
    // Sets task_size to the number of sessions and adds, per rank, the log2 of
    // every session's full click probability.
    void evaluate(ClickModel_Hst* cm, TrainSet& testing_queries);
    void import(std::array<float, MAX_SERP>& task_rank_perplexities, float& task_size);
};

// em_parallel (parallel_em/parallel_em.cu:349-746) on one GPU: creates the
// model, uploads, runs config.iterations fused iterations, evaluates the test
// set on the device, writes the parameter CSVs when config.output_path is set,
// and prints the reference's result lines.
void em_parallel(const ProcessingConfig& config, LocalPartitions& device_partitions);

// The parameter CSVs of communicator.cpp:423-516 for one worker (private
// parameter files carry no header line, as the reference's do).
void output_parameters(const std::string& file_path, const Partition& partition, ClickModel_Hst* cm);

}  // namespace mclicks

#endif  // MCLICKS_HOST_HPP
