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

#include <cuda_runtime.h>
#include <unistd.h>

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

SERP_Hst::SERP_Hst(const std::vector<std::string>& line) {
    query_ = std::stoi(line.at(3));
    for (int r = 0; r < MAX_SERP; r++) session_[r] = SearchResult_Hst(std::stoi(line.at((size_t)r + 5)), 0, -1);
}

bool SERP_Hst::update_click_res(const std::vector<std::string>& line) {
    const int doc = std::stoi(line.at(3));
    for (int r = 0; r < MAX_SERP; r++)
        if (session_[r].get_doc_id() == doc) {
            session_[r].update_click(1);
            return true;
        }
    return false;
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

ClusterProperties local_cluster_properties(const ProcessingConfig& config) {
    ClusterProperties c;
    NodeProperties node;
    node.host.node_id = config.node_id;
    node.host.thread_count = config.thread_count;
    if (config.host_name[0]) std::snprintf(node.host.host_name, HOST_NAME_MAX, "%s", config.host_name);
    else if (gethostname(node.host.host_name, HOST_NAME_MAX) != 0) node.host.host_name[0] = 0;
    node.host.host_name[HOST_NAME_MAX - 1] = 0;
    const long pages = sysconf(_SC_PHYS_PAGES), avail = sysconf(_SC_AVPHYS_PAGES), psize = sysconf(_SC_PAGE_SIZE);
    if (pages > 0 && psize > 0) node.host.total_memory = (size_t)pages * (size_t)psize;
    if (avail > 0 && psize > 0) node.host.free_memory = (size_t)avail * (size_t)psize;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    for (int d = 0; d < n; d++) {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, d) != cudaSuccess) continue;
        DeviceProperties dp;
        dp.device_id = d;
        dp.compute_capability = p.major * 10 + p.minor;
        dp.registers_per_block = p.regsPerBlock;
        dp.registers_per_sm = p.regsPerMultiprocessor;
        dp.threads_per_block = p.maxThreadsPerBlock;
        dp.threads_per_sm = p.maxThreadsPerMultiProcessor;
        dp.warp_size = p.warpSize;
        dp.memory_bus_width = p.memoryBusWidth;
        dp.multiprocessor_count = p.multiProcessorCount;
        dp.total_global_memory = p.totalGlobalMem;
        dp.shared_memory_per_block = p.sharedMemPerBlock;
        dp.total_constant_memory = p.totalConstMem;
        size_t fr = 0, tot = 0;
        int cur = 0;
        if (cudaGetDevice(&cur) == cudaSuccess && cudaSetDevice(d) == cudaSuccess) {
            if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) dp.available_memory = fr;
            cudaSetDevice(cur);
        }
        std::snprintf(dp.device_name, sizeof dp.device_name, "%s", p.name);
        node.devices.push_back(dp);
    }
    node.host.device_count = (int)node.devices.size();
    c.node_count = 1;
    c.device_count = node.host.device_count;
    c.nodes.push_back(node);
    return c;
}

namespace Dataset {
int parse_dataset(const ClusterProperties& cluster_properties, const ProcessingConfig& config,
                  LocalPartitions& my_partitions) {
    if (cluster_properties.node_count > 1 || cluster_properties.nodes.size() > 1 || config.total_nodes > 1) {
        std::cerr << "[" << config.host_name << "] Error: this build trains on one node; "
                  << std::max<size_t>((size_t)config.total_nodes, cluster_properties.nodes.size())
                  << " nodes were given." << std::endl;
        return 1;
    }
    LocalPartitions parts;
    if (parse_dataset(config, parts)) return 1;
    if (my_partitions.empty()) my_partitions.resize(1);
    for (Partition& p : my_partitions) p = Partition();
    my_partitions[0] = std::move(parts[0]);
    return 0;
}

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

size_t ClickModel_Hst::compute_memory_footprint(int, int n_qd) {
    // Rounded as the device arrays are: qd arrays padded to a multiple of 4
    // plus 4 slots.
    const size_t qd = (size_t)(((std::max(n_qd, 1) + 3) & ~3) + 4);
    const size_t n_private = model_type_ == MC_DBN ? 2 : 1;
    const size_t n_pub = model_type_ == MC_PBM ? 10 : model_type_ == MC_UBM ? 55 : model_type_ == MC_DBN ? 1 : 3;
    // FP32 values per private parameter; uint2 occurrence / clicked counts and
    // their packed 16-bit copy; FP32 public values (two halves of 128); FP64
    // public bins and constants (numerator, denominator).
    return qd * (4 * n_private + 8 + 4) + 2 * 128 * 4 + 2 * (2 * n_pub * 8);
}

void ClickModel_Hst::free_device_references() {
    for (void* a : dev_ref_arrays_) cudaFree(a);
    dev_ref_arrays_.clear();
    if (dev_refs_) cudaFree(dev_refs_);
    if (dev_sizes_) cudaFree(dev_sizes_);
    dev_refs_ = dev_sizes_ = nullptr;
}

void ClickModel_Hst::get_device_references(Param**& param_refs, int*& param_sizes) {
    static_assert(sizeof(Param) == 2 * sizeof(float), "Param must be two floats");
    if (!m_) throw std::runtime_error("mclicks: get_device_references before init_parameters");
    free_device_references();
    int cur = 0;
    check(cudaGetDevice(&cur) == cudaSuccess ? MC_OK : MC_ERR_CUDA);
    if (cur != device_ && cudaSetDevice(device_) != cudaSuccess) check(MC_ERR_CUDA);
    const int n = mc_model_param_count(m_);
    std::vector<Param*> refs((size_t)n, nullptr);
    std::vector<int> sizes((size_t)n, 0);
    auto fail = [&](const char* what) {
        free_device_references();
        cudaSetDevice(cur);
        throw std::runtime_error(std::string("mclicks: get_device_references: ") + what);
    };
    for (int i = 0; i < n; i++) {
        char name[64];
        int64_t size = 0;
        int pub = 0;
        check(mc_model_param_info(m_, i, name, sizeof name, &size, &pub));
        std::vector<float> v((size_t)size);
        check(mc_model_get_param(m_, i, v.data(), nullptr));
        std::vector<Param> host((size_t)size);
        for (int64_t j = 0; j < size; j++) host[(size_t)j] = Param(v[(size_t)j], 1.f);
        void* d = nullptr;
        if (cudaMalloc(&d, std::max<size_t>(1, host.size()) * sizeof(Param)) != cudaSuccess) fail("cudaMalloc failed");
        dev_ref_arrays_.push_back(d);
        if (!host.empty() && cudaMemcpy(d, host.data(), host.size() * sizeof(Param), cudaMemcpyHostToDevice) != cudaSuccess)
            fail("cudaMemcpy failed");
        refs[(size_t)i] = (Param*)d;
        sizes[(size_t)i] = (int)size;
    }
    if (cudaMalloc(&dev_refs_, std::max(1, n) * sizeof(Param*)) != cudaSuccess ||
        cudaMalloc(&dev_sizes_, std::max(1, n) * sizeof(int)) != cudaSuccess)
        fail("cudaMalloc failed");
    if (cudaMemcpy(dev_refs_, refs.data(), (size_t)n * sizeof(Param*), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dev_sizes_, sizes.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess)
        fail("cudaMemcpy failed");
    cudaSetDevice(cur);
    param_refs = (Param**)dev_refs_;
    param_sizes = (int*)dev_sizes_;
}

float ClickModel_Hst::private_value(size_t k, int p) const {
    return p != -1 ? private_[k][(size_t)p].value() : 1.f / 2.f;
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
    free_device_references();
    if (m_) mc_model_destroy(m_);
    m_ = nullptr;
}

void ClickModel_Hst::set_device(int device, int mode) {
    if (m_ && (device != device_ || mode != mode_))
        throw std::runtime_error("mclicks: set_device after init_parameters");
    device_ = device;
    mode_ = mode;
}

void ClickModel_Hst::em(int iterations, int impl) { check(mc_model_em(m_, iterations, impl, nullptr)); }

void ClickModel_Hst::evaluate_device(int which, double& ll_sum, std::array<double, MAX_SERP>& log2_sums, int64_t& n) {
    check(mc_model_evaluate(m_, which, &ll_sum, log2_sums.data(), &n, nullptr));
}

// ---------------------------------------------------------------------------
// Per-session probabilities from the host-side values, in FP32 with the
// reference's expressions (pbm.cu:351-420, ubm.cu:345-468, dbn.cu:572-683,
// ccm.cu:566-650).
// ---------------------------------------------------------------------------
void PBM_Hst::get_serp_probability(SERP_Hst& q, float (&prob)[MAX_SERP]) {
    for (int r = 0; r < MAX_SERP; r++) prob[r] = private_value(0, q[r].get_param_index()) * public_value((size_t)r);
}

void PBM_Hst::get_log_conditional_click_probs(SERP_Hst& q, std::vector<float>& out) {
    for (int r = 0; r < MAX_SERP; r++) {
        const float ae = private_value(0, q[r].get_param_index()) * public_value((size_t)r);
        out.push_back(q[r].get_click() == 1 ? std::log(ae) : std::log(1 - ae));
    }
}

void PBM_Hst::get_full_click_probs(SERP_Hst& q, std::vector<float>& out) {
    for (int r = 0; r < MAX_SERP; r++) {
        const float ae = private_value(0, q[r].get_param_index()) * public_value((size_t)r);
        out.push_back(q[r].get_click() == 1 ? ae : 1 - ae);
    }
}

// UBM examination slot of rank r after a previous click at rank p (9 = none).
static inline size_t ubm_slot(int r, int p) { return (size_t)(r * (r + 1) / 2 + p); }

void UBM_Hst::get_serp_probability(SERP_Hst& q, float (&prob)[MAX_SERP]) {
    int prev[MAX_SERP];
    q.prev_clicked_rank(prev);
    for (int r = 0; r < MAX_SERP; r++)
        prob[r] = private_value(0, q[r].get_param_index()) * public_value(ubm_slot(r, prev[r]));
}

void UBM_Hst::get_log_conditional_click_probs(SERP_Hst& q, std::vector<float>& out) {
    int prev[MAX_SERP];
    q.prev_clicked_rank(prev);
    for (int r = 0; r < MAX_SERP; r++) {
        const float ae = private_value(0, q[r].get_param_index()) * public_value(ubm_slot(r, prev[r]));
        out.push_back(q[r].get_click() == 1 ? std::log(ae) : std::log(1 - ae));
    }
}

void UBM_Hst::get_full_click_probs(SERP_Hst& q, std::vector<float>& out) {
    // Marginal click probability of rank r: a sum over the rank of the
    // previous click (none = -1, whose slot is 9), each term the probability
    // of that click, of no click in between, and of a click at r.
    float marg[MAX_SERP];
    for (int r = 0; r < MAX_SERP; r++) {
        const float a = private_value(0, q[r].get_param_index());
        float cp = 0;
        for (int pc = -1; pc < r; pc++) {
            const int slot_prev = pc == -1 ? 9 : pc;
            float none_between = 1.f;
            for (int b = pc + 1; b < r; b++)
                none_between *= 1 - private_value(0, q[b].get_param_index()) * public_value(ubm_slot(b, slot_prev));
            const float t = none_between * (a * public_value(ubm_slot(r, slot_prev)));
            cp += pc >= 0 ? marg[pc] * t : t;
        }
        marg[r] = cp;
        out.push_back(q[r].get_click() == 1 ? cp : 1 - cp);
    }
}

// DBN / CCM: the conditional probability of what happened at each rank,
// given the ranks before it (get_serp_probability), is also the one whose
// log the log-likelihood takes.
void DBN_Hst::get_serp_probability(SERP_Hst& q, float (&prob)[MAX_SERP]) {
    const float g = public_value(0);
    float ex = 1.f;
    for (int r = 0; r < MAX_SERP; r++) {
        const int p = q[r].get_param_index();
        const float a = private_value(0, p), sv = private_value(1, p);
        if (q[r].get_click() == 1) {
            prob[r] = a * ex;
            ex = g * (1 - sv);
        } else {
            prob[r] = 1 - a * ex;
            ex *= g * (1 - a) / prob[r];
        }
    }
}

void DBN_Hst::get_log_conditional_click_probs(SERP_Hst& q, std::vector<float>& out) {
    float cp[MAX_SERP];
    get_serp_probability(q, cp);
    for (int r = 0; r < MAX_SERP; r++) out.push_back(std::log(cp[r]));
}

void DBN_Hst::get_full_click_probs(SERP_Hst& q, std::vector<float>& out) {
    const float g = public_value(0);
    float ex = 1.f;
    for (int r = 0; r < MAX_SERP; r++) {
        const int p = q[r].get_param_index();
        const float a = private_value(0, p), sv = private_value(1, p);
        const float ae = a * ex;
        out.push_back(q[r].get_click() == 1 ? ae : 1 - ae);
        ex *= g * (1 - a) + g * a * (1 - sv);
    }
}

void CCM_Hst::get_serp_probability(SERP_Hst& q, float (&prob)[MAX_SERP]) {
    const float t1 = public_value(0), t2 = public_value(1), t3 = public_value(2);
    float ex = 1.f;
    for (int r = 0; r < MAX_SERP; r++) {
        const float a = private_value(0, q[r].get_param_index());
        if (q[r].get_click() == 1) {
            prob[r] = a * ex;
            ex = t2 * (1 - a) + t3 * a;
        } else {
            prob[r] = 1 - a * ex;
            ex *= t1 * (1 - a) / prob[r];
        }
    }
}

void CCM_Hst::get_log_conditional_click_probs(SERP_Hst& q, std::vector<float>& out) {
    float cp[MAX_SERP];
    get_serp_probability(q, cp);
    for (int r = 0; r < MAX_SERP; r++) out.push_back(std::log(cp[r]));
}

void CCM_Hst::get_full_click_probs(SERP_Hst& q, std::vector<float>& out) {
    const float t1 = public_value(0), t2 = public_value(1), t3 = public_value(2);
    float ex = 1.f;
    for (int r = 0; r < MAX_SERP; r++) {
        const float a = private_value(0, q[r].get_param_index());
        const float ae = a * ex;
        out.push_back(q[r].get_click() == 1 ? ae : 1 - ae);
        ex *= (1 - a) * t1 + a * ((1 - a) * t2 + a * t3);
    }
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
    for (SERP_Hst session : testing_queries) {
        std::vector<float> lp;
        lp.reserve(MAX_SERP);
        cm_->get_log_conditional_click_probs(session, lp);
        llh_values_.push_back(std::accumulate(lp.begin(), lp.end(), 0.f) / MAX_SERP);
    }
    return std::accumulate(llh_values_.begin(), llh_values_.end(), 0.f);
}

void Perplexity::evaluate(ClickModel_Hst* cm, TrainSet& testing_queries) {
    task_size = static_cast<float>(testing_queries.size());
    for (SERP_Hst session : testing_queries) {
        std::vector<float> fp;
        fp.reserve(MAX_SERP);
        cm->get_full_click_probs(session, fp);
        for (int r = 0; r < MAX_SERP; r++) task_rank_perplexities[(size_t)r] += std::log2(fp[(size_t)r]);
    }
}

void Perplexity::import(std::array<float, MAX_SERP>& rank_perplexities, float& size) {
    task_rank_perplexities = rank_perplexities;
    task_size = size;
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
    cm->set_device(config.device, config.mode);
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
