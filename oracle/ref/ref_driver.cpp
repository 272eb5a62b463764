// Driver for the reference's own CPU training path, compiled out of tree from
// the reference sources (see Makefile beside this file).  Test infrastructure:
// it produces the golden vectors that pin the oracle; nothing in the product
// links it.
//
// It replaces the reference's main.cpp, which cannot run on a host without a
// GPU (main.cpp:106-111 dereferences the maximum of an empty device list).  The
// configuration it builds is the reference's CPU-only mode with one node and
// one worker (main.cpp:200-213, 290-300).
//
// Commands (all write into OUTDIR):
//   ingest     DATASET MAX_SESSIONS TEST_SHARE OUTDIR
//       Dataset::parse_dataset (dataset.cpp:421-455) and a dump of the
//       partition: train/test query ids, doc ids, clicks, parameter indices.
//   em         DATASET MAX_SESSIONS TEST_SHARE MODEL ITERS THREADS OUTDIR DUMP_EVERY
//       ingest, then the CPU EM loop of em_parallel (parallel_em.cu:462-609,
//       exec_mode 1) driven through the ClickModel_Hst virtuals, dumping every
//       parameter (numerator, denominator) after selected iterations, then the
//       reference's LogLikelihood / Perplexity on the test set
//       (evaluation.cpp:25-66) and the final reduction (parallel_em.cu:697-723).
//   em_parallel DATASET MAX_SESSIONS TEST_SHARE MODEL ITERS THREADS [OUT_PREFIX]
//       ingest, then the unmodified em_parallel() itself (prints its log lines
//       and, with OUT_PREFIX, writes its parameter CSVs).

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>
#include <array>
#include <numeric>
#include <cmath>
#include <thread>
#include <chrono>
#include <unistd.h>
#include <climits>

#include "utils/definitions.h"
#include "utils/types.h"
#include "utils/utils.cuh"
#include "parallel_em/parallel_em.cuh"
#include "parallel_em/communicator.h"
#include "data/dataset.h"
#include "click_models/base.cuh"
#include "click_models/evaluation.h"

// Defined in parallel_em.cu (non-static there).
void allocate_threads_to_devices(const ProcessingConfig& config, std::vector<std::vector<int>>& thread_start_idx,
                                 const LocalPartitions& device_partitions, int total_queries);
void calculate_queries_per_thread(const ProcessingConfig& config, std::vector<std::vector<int>>& thread_start_idx,
                                  const LocalPartitions& device_partitions);
int calculate_total_queries(const LocalPartitions& device_partitions);

static void write_blob(const std::string& path, const void* data, size_t bytes) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) { perror(path.c_str()); exit(2); }
    if (bytes) fwrite(data, 1, bytes, f);
    fclose(f);
}

static void dump_set(const std::string& dir, const std::string& name, const std::vector<SERP_Hst>& set) {
    size_t n = set.size();
    std::vector<int> q(n), doc(n * MAX_SERP), pidx(n * MAX_SERP);
    std::vector<unsigned char> click(n * MAX_SERP);
    for (size_t i = 0; i < n; i++) {
        q[i] = set[i].get_query();
        for (int r = 0; r < MAX_SERP; r++) {
            SearchResult_Hst sr = set[i][r];
            doc[i * MAX_SERP + r] = sr.get_doc_id();
            pidx[i * MAX_SERP + r] = sr.get_param_index();
            click[i * MAX_SERP + r] = (unsigned char)sr.get_click();
        }
    }
    write_blob(dir + "/" + name + "_query.i32", q.data(), q.size() * 4);
    write_blob(dir + "/" + name + "_doc.i32", doc.data(), doc.size() * 4);
    write_blob(dir + "/" + name + "_pidx.i32", pidx.data(), pidx.size() * 4);
    write_blob(dir + "/" + name + "_click.u8", click.data(), click.size());
}

struct Setup {
    ProcessingConfig config;
    ClusterProperties cluster;
    int devices_per_node[1];
    LocalPartitions partitions;
};

static void make_setup(Setup& s, const char* dataset, int max_sessions, float test_share, int model, int iters, int threads) {
    ProcessingConfig& c = s.config;
    c.dataset_path = dataset;
    c.output_path = "";
    c.job_id = 0;
    c.max_sessions = max_sessions;
    c.model_type = model;
    c.partitioning_type = 0;
    c.node_id = 0;
    c.total_nodes = 1;
    c.thread_count = threads;
    s.devices_per_node[0] = 1;
    c.devices_per_node = s.devices_per_node;
    c.iterations = iters;
    c.exec_mode = 1;
    c.test_share = test_share;
    c.device_count = 0;
    c.max_gpus = 0;
    c.worker_count = 1;
    c.help = false;
    strncpy(c.host_name, "oracle-host", HOST_NAME_MAX - 1);
    c.host_name[HOST_NAME_MAX - 1] = 0;

    s.cluster.node_count = 1;
    s.cluster.device_count = 0;
    NodeProperties node;
    node.host.node_id = 0;
    node.host.device_count = 0;
    node.host.thread_count = threads;
    node.host.free_memory = (size_t)64 << 30;
    node.host.total_memory = (size_t)64 << 30;
    strncpy(node.host.host_name, c.host_name, HOST_NAME_MAX);
    s.cluster.nodes.push_back(node);

    s.partitions.resize(1);
    if (Dataset::parse_dataset(s.cluster, c, s.partitions)) {
        fprintf(stderr, "cannot open dataset %s\n", dataset);
        exit(2);
    }
}

static void dump_partition(const Setup& s, const std::string& outdir) {
    const Partition& p = s.partitions[0];
    dump_set(outdir, "train", std::get<0>(p));
    dump_set(outdir, "test", std::get<1>(p));
    FILE* f = fopen((outdir + "/meta.txt").c_str(), "w");
    fprintf(f, "%zu %zu %d\n", std::get<0>(p).size(), std::get<1>(p).size(), std::get<2>(p));
    fclose(f);
}

static void dump_params(ClickModel_Hst* cm, const std::string& path) {
    std::vector<std::vector<Param>> all;
    cm->get_parameters(all, ALL);
    std::vector<float> flat;
    for (auto& v : all)
        for (auto& p : v) { flat.push_back(p.numerator_val()); flat.push_back(p.denominator_val()); }
    write_blob(path, flat.data(), flat.size() * 4);
}

int main(int argc, char** argv) {
    if (argc < 2) { fprintf(stderr, "usage: ref_driver ingest|em|em_parallel ...\n"); return 2; }
    std::string cmd = argv[1];
    int n_nodes = 1, node_id = 0;
    Communicate::initiate(argc, argv, n_nodes, node_id);

    if (cmd == "ingest" && argc == 6) {
        Setup s;
        make_setup(s, argv[2], atoi(argv[3]), (float)atof(argv[4]), 0, 1, 1);
        dump_partition(s, argv[5]);
    } else if (cmd == "em" && argc == 10) {
        Setup s;
        int model = atoi(argv[5]), iters = atoi(argv[6]), threads = atoi(argv[7]);
        std::string outdir = argv[8];
        int dump_every = atoi(argv[9]);
        make_setup(s, argv[2], atoi(argv[3]), (float)atof(argv[4]), model, iters, threads);
        dump_partition(s, outdir);

        Partition& part = s.partitions[0];
        ClickModel_Hst* cm = create_cm_host(model);
        cm->init_parameters(part, (size_t)64 << 30, false);
        // Thread start indices exactly as em_parallel computes them
        // (parallel_em.cu:377-383).
        std::vector<std::vector<int>> tsi(1);
        allocate_threads_to_devices(s.config, tsi, s.partitions, calculate_total_queries(s.partitions));
        calculate_queries_per_thread(s.config, tsi, s.partitions);
        std::vector<int>& start_idx = tsi[0];
        double total = 0;
        for (int itr = 0; itr < iters; itr++) {
            auto t0 = std::chrono::steady_clock::now();
            cm->process_session(std::get<0>(part), start_idx);
            cm->reset_parameters(false);
            cm->update_parameters(std::get<0>(part), start_idx);
            auto t1 = std::chrono::steady_clock::now();
            total += std::chrono::duration<double>(t1 - t0).count();
            if (dump_every > 0 && ((itr + 1) % dump_every == 0 || itr + 1 == iters)) {
                char name[64];
                snprintf(name, sizeof(name), "/params_%04d.f32", itr + 1);
                dump_params(cm, outdir + name);
            }
        }
        LogLikelihood llh(cm);
        float llh_val = llh.evaluate(std::get<1>(part));
        Perplexity ppl;
        ppl.evaluate(cm, std::get<1>(part));
        float task_size = (float)std::get<1>(part).size();
        // Final reduction as in em_parallel (parallel_em.cu:697-723), one worker.
        float total_llh = llh_val / task_size;
        std::array<float, 10> ppl_rank{};
        for (int i = 0; i < 10; i++) ppl_rank[i] = std::pow(2, (-1 * ppl.task_rank_perplexities[i]) / ppl.task_size);
        float ppl_value = std::accumulate(ppl_rank.begin(), ppl_rank.end(), 0.0) / 10.0;
        FILE* f = fopen((outdir + "/eval.txt").c_str(), "w");
        fprintf(f, "llh_sum %a\nn_test %a\nllh %a\nppl %a\n", llh_val, task_size, total_llh, ppl_value);
        for (int i = 0; i < 10; i++) fprintf(f, "log2sum_%d %a\nppl_%d %a\n", i, ppl.task_rank_perplexities[i], i, ppl_rank[i]);
        fprintf(f, "seconds_per_iteration %.9f\n", total / (iters > 0 ? iters : 1));
        fclose(f);
    } else if (cmd == "em_parallel" && (argc == 8 || argc == 9)) {
        Setup s;
        make_setup(s, argv[2], atoi(argv[3]), (float)atof(argv[4]), atoi(argv[5]), atoi(argv[6]), atoi(argv[7]));
        if (argc == 9) s.config.output_path = argv[8];  // parameter CSVs (communicator.cpp:423-516)
        em_parallel(s.config, s.partitions);
    } else {
        fprintf(stderr, "bad arguments for %s\n", cmd.c_str());
        return 2;
    }
    return 0;
}
