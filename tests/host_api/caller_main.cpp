// A host program shaped like the reference's mclicks driver (main.cpp:149-448)
// with its MPI calls taken out: it fills a ProcessingConfig field by field
// from flags, describes the cluster with ClusterProperties, sizes
// LocalPartitions by the node's workers, calls the three-argument
// Dataset::parse_dataset and then em_parallel.  It is compiled against
// include/mclicks_host.hpp and linked with libmclicks.so by the tests, to show
// that code written against the reference's host API builds and runs on this
// one.
//
//   caller_main --raw-path LOG [--max-sessions N] [--itr K] [--model-type M]
//               [--test-share T] [--nodes N] [--parse-only 1]
#include <unistd.h>

#include <cstdio>
#include <functional>
#include <iostream>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "mclicks_host.hpp"

using namespace mclicks;

int main(int argc, char** argv) {
    ProcessingConfig config;
    config.total_nodes = 1;
    config.node_id = 0;
    ClusterProperties cluster_properties = local_cluster_properties(config);
    config.device_count = (int)cluster_properties.nodes[config.node_id].devices.size();
    int workers = config.device_count > 0 ? config.device_count : 1;

    std::map<int, std::string> supported_click_models{{0, "PBM"}, {1, "CCM"}, {2, "DBN"}, {3, "UBM"}};
    config.dataset_path = "YandexRelPredChallenge100k.txt";
    config.output_path = "";
    config.thread_count = (int)std::thread::hardware_concurrency();
    config.max_gpus = config.device_count;
    config.iterations = 50;
    config.max_sessions = 40000;
    config.model_type = 0;
    config.partitioning_type = 0;
    config.job_id = 0;
    config.exec_mode = 0;
    config.test_share = 0.2f;
    config.help = false;
    gethostname(config.host_name, HOST_NAME_MAX);

    bool parse_only = false;
    int nodes = 1;
    struct Option {
        std::string long_form, short_form;
        std::function<void(const char*)> handler;
    };
    std::vector<Option> options = {
        {"--raw-path", "-r", [&](const char* v) { config.dataset_path = v; }},
        {"--output", "-o", [&](const char* v) { config.output_path = v; }},
        {"--itr", "-i", [&](const char* v) { config.iterations = std::stoi(v); }},
        {"--max-sessions", "-s", [&](const char* v) { config.max_sessions = std::stoi(v); }},
        {"--model-type", "-m", [&](const char* v) { config.model_type = std::stoi(v); }},
        {"--test-share", "-t", [&](const char* v) { config.test_share = std::stof(v); }},
        {"--nodes", "-N", [&](const char* v) { nodes = std::stoi(v); }},
        {"--parse-only", "-P", [&](const char* v) { parse_only = std::stoi(v) != 0; }},
    };
    for (int i = 1; i + 1 < argc; i += 2) {
        const std::string name = argv[i];
        bool handled = false;
        for (const auto& o : options)
            if (name == o.long_form || name == o.short_form) {
                o.handler(argv[i + 1]);
                handled = true;
            }
        if (!handled) {
            std::cerr << "unknown flag " << name << std::endl;
            return 2;
        }
    }
    // A cluster of several nodes, as the reference's MPI launch would gather.
    config.total_nodes = nodes;
    while ((int)cluster_properties.nodes.size() < nodes) {
        cluster_properties.nodes.push_back(cluster_properties.nodes[0]);
        cluster_properties.node_count++;
    }
    std::vector<int> workers_per_node((size_t)config.total_nodes, workers);
    config.devices_per_node = workers_per_node.data();
    config.worker_count = workers;

    std::cout << "Job ID: " << config.job_id << "\nNumber of machines: " << config.total_nodes
              << "\nModel type: " << supported_click_models[config.model_type] << std::endl;
    for (const auto& node : cluster_properties.nodes)
        for (const auto& device : node.devices)
            std::cout << node.host.host_name << " " << device.device_name << " " << device.compute_capability << " "
                      << device.available_memory / 1e6 << std::endl;

    LocalPartitions device_partitions((size_t)workers);
    if (Dataset::parse_dataset(cluster_properties, config, device_partitions)) {
        std::cerr << "[" << config.host_name << "] Error: Unable to open the raw dataset." << std::endl;
        return 1;
    }
    for (size_t d = 0; d < device_partitions.size(); d++)
        std::cout << "PARTITION " << d << " " << std::get<0>(device_partitions[d]).size() << " "
                  << std::get<1>(device_partitions[d]).size() << " " << std::get<2>(device_partitions[d]) << std::endl;
    if (parse_only) return 0;
    em_parallel(config, device_partitions);
    return 0;
}
