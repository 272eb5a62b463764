// mclicks: command-line trainer with the reference's flags (main.cpp:223-236).
//
//   mclicks --raw-path LOG --max-sessions N --itr K --model-type M --test-share T [--output PREFIX]
//
// Model ids: 0 PBM, 1 CCM, 2 DBN, 3 UBM.  --n-threads, --n-gpus,
// --partition-type, --job-id and --exec-mode are accepted for compatibility
// (one GPU, GPU execution).  Added: --device D (CUDA device), --mode
// parity|clean (statistics of slots the E-step does not write).
#include <chrono>
#include <functional>
#include <iomanip>
#include <iostream>
#include <map>
#include <string>
#include <thread>
#include <vector>

#include "mclicks_host.hpp"

using namespace mclicks;

static void show_help() {
    std::cout << "Usage: mclicks [options]\n"
                 "  --raw-path, -r PATH        click log in the reference's text format\n"
                 "  --max-sessions, -s N       sessions to read (default 40000; -1 = all)\n"
                 "  --itr, -i K                EM iterations (default 50)\n"
                 "  --model-type, -m M         0 PBM, 1 CCM, 2 DBN, 3 UBM (default 0)\n"
                 "  --test-share, -t T         share of sessions held out for testing (default 0.2)\n"
                 "  --output, -o PREFIX        write <PREFIX>_<parameter>.csv files\n"
                 "  --device, -d D             CUDA device (default 0)\n"
                 "  --mode parity|clean        statistics of unwritten slots (default parity)\n"
                 "  --n-threads, -n, --n-gpus, -g, --partition-type, -p, --job-id, -j, --exec-mode, -e\n"
                 "                             accepted for compatibility\n"
                 "  --help, -h\n";
}

int main(int argc, char** argv) {
    using clock = std::chrono::steady_clock;
    auto t_start = clock::now();
    ProcessingConfig config;
    config.thread_count = (int)std::thread::hardware_concurrency();
    struct Option {
        std::string long_form, short_form;
        std::function<void(const char*)> handler;
    };
    std::vector<Option> options = {
        {"--n-threads", "-n", [&](const char* v) { config.thread_count = std::stoi(v); }},
        {"--n-gpus", "-g", [&](const char* v) { config.max_gpus = std::stoi(v); }},
        {"--raw-path", "-r", [&](const char* v) { config.dataset_path = v; }},
        {"--output", "-o", [&](const char* v) { config.output_path = v; }},
        {"--itr", "-i", [&](const char* v) { config.iterations = std::stoi(v); }},
        {"--max-sessions", "-s", [&](const char* v) { config.max_sessions = std::stoi(v); }},
        {"--model-type", "-m", [&](const char* v) { config.model_type = std::stoi(v); }},
        {"--partition-type", "-p", [&](const char* v) { config.partitioning_type = std::stoi(v); }},
        {"--test-share", "-t", [&](const char* v) { config.test_share = std::stof(v); }},
        {"--job-id", "-j", [&](const char* v) { config.job_id = std::stoi(v); }},
        {"--exec-mode", "-e", [&](const char* v) { config.exec_mode = std::stoi(v); }},
        {"--device", "-d", [&](const char* v) { config.device = std::stoi(v); }},
        {"--mode", "", [&](const char* v) { config.mode = std::string(v) == "clean" ? MC_MODE_CLEAN : MC_MODE_PARITY; }},
        {"--help", "-h", [&](const char*) { config.help = true; }},
    };
    for (int i = 1; i < argc; i += 2) {
        std::string name = argv[i];
        const char* value = i + 1 < argc ? argv[i + 1] : "";
        bool handled = false;
        try {
            for (const auto& o : options)
                if (name == o.long_form || (!o.short_form.empty() && name == o.short_form)) {
                    o.handler(value);
                    handled = true;
                    break;
                }
        } catch (const std::exception&) {
            std::cerr << "Error: Invalid argument '" << value << "' for flag '" << name << "'." << std::endl;
            config.help = true;
        }
        if (!handled && name.rfind("-", 0) == 0) {
            std::cerr << "Error: Did not recognize flag '" << name << "'." << std::endl;
            config.help = true;
        }
    }
    if (config.help) {
        show_help();
        return 0;
    }
    if (config.model_type < 0 || config.model_type > 3) config.model_type = 0;  // base.cu:41-45
    static const std::map<int, std::string> names = {{0, "PBM"}, {1, "CCM"}, {2, "DBN"}, {3, "UBM"}};
    std::cout << "Job ID: " << config.job_id << "\nNumber of machines: 1\nNumber of workers: 1"
              << "\nExecution mode: GPU-only\nRaw data path: " << config.dataset_path
              << "\nNumber of EM iterations: " << config.iterations
              << "\nShare of data used for testing: " << config.test_share * 100 << "%"
              << "\nMax number of sessions: " << config.max_sessions
              << "\nModel type: " << names.at(config.model_type) << std::endl << std::endl;

    std::cout << "Parsing dataset..." << std::endl;
    auto t0 = clock::now();
    LocalPartitions partitions;
    if (Dataset::parse_dataset(config, partitions)) {
        std::cerr << "Error: Unable to open the raw dataset." << std::endl;
        return 1;
    }
    double pre = std::chrono::duration<double>(clock::now() - t0).count();
    std::cout << "Train " << std::get<0>(partitions[0]).size() << " Test " << std::get<1>(partitions[0]).size()
              << " QD Pairs " << std::get<2>(partitions[0]) << std::endl;
    auto t1 = clock::now();
    try {
        em_parallel(config, partitions);
    } catch (const std::exception& e) {
        std::cerr << "Error: " << e.what() << std::endl;
        return 1;
    }
    double em = std::chrono::duration<double>(clock::now() - t1).count();
    double total = std::chrono::duration<double>(clock::now() - t_start).count();
    std::cout << std::endl << std::fixed << std::setprecision(7)
              << std::left << std::setw(27) << "Pre-processing time: " << pre << " seconds" << std::endl
              << std::left << std::setw(27) << "Parameter estimation time: " << em << " seconds" << std::endl
              << std::left << std::setw(27) << "Total elapsed time: " << total << " seconds" << std::endl;
    return 0;
}
