// Stress of the library's host thread pool (csrc/host/pool.cpp): many jobs of
// random sizes, most smaller than the number of workers, each index run
// exactly once.  One array is reused by every job, so a worker that ran a
// finished job's function would show as a second hit.
#include "pool.h"

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

int main(int argc, char** argv) {
    const long jobs = argc > 1 ? std::atol(argv[1]) : 20000;
    std::mt19937 rng(7);
    std::vector<std::atomic<int>> hits(4096);
    long bad = 0;
    for (long j = 0; j < jobs; j++) {
        const size_t n = 2 + rng() % (j % 3 == 0 ? 4000 : 40);
        for (size_t i = 0; i < n; i++) hits[i].store(0);
        mch::parallel_for(n, [&](size_t i) { hits[i].fetch_add(1); });
        for (size_t i = 0; i < n; i++) bad += hits[i].load() != 1;
    }
    std::printf("JOBS %ld BAD %ld THREADS %zu\n", jobs, bad, mch::pool_threads());
    return bad != 0;
}
