// Persistent host thread pool (see pool.h).
//
// Every worker takes part in every job: run() publishes the job under the
// lock, wakes all workers, takes tasks itself, and returns once each worker
// has reported the job done, so no worker can still hold a job that has
// returned.  The pool is created on first use and never destroyed (its threads
// sleep between jobs and end with the process); a process forked after it was
// created gets a new pool, since the threads do not exist in the child.
#include "pool.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <vector>
#include <unistd.h>

namespace mch {
namespace {

class Pool {
public:
    explicit Pool(size_t n_workers) {
        for (size_t i = 0; i < n_workers; i++) workers_.emplace_back([this] { loop(); });
    }

    size_t size() const { return workers_.size(); }

    void run(size_t n, const std::function<void(size_t)>& fn) {
        std::lock_guard<std::mutex> one(run_mu_);
        {
            std::lock_guard<std::mutex> lk(mu_);
            job_ = &fn;
            n_ = n;
            next_.store(0);
            pending_ = workers_.size();
            gen_++;
        }
        cv_work_.notify_all();
        for (size_t i; (i = next_.fetch_add(1)) < n;) fn(i);
        std::unique_lock<std::mutex> lk(mu_);
        cv_done_.wait(lk, [&] { return pending_ == 0; });
        job_ = nullptr;
    }

private:
    void loop() {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_work_.wait(lk, [&] { return gen_ != seen; });
            seen = gen_;
            const std::function<void(size_t)>* fn = job_;
            const size_t n = n_;
            lk.unlock();
            for (size_t i; (i = next_.fetch_add(1)) < n;) (*fn)(i);
            lk.lock();
            if (--pending_ == 0) cv_done_.notify_all();
        }
    }

    std::vector<std::thread> workers_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_work_, cv_done_;
    const std::function<void(size_t)>* job_ = nullptr;
    size_t n_ = 0, pending_ = 0;
    uint64_t gen_ = 0;
    std::atomic<size_t> next_{0};
};

std::mutex g_pool_mu;
Pool* g_pool = nullptr;  // deliberately never freed
pid_t g_pool_pid = 0;

Pool& pool() {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool || g_pool_pid != getpid()) {
        const size_t hw = std::max<size_t>(1, std::thread::hardware_concurrency());
        g_pool = new Pool(hw - 1);
        g_pool_pid = getpid();
    }
    return *g_pool;
}

}  // namespace

void parallel_for(size_t n, const std::function<void(size_t)>& fn) {
    if (n == 0) return;
    if (n == 1) {
        fn(0);
        return;
    }
    pool().run(n, fn);
}

size_t pool_threads() { return pool().size() + 1; }

}  // namespace mch
