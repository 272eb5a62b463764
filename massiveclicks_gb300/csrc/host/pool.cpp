// Persistent host thread pool (see pool.h).
//
// run() publishes a job under the lock, wakes the workers, takes tasks itself
// and returns once all n tasks have completed.  Tasks are claimed from one
// 64-bit ticket that carries the job's generation in its high half and the
// next task index in its low half, so a worker can only claim tasks of the job
// it woke for: one that wakes late, after its job has returned, finds the
// generation changed or no index left and never calls the job's function.  A
// job therefore waits for its tasks, not for every worker to wake (one worker
// scheduled late would otherwise hold the whole job).  The pool is created on
// first use and never destroyed (its threads sleep between jobs and end with
// the process); a process forked after it was created gets a new pool, since
// the threads do not exist in the child.
#include "pool.h"

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
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
        uint64_t g;
        {
            std::lock_guard<std::mutex> lk(mu_);
            g = ++gen_;
            job_ = &fn;
            n_ = n;
            done_ = 0;
            ticket_.store((g & 0xFFFFFFFFu) << 32);
        }
        cv_work_.notify_all();
        work(g, fn, n);
        std::unique_lock<std::mutex> lk(mu_);
        cv_done_.wait(lk, [&] { return done_ == n; });
        job_ = nullptr;
    }

private:
    // Claims and runs tasks of generation g while any are left, then adds the
    // number run to done_.  fn stays valid meanwhile: run() waits for done_
    // to reach n, which counts every task claimed.
    void work(uint64_t g, const std::function<void(size_t)>& fn, size_t n) {
        const uint64_t tag = g & 0xFFFFFFFFu;
        size_t mine = 0;
        uint64_t t = ticket_.load();
        while ((t >> 32) == tag && (t & 0xFFFFFFFFu) < n) {
            if (!ticket_.compare_exchange_weak(t, t + 1)) continue;  // t reloaded
            fn((size_t)(t & 0xFFFFFFFFu));
            mine++;
            t = ticket_.load();
        }
        if (mine) {
            std::lock_guard<std::mutex> lk(mu_);
            done_ += mine;
            if (done_ == n_) cv_done_.notify_all();
        }
    }

    void loop() {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_work_.wait(lk, [&] { return gen_ != seen; });
            seen = gen_;
            const std::function<void(size_t)>* fn = job_;
            const size_t n = n_;
            lk.unlock();
            if (fn) work(seen, *fn, n);
            lk.lock();
        }
    }

    std::vector<std::thread> workers_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_work_, cv_done_;
    const std::function<void(size_t)>* job_ = nullptr;
    size_t n_ = 0, done_ = 0;
    uint64_t gen_ = 0;
    std::atomic<uint64_t> ticket_{0};
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
