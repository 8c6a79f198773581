// canon_hostpool.h -- a persistent pool of host threads for the host-side work around
// the kernels (packing batches, building enumeration levels on the host cores).
#pragma once
#include <sched.h>

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace canon {

// Host threads kept for the work around the kernels: starting and joining 16 threads
// costs about 0.35 ms on a Grace host, a quarter of the submit of a 100 MB batch.  run(n, job)
// calls job(0 .. n-1) on the calling thread and the pool's, and returns when every call has
// ended and no pool thread still holds the job.  Calls from several host threads are
// serialised.  The pool lives until the process ends (its threads wait for work).
class HostPool {
  public:
    static HostPool &get() {
        static HostPool *pool = new HostPool();
        return *pool;
    }
    // fn(lo, hi) over [0, n) in contiguous ranges, four per thread of the pool, taken in
    // turn by whichever thread is free (the work per element may vary)
    template <typename F>
    void ranges(uint64_t n, F fn) {
        const unsigned nt = threads();
        if (nt < 2 || n < 2) {
            fn((uint64_t)0, n);
            return;
        }
        const unsigned parts = n < 4ull * nt ? (unsigned)n : 4u * nt;
        const std::function<void(unsigned)> job = [&](unsigned t) { fn(n * t / parts, n * (t + 1) / parts); };
        run(parts, job);
    }
    unsigned threads() const { return (unsigned)workers_.size() + 1u; }
    void run(unsigned n, const std::function<void(unsigned)> &job) {
        std::lock_guard<std::mutex> serial(run_mu_);
        {
            std::lock_guard<std::mutex> lk(mu_);
            job_ = &job;
            n_ = n;
            done_ = 0;
            next_.store(0);
            ++gen_;
        }
        cv_work_.notify_all();
        const unsigned k = take(job, n);
        std::unique_lock<std::mutex> lk(mu_);
        done_ += k;
        cv_done_.wait(lk, [&] { return done_ == n_ && active_ == 0; });
        job_ = nullptr;
    }

  private:
    // the host cores this process may run on (its CPU affinity), not every core of the
    // machine: a container or a job slot often holds fewer
    static unsigned host_cores() {
        cpu_set_t set;
        CPU_ZERO(&set);
        if (sched_getaffinity(0, sizeof(set), &set) == 0) {
            const int c = CPU_COUNT(&set);
            if (c > 0)
                return (unsigned)c;
        }
        const unsigned n = std::thread::hardware_concurrency();
        return n ? n : 1;
    }
    HostPool() {
        unsigned nt = host_cores();
        nt = nt > 16 ? 16 : nt;
        for (unsigned t = 1; t < nt; ++t)
            workers_.emplace_back([this] { loop(); });
        for (auto &w : workers_)
            w.detach();
    }
    unsigned take(const std::function<void(unsigned)> &job, unsigned n) {
        unsigned k = 0;
        for (unsigned t; (t = next_.fetch_add(1)) < n; ++k)
            job(t);
        return k;
    }
    void loop() {
        uint64_t seen = 0;
        for (;;) {
            std::unique_lock<std::mutex> lk(mu_);
            cv_work_.wait(lk, [&] { return gen_ != seen && job_ != nullptr; });
            seen = gen_;
            const std::function<void(unsigned)> *job = job_;
            const unsigned n = n_;
            ++active_;
            lk.unlock();
            const unsigned k = take(*job, n);
            lk.lock();
            done_ += k;
            --active_;
            if (done_ == n_ && active_ == 0)
                cv_done_.notify_all();
        }
    }
    std::vector<std::thread> workers_;
    std::mutex run_mu_, mu_;
    std::condition_variable cv_work_, cv_done_;
    const std::function<void(unsigned)> *job_ = nullptr;
    unsigned n_ = 0, done_ = 0, active_ = 0;
    uint64_t gen_ = 0;
    std::atomic<unsigned> next_{0};
};


}  // namespace canon
