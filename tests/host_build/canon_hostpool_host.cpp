// canon_hostpool_host.cpp -- the persistent host thread pool (canon_hostpool.h) compiled
// for the host (test only): every job index runs exactly once per call, ranges cover
// [0, n) without overlap, and calls from several host threads are serialised.
#include <atomic>
#include <thread>
#include <vector>

#include "../../incidence-system-enumeration_gb300/csrc/canon_hostpool.h"

// runs `calls` pool calls of n jobs each, from `callers` host threads at once; returns the
// number of (call, job) executions that did not happen exactly once (0 = correct)
extern "C" long emu_pool_run(unsigned n, unsigned calls, unsigned callers) {
    std::atomic<long> bad{0};
    auto body = [&]() {
        for (unsigned c = 0; c < calls; ++c) {
            std::vector<std::atomic<int>> hits(n);
            for (auto &h : hits)
                h.store(0);
            const std::function<void(unsigned)> job = [&](unsigned t) { hits[t].fetch_add(1); };
            canon::HostPool::get().run(n, job);
            for (auto &h : hits)
                if (h.load() != 1)
                    bad.fetch_add(1);
        }
    };
    std::vector<std::thread> th;
    for (unsigned k = 1; k < callers; ++k)
        th.emplace_back(body);
    body();
    for (auto &t : th)
        t.join();
    return bad.load();
}

// ranges(n): returns the number of elements of [0, n) not covered exactly once
extern "C" long emu_pool_ranges(unsigned long long n) {
    std::vector<std::atomic<int>> hits(n);
    for (auto &h : hits)
        h.store(0);
    canon::HostPool::get().ranges(n, [&](uint64_t lo, uint64_t hi) {
        for (uint64_t i = lo; i < hi; ++i)
            hits[i].fetch_add(1);
    });
    long bad = 0;
    for (auto &h : hits)
        bad += h.load() != 1;
    return bad;
}

extern "C" unsigned emu_pool_threads() { return canon::HostPool::get().threads(); }
