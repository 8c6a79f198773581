// canon_enum.cpp -- frontier-batched orderly enumeration of k-systems on top of
// the GPU check (the BIBD enumerator keeps its levels on the GPU: canon_levels.cu).
//
// The reference enumerates depth-first and checks one partial matrix at a time
// (alldata::Run, k-Factorization/TripleSys/Source/TripleSys.cpp:80-775, check at
// checkCurrentResult.cpp:91).  Here the search runs level by level: every
// canonical partial matrix of level n is extended by all admissible next rounds
// on the host, the whole level is checked in batches on the GPU, and the
// canonical ones form level n+1.  Orderly generation makes the result independent of the
// visiting order: every prefix of a canonical matrix is canonical, so the set of
// canonical complete matrices is the same as the depth-first search finds.
#include <sched.h>

#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/canon_gb300.h"

namespace canon {
uint32_t batch_capacity(const canon_ctx *c, uint32_t words, uint32_t bytes);
}

namespace {

struct Timer {
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    double seconds() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

// ---- k-system rounds -------------------------------------------------------
// Round d is a perfect matching of pairs not used before, written as result()
// holds it (pairs ascending, ordered by first player); player 0 meets d+1, as in
// every canonical matrix (rounds sorted by their second entry).
struct KsysGen {
    int np;
    const uint8_t *parent;
    int d;
    bool used[16][16];
    uint8_t row[16];
    std::vector<uint8_t> *out;

    void rec(int pos, unsigned taken) {
        if (pos == np) {
            out->insert(out->end(), parent, parent + d * np);
            out->insert(out->end(), row, row + np);
            return;
        }
        int a = 0;
        while (taken & (1u << a))
            ++a;
        for (int c = a + 1; c < np; ++c) {
            if ((taken & (1u << c)) || used[a][c])
                continue;
            if (a == 0 && c != d + 1)
                continue;
            row[pos] = (uint8_t)a;
            row[pos + 1] = (uint8_t)c;
            rec(pos + 2, taken | (1u << a) | (1u << c));
        }
    }
    void children(const uint8_t *p, int nrounds, std::vector<uint8_t> &dst) {
        parent = p;
        d = nrounds;
        out = &dst;
        std::memset(used, 0, sizeof(used));
        for (int r = 0; r < nrounds; ++r)
            for (int i = 0; i < np; i += 2)
                used[p[r * np + i]][p[r * np + i + 1]] = used[p[r * np + i + 1]][p[r * np + i]] = true;
        rec(0, 0);
    }
};

// the host cores this process may run on (its CPU affinity), not every core of
// the machine: a container or a job slot often holds fewer
unsigned host_threads() {
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

// children of every parent of a level, generated on all host cores; the
// concatenation keeps the parents' order, so the result does not depend on the
// number of threads
template <typename Gen, typename T>
void level_children(const Gen &proto, const std::vector<T> &level, size_t stride, int n, std::vector<T> &out) {
    const size_t parents = level.size() / stride;
    unsigned nt = host_threads();
    if (nt > 32)
        nt = 32;
    if (parents < 64)
        nt = 1;
    std::vector<std::vector<T>> part(nt);
    auto work = [&](unsigned t) {
        Gen g = proto;
        const size_t lo = parents * t / nt, hi = parents * (t + 1) / nt;
        for (size_t p = lo; p < hi; ++p)
            g.children(level.data() + p * stride, n, part[t]);
    };
    if (nt == 1) {
        work(0);
    } else {
        std::vector<std::thread> th;
        for (unsigned t = 0; t < nt; ++t)
            th.emplace_back(work, t);
        for (auto &x : th)
            x.join();
    }
    out.clear();
    for (auto &v : part)
        out.insert(out.end(), v.begin(), v.end());
}

}  // namespace

extern "C" {

int canon_enumerate_ksys(canon_ctx *ctx, uint32_t np, canon_design_cb cb, void *user, canon_enum_stats *stats) {
    if (!ctx || np < 4 || np > 12 || (np & 1u))
        return CANON_EINVAL;
    Timer t;
    canon_enum_stats st{};
    std::vector<uint8_t> level(np);
    for (uint32_t i = 0; i < np; ++i)
        level[i] = (uint8_t)i;
    int n = 1;
    KsysGen gen{};
    gen.np = (int)np;
    const uint32_t chunk = canon::batch_capacity(ctx, 0, np * (np - 1));
    if (!chunk)
        return CANON_ENOMEM;
    const int rounds = (int)np - 1;
    while (n < rounds && !level.empty()) {
        std::vector<uint8_t> cand;
        Timer tg;
        level_children(gen, level, (size_t)n * np, n, cand);
        st.gen_seconds += tg.seconds();
        const int m = n + 1;
        const size_t count = cand.size() / (m * np);
        std::vector<uint8_t> next;
        for (size_t off = 0; off < count; off += chunk) {
            const uint32_t cnt = (uint32_t)((count - off < chunk) ? count - off : chunk);
            canon_ksys_batch bt{cnt, np, (uint32_t)m, 0u, cand.data() + off * m * np, nullptr};
            int rc = canon_submit_ksys(ctx, &bt);
            canon_results res{};
            if (rc == CANON_OK)
                rc = canon_sync(ctx, &res);
            if (rc != CANON_OK)
                return rc;
            st.checks += cnt;
            st.kernel_ms += res.kernel_ms;
            st.level_checks[m - 1] += cnt;
            st.level_kernel_ms[m - 1] += res.kernel_ms;
            ++st.batches;
            for (uint32_t i = 0; i < cnt; ++i) {
                if (!res.canonical[i])
                    continue;
                const uint8_t *mp = cand.data() + (off + i) * m * np;
                if (m == rounds) {
                    ++st.designs;
                    if (cb)
                        cb(user, mp, (uint32_t)m, np, res.aut[2 * i], 0);
                } else {
                    next.insert(next.end(), mp, mp + m * np);
                }
            }
        }
        level.swap(next);
        n = m;
        ++st.levels;
    }
    st.seconds = t.seconds();
    if (stats)
        *stats = st;
    return CANON_OK;
}

}  // extern "C"
