// canon_enum.cpp -- frontier-batched orderly enumeration on top of the GPU check.
//
// The reference enumerates depth-first and checks one partial matrix at a time
// (CEnumerator::Enumerate, Source/Enumerator.cpp:540-1024, check at :446-447 and
// :364; alldata::Run, k-Factorization/TripleSys/Source/TripleSys.cpp:80-775, check
// at checkCurrentResult.cpp:91).  Here the search runs level by level: every
// canonical partial matrix of level n is extended by all admissible next rows on
// the host, the whole level is checked in batches on the GPU, and the canonical
// ones form level n+1.  Orderly generation makes the result independent of the
// visiting order: every prefix of a canonical matrix is canonical, so the set of
// canonical complete matrices is the same as the depth-first search finds.
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

// ---- BIBD rows -------------------------------------------------------------
// The next row is chosen as a number of 1s per column orbit (the row solutions of
// CRowSolution / CInSysSolver): r ones in total, lambda in common with every row
// above, no column above k, and columns that need all remaining rows forced.
struct BibdGen {
    int v, b, r, k, lambda;
    const uint64_t *rows;     // the n rows of the parent
    int n;
    int norb;
    int start[64], len[64], weight[64];
    uint64_t onesmask[64];    // bit i: row i has 1s in this orbit
    int x[64];
    int lam_left[16];
    std::vector<uint64_t> *out;

    void emit() {
        uint64_t row = 0;
        for (int q = 0; q < norb; ++q)
            if (x[q])
                row |= ((1ull << x[q]) - 1ull) << start[q];
        out->insert(out->end(), rows, rows + n);
        out->push_back(row);
    }
    void rec(int q, int left) {
        if (q == norb) {
            if (left)
                return;
            for (int i = 0; i < n; ++i)
                if (lam_left[i])
                    return;
            emit();
            return;
        }
        // capacity left in the orbits after q bounds the choice
        int cap_after = 0;
        for (int t = q + 1; t < norb; ++t)
            cap_after += (weight[t] < k) ? len[t] : 0;
        const int rem_rows = v - n - 1;
        int minx = (k - weight[q] > rem_rows) ? len[q] : 0;
        int maxx = (weight[q] >= k) ? 0 : len[q];
        if (maxx > left)
            maxx = left;
        if (minx < left - cap_after)
            minx = left - cap_after;
        for (int xv = maxx; xv >= minx; --xv) {
            bool ok = true;
            for (int i = 0; i < n; ++i)
                if (((onesmask[q] >> i) & 1u) && lam_left[i] < xv) {
                    ok = false;
                    break;
                }
            if (!ok)
                continue;
            for (int i = 0; i < n; ++i)
                if ((onesmask[q] >> i) & 1u)
                    lam_left[i] -= xv;
            x[q] = xv;
            rec(q + 1, left - xv);
            for (int i = 0; i < n; ++i)
                if ((onesmask[q] >> i) & 1u)
                    lam_left[i] += xv;
        }
    }
    void children(const uint64_t *parent, int nrows, std::vector<uint64_t> &dst) {
        rows = parent;
        n = nrows;
        out = &dst;
        // orbits of level n: runs of columns equal in rows 0..n-1
        norb = 0;
        int s = 0;
        for (int c = 1; c <= b; ++c) {
            bool same = c < b;
            for (int i = 0; same && i < n; ++i)
                if (((rows[i] >> c) & 1u) != ((rows[i] >> (c - 1)) & 1u))
                    same = false;
            if (!same) {
                start[norb] = s;
                len[norb] = c - s;
                int w = 0;
                uint64_t om = 0;
                for (int i = 0; i < n; ++i)
                    if ((rows[i] >> s) & 1u) {
                        ++w;
                        om |= 1ull << i;
                    }
                weight[norb] = w;
                onesmask[norb] = om;
                ++norb;
                s = c;
            }
        }
        for (int i = 0; i < n; ++i)
            lam_left[i] = lambda;
        rec(0, r);
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

// children of every parent of a level, generated on all host cores; the
// concatenation keeps the parents' order, so the result does not depend on the
// number of threads
template <typename Gen, typename T>
void level_children(const Gen &proto, const std::vector<T> &level, size_t stride, int n, std::vector<T> &out) {
    const size_t parents = level.size() / stride;
    unsigned nt = std::thread::hardware_concurrency();
    if (nt < 1)
        nt = 1;
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

int canon_enumerate_bibd(canon_ctx *ctx, uint32_t v, uint32_t b, uint32_t r, uint32_t k, uint32_t lambda,
                         canon_design_cb cb, void *user, canon_enum_stats *stats) {
    if (!ctx || v < 2 || v > 16 || b < 1 || b > 63 || r < 1 || r > b || k < 1 || k > v)
        return CANON_EINVAL;
    Timer t;
    canon_enum_stats st{};
    // row 0 is forced: r ones first
    std::vector<uint64_t> level = {(1ull << r) - 1ull};
    int n = 1;
    BibdGen gen{};
    gen.v = (int)v;
    gen.b = (int)b;
    gen.r = (int)r;
    gen.k = (int)k;
    gen.lambda = (int)lambda;
    const uint32_t chunk = canon::batch_capacity(ctx, v, 0);
    if (!chunk)
        return CANON_ENOMEM;
    while (n < (int)v && !level.empty()) {
        std::vector<uint64_t> cand;
        level_children(gen, level, (size_t)n, n, cand);
        const int m = n + 1;
        const size_t count = cand.size() / m;
        const bool complete = m == (int)v;
        std::vector<uint64_t> next;
        for (size_t off = 0; off < count; off += chunk) {
            const uint32_t cnt = (uint32_t)((count - off < chunk) ? count - off : chunk);
            canon_bibd_batch bt{cnt, (uint32_t)m, b, complete ? CANON_COMPLETE : 0u, cand.data() + off * m, nullptr};
            int rc = canon_submit_bibd(ctx, &bt);
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
                const uint64_t *rowsp = cand.data() + (off + i) * m;
                if (complete) {
                    ++st.designs;
                    if (cb)
                        cb(user, (const uint8_t *)rowsp, v, b, res.aut[2 * i], res.aut[2 * i + 1]);
                } else {
                    next.insert(next.end(), rowsp, rowsp + m);
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
        level_children(gen, level, (size_t)n * np, n, cand);
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
