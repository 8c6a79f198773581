// canon_workload.cpp -- seeded partial designs made by random backtracking of their rows:
// the inputs of an uneven batched check (partial matrices of several shapes and fill
// depths, as an orderly enumerator meets them).
//
// An incidence item is built row by row.  Each row is a random admissible row for the
// rows above it -- weight r, lambda common columns with every earlier row, no column
// above k ones, and no column left short of k ones with the rows that remain -- found
// by a randomised depth-first search over the columns.  When a level has no admissible
// row, the row above is dropped and drawn again (backtracking).  The rows are the
// reference enumerator's row constraints (a row solution of C_InSysEnumerator,
// Source/Enumerator.cpp:726-975 with MakeRow, Source/MatrixCanonChecker.cpp:14-93), but
// drawn at random rather than in order, so the partial matrices include dead ends that
// no complete design extends.  A Steiner triple system with v-1 or v rows filled is a
// complete design (v-1 admissible rows of an STS(v) determine the last one), which
// random row-by-row backtracking reaches only rarely; such items, and any whose
// search budget runs out, are taken from a complete random STS(v) made by Stinson's
// hill-climbing under a uniform row and column permutation.  A k-system item is built round by round the same way:
// round 0 is (0 1)(2 3)..., every further round a random perfect matching of pairs not
// used before, written as result() holds it (pairs ascending, ordered by first player);
// the rounds are then ordered by the partner of player 0.  Item i uses its own stream (seed, i), so the output does not depend on the threads.
#include <sched.h>

#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/canon_gb300.h"
#include "canon_sts.cuh"

namespace {

uint32_t below(uint64_t &s, uint32_t n) { return canon::rand_below(s, n); }

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

template <typename F>
void parallel_items(uint32_t n, F &&f) {
    unsigned nt = host_threads();
    if (nt > 64)
        nt = 64;
    if (n < 1024)
        nt = 1;
    if (nt == 1) {
        for (uint32_t i = 0; i < n; ++i)
            f(i);
        return;
    }
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nt; ++t)
        th.emplace_back([&, t] {
            const uint32_t lo = (uint32_t)((uint64_t)n * t / nt), hi = (uint32_t)((uint64_t)n * (t + 1) / nt);
            for (uint32_t i = lo; i < hi; ++i)
                f(i);
        });
    for (auto &x : th)
        x.join();
}

// ---- incidence matrices ------------------------------------------------------
struct RowDraw {
    uint32_t v, b, r, k, lam;
    uint64_t rows[16];
    uint8_t col[64];           // ones per column in rows 0..j-1
    uint8_t order[64];         // the random column order of the current draw
    uint32_t inter[16];        // common columns of the row being drawn with each earlier row
    uint64_t budget;           // search nodes left for this item
    uint64_t *rng;

    // columns order[t..b-1] still open; the row has `w` ones so far
    bool dfs(uint32_t j, uint32_t t, uint32_t w, uint64_t row) {
        if (!budget)
            return false;
        --budget;
        if (w == r) {
            for (uint32_t i = 0; i < j; ++i)
                if (inter[i] != lam)
                    return false;
            // a column that row j leaves empty must still reach k ones with the rows below
            const uint32_t left = v - j - 1;
            for (uint32_t c = 0; c < b; ++c)
                if (!((row >> c) & 1u) && col[c] + left < k)
                    return false;
            rows[j] = row;
            return true;
        }
        if (t == b || b - t < r - w)
            return false;
        // every earlier row must still be able to reach lambda common columns
        for (uint32_t i = 0; i < j; ++i) {
            if (inter[i] > lam)
                return false;
            uint32_t avail = 0;
            for (uint32_t q = t; q < b; ++q)
                avail += (uint32_t)((rows[i] >> order[q]) & 1u);
            if (inter[i] + avail < lam)
                return false;
        }
        const uint32_t c = order[t];
        const bool one_first = below(*rng, 2) != 0;
        for (int pass = 0; pass < 2; ++pass) {
            const bool one = (pass == 0) == one_first;
            if (one) {
                if (col[c] >= k)
                    continue;
                bool ok = true;
                for (uint32_t i = 0; i < j; ++i)
                    if (((rows[i] >> c) & 1u) && inter[i] >= lam)
                        ok = false;
                if (!ok)
                    continue;
                for (uint32_t i = 0; i < j; ++i)
                    inter[i] += (uint32_t)((rows[i] >> c) & 1u);
                const bool found = dfs(j, t + 1, w + 1, row | (1ull << c));
                for (uint32_t i = 0; i < j; ++i)
                    inter[i] -= (uint32_t)((rows[i] >> c) & 1u);
                if (found)
                    return true;
            } else {
                // a column left empty here must still reach k ones in the rows below
                if (col[c] + (v - j - 1) < k)
                    continue;
                if (dfs(j, t + 1, w, row))
                    return true;
            }
            if (!budget)
                return false;
        }
        return false;
    }

    bool draw(uint32_t j) {
        for (uint32_t c = 0; c < b; ++c)
            order[c] = (uint8_t)c;
        for (uint32_t c = b; c > 1; --c) {
            const uint32_t q = below(*rng, c);
            const uint8_t t = order[c - 1];
            order[c - 1] = order[q];
            order[q] = t;
        }
        std::memset(inter, 0, sizeof(inter));
        return dfs(j, 0, 0, 0ull);
    }

    // rows 0..m-1; false if the item's budget ran out
    bool build(uint32_t m) {
        std::memset(col, 0, sizeof(col));
        uint32_t j = 0;
        uint32_t fails = 0;
        while (j < m) {
            if (!budget)
                return false;
            if (draw(j)) {
                for (uint32_t c = 0; c < b; ++c)
                    col[c] += (uint8_t)((rows[j] >> c) & 1u);
                ++j;
            } else if (j > 0) {
                // no admissible row below: drop the row above and draw it again; after
                // many such steps start the item afresh
                --j;
                for (uint32_t c = 0; c < b; ++c)
                    col[c] -= (uint8_t)((rows[j] >> c) & 1u);
                if (++fails > 4 * v)
                    j = 0, std::memset(col, 0, sizeof(col)), fails = 0;
            } else {
                return false;
            }
        }
        return true;
    }
};

// ---- k-system rounds ------------------------------------------------------------
struct RoundDraw {
    uint32_t np;
    uint8_t rounds[16][16];
    bool used[16][16];
    uint64_t budget;
    uint64_t *rng;

    bool match(uint8_t *row, uint32_t pos, unsigned taken) {
        if (!budget)
            return false;
        --budget;
        if (pos == np)
            return true;
        uint32_t a = 0;
        while (taken & (1u << a))
            ++a;
        uint8_t cand[16];
        uint32_t nc = 0;
        for (uint32_t c = a + 1; c < np; ++c)
            if (!(taken & (1u << c)) && !used[a][c])
                cand[nc++] = (uint8_t)c;
        for (uint32_t q = nc; q > 1; --q) {
            const uint32_t x = below(*rng, q);
            const uint8_t t = cand[q - 1];
            cand[q - 1] = cand[x];
            cand[x] = t;
        }
        for (uint32_t q = 0; q < nc; ++q) {
            row[pos] = (uint8_t)a;
            row[pos + 1] = cand[q];
            if (match(row, pos + 2, taken | (1u << a) | (1u << cand[q])))
                return true;
            if (!budget)
                return false;
        }
        return false;
    }
    void mark(uint32_t d, bool on) {
        for (uint32_t i = 0; i < np; i += 2)
            used[rounds[d][i]][rounds[d][i + 1]] = used[rounds[d][i + 1]][rounds[d][i]] = on;
    }
    bool build(uint32_t m) {
        std::memset(used, 0, sizeof(used));
        for (uint32_t i = 0; i < np; ++i)
            rounds[0][i] = (uint8_t)i;
        mark(0, true);
        uint32_t d = 1, fails = 0;
        while (d < m) {
            if (!budget)
                return false;
            if (match(rounds[d], 0, 0u)) {
                mark(d, true);
                ++d;
            } else if (d > 1) {
                // no matching left: drop the round above and draw it again; after many
                // such steps start the item afresh
                --d;
                mark(d, false);
                if (++fails > 4 * np) {
                    while (d > 1)
                        mark(--d, false);
                    fails = 0;
                }
            } else {
                return false;
            }
        }
        return true;
    }
};

constexpr uint64_t ITEM_BUDGET = 1ull << 20;   // search nodes per item (all attempts)

}  // namespace

extern "C" {

int canon_generate_partial_bibd(uint32_t v, uint32_t b, uint32_t r, uint32_t k, uint32_t lambda, uint32_t n,
                                uint64_t seed, uint32_t min_rows, uint32_t max_rows, uint64_t *rows,
                                uint8_t *nrows, uint32_t *n_from_complete) {
    if (v < 2 || v > 16 || b < 2 || b > 63 || !r || r > b || !k || k > v || lambda > r || min_rows < 1 ||
        min_rows > max_rows || max_rows > v || (n && (!rows || !nrows)))
        return CANON_EINVAL;
    const bool sts = k == 3 && lambda == 1 && r == (v - 1) / 2 && b == v * (v - 1) / 6 && v <= 15 &&
                     (v % 6 == 1 || v % 6 == 3);
    std::atomic<bool> ok{true};
    std::atomic<uint32_t> from_complete{0};
    parallel_items(n, [&](uint32_t i) {
        uint64_t s = seed ^ ((uint64_t)i * 0xD1B54A32D192ED03ull);
        const uint32_t m = min_rows + below(s, max_rows - min_rows + 1);
        RowDraw g{};
        g.v = v, g.b = b, g.r = r, g.k = k, g.lam = lambda;
        g.budget = ITEM_BUDGET;
        g.rng = &s;
        bool built = false;
        if (!(sts && m + 1 >= v))
            built = g.build(m);
        if (!built && sts) {
            // a complete STS(v) under a uniform row permutation: its first m rows
            canon::sts_random_rows(v, s, g.rows);
            built = true;
            from_complete.fetch_add(1);
        }
        uint64_t *dst = rows + (size_t)i * v;
        for (uint32_t q = 0; q < v; ++q)
            dst[q] = (built && q < m) ? g.rows[q] : 0ull;
        nrows[i] = built ? (uint8_t)m : 0;
        if (!built)
            ok.store(false);
    });
    if (n_from_complete)
        *n_from_complete = from_complete.load();
    return ok.load() ? CANON_OK : CANON_ETIMEOUT;
}

int canon_generate_partial_ksys(uint32_t np, uint32_t n, uint64_t seed, uint32_t min_rounds, uint32_t max_rounds,
                                uint8_t *data, uint8_t *nrows) {
    if (np < 4 || np > 12 || (np & 1u) || min_rounds < 1 || min_rounds > max_rounds || max_rounds > np - 1 ||
        (n && (!data || !nrows)))
        return CANON_EINVAL;
    const uint32_t rounds = np - 1;
    std::atomic<bool> ok{true};
    parallel_items(n, [&](uint32_t i) {
        uint64_t s = seed ^ ((uint64_t)i * 0xD1B54A32D192ED03ull);
        const uint32_t m = min_rounds + below(s, max_rounds - min_rounds + 1);
        RoundDraw g{};
        g.np = np;
        g.budget = ITEM_BUDGET;
        g.rng = &s;
        const bool built = g.build(m);
        uint8_t *dst = data + (size_t)i * rounds * np;
        std::memset(dst, 0, (size_t)rounds * np);
        if (built) {
            // rounds ordered by the partner of player 0, as the enumerator lays them out
            uint8_t order[16];
            for (uint32_t d = 0; d < m; ++d)
                order[d] = (uint8_t)d;
            for (uint32_t d = 1; d < m; ++d)
                for (uint32_t e = d; e > 0 && g.rounds[order[e]][1] < g.rounds[order[e - 1]][1]; --e) {
                    const uint8_t t = order[e];
                    order[e] = order[e - 1];
                    order[e - 1] = t;
                }
            for (uint32_t d = 0; d < m; ++d)
                std::memcpy(dst + d * np, g.rounds[order[d]], np);
        }
        nrows[i] = built ? (uint8_t)m : 0;
        if (!built)
            ok.store(false);
    });
    return ok.load() ? CANON_OK : CANON_ETIMEOUT;
}

}  // extern "C"
