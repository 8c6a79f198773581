// canon_kenum.cu -- orderly enumeration of k-systems with groups of 3 or 4 (resolvable
// designs with blocks of 3 or 4 such as the Kirkman triple systems of 15 players): the
// next rounds of every canonical parent are built on the host cores, checked in batches
// by the GPU check of canon_submit_ksys_groups (kgen_seg_kernel), and the canonical
// ones kept.  The work of alldata::Run() for group size 3 or 4 with the check at every
// level (k-Factorization/TripleSys/Source/TripleSys.cpp:80-775, rounds built by
// processOneDay()/getNextPlayer() :487-775, check at checkCurrentResult.cpp:91).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/canon_gb300.h"
#include "canon_ctx.h"
#include "canon_internal.h"
#include "canon_hostpool.h"
#include "canon_kenum_rounds.h"

namespace {

using canon::kenum::RoundBuilder;

// the children of every parent (in parent order), built on up to 16 host threads; the
// unit of work is (parent, second entry of the new round), so the single parent of the
// first level is split too, and units in order give the children in order
void build_level(const std::vector<uint8_t> &parents, int d, int np, int g, std::vector<uint8_t> &out) {
    const size_t pl = (size_t)d * np, n = parents.size() / pl;
    std::vector<std::pair<uint32_t, uint8_t>> units;
    for (size_t i = 0; i < n; ++i)
        for (int b = parents[i * pl + (size_t)(d - 1) * np + 1] + 1; b < np; ++b)
            units.emplace_back((uint32_t)i, (uint8_t)b);
    const size_t nu = units.size();
    // The links test drops almost nothing while more than half of the rounds are still to
    // come (the 15-player triples: 20 of 16,450 children with 3 rounds, none with 2) and
    // costs more than building the rounds, so it runs once at most half remain (69,795 ->
    // 298 children with 4 rounds).
    const int total_rounds = (np - 1) / (g - 1), left = total_rounds - (d + 1);
    const bool links = 2 * left <= total_rounds - 1;
    canon::HostPool &pool = canon::HostPool::get();
    const unsigned nt = nu < 2 ? 1u : (nu < pool.threads() ? (unsigned)nu : pool.threads());
    std::vector<std::vector<uint8_t>> part(nt);
    const std::function<void(unsigned)> work = [&](unsigned t) {
        for (size_t k = nu * t / nt; k < nu * (t + 1) / nt; ++k) {
            RoundBuilder rb;
            rb.np = np;
            rb.g = g;
            rb.d = d;
            rb.second = units[k].second;
            rb.links = links;
            rb.parent = parents.data() + (size_t)units[k].first * pl;
            rb.out = &part[t];
            rb.run();
        }
    };
    if (nt == 1)
        work(0);
    else
        pool.run(nt, work);
    out.clear();
    for (auto &p : part)
        out.insert(out.end(), p.begin(), p.end());
}

}  // namespace

extern "C" int canon_enumerate_ksys_groups(canon_ctx *c, uint32_t np, uint32_t g, canon_design_cb cb, void *user,
                                           canon_enum_stats *stats) {
    if (!c)
        return CANON_EINVAL;
    if (g == 2)
        return canon_enumerate_ksys(c, np, cb, user, stats);
    if ((g != 3 && g != 4) || np > 16 || np % g || np / g < 2 || (np - 1) % (g - 1)) {
        c->err = "enumerate ksys groups: group size 3 or 4, np <= 16 a multiple of it with (np - 1) a "
                 "multiple of g - 1";
        return CANON_EINVAL;
    }
    if (c->n_bitems || c->n_kitems) {
        c->err = "enumerate ksys groups: the context's queue must be empty (canon_sync first)";
        return CANON_EINVAL;
    }
    const auto t0 = std::chrono::steady_clock::now();
    const int rounds = (int)((np - 1) / (g - 1));
    canon_enum_stats st{};
    // the check's |Aut| and relabelings tried are read back: no verdict-only sync here
    const uint32_t saved_options = c->cfg.options;
    c->cfg.options &= ~CANON_OPT_VERDICT_SYNC;
    std::vector<uint8_t> parents(np), children, kept;
    for (uint32_t p = 0; p < np; ++p)
        parents[p] = (uint8_t)p;
    int rc = CANON_OK;
    for (int d = 1; d < rounds && !parents.empty() && rc == CANON_OK; ++d) {
        const auto g0 = std::chrono::steady_clock::now();
        build_level(parents, d, (int)np, (int)g, children);
        const double gs = std::chrono::duration<double>(std::chrono::steady_clock::now() - g0).count();
        st.gen_seconds += gs;
        st.level_gen_ms[d] += 1e3 * gs;
        const size_t cl = (size_t)(d + 1) * np, m = children.size() / cl;
        st.level_checks[d] += m;
        st.checks += m;
        kept.clear();
        const uint32_t cap = canon::batch_capacity(c, 0, (uint32_t)cl);
        if (!cap) {
            c->err = "enumerate ksys groups: the context holds no matrix of this size";
            rc = CANON_ENOMEM;
            break;
        }
        for (size_t lo = 0; lo < m && rc == CANON_OK; lo += cap) {
            const uint32_t n = (uint32_t)std::min<size_t>(cap, m - lo);
            canon_ksys_batch bt{};
            bt.n = n;
            bt.np = np;
            bt.rounds = (uint32_t)(d + 1);
            bt.data = children.data() + lo * cl;
            rc = canon_submit_ksys_groups(c, &bt, g);
            canon_results r{};
            if (rc == CANON_OK)
                rc = canon_sync(c, &r);
            if (rc != CANON_OK)
                break;
            ++st.batches;
            st.kernel_ms += r.kernel_ms;
            st.level_kernel_ms[d] += r.kernel_ms;
            for (uint32_t i = 0; i < n; ++i) {
                st.trials += r.trials[i];
                if (r.status[i]) {
                    c->err = "enumerate ksys groups: a built round was refused by the check";
                    rc = CANON_EINVAL;
                    break;
                }
                if (!r.canonical[i])
                    continue;
                const uint8_t *child = children.data() + (lo + i) * cl;
                if (d + 1 == rounds) {
                    ++st.designs;
                    if (cb)
                        cb(user, child, (uint32_t)rounds, np, r.aut[2 * (size_t)i], r.aut[2 * (size_t)i + 1]);
                } else {
                    kept.insert(kept.end(), child, child + cl);
                }
            }
        }
        st.levels = (uint32_t)d;
        parents.swap(kept);
    }
    c->cfg.options = saved_options;
    st.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (stats)
        *stats = st;
    return rc;
}
