// canon_kenum_rounds.h -- the next rounds of a partial k-system with groups of 3 or 4 and
// the links test, host code (canon_enumerate_ksys_groups builds every level's candidates
// with it on the host cores; a host build tests it).
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>

namespace canon {
namespace kenum {

inline int ctz32(unsigned x) { return __builtin_ctz(x); }

// The pairs not yet used (bit y of free[x]: x and y have not met) must still split into
// groups: for every player, the players it has not met must fall into groups of g - 1
// that have not met each other either, or no later rounds complete the matrix.  The links
// test of the reference (CChecklLink::checkLinksV, k-Factorization/TripleSys/Source/
// checkLinksV.cpp, applied to every player in checkLinks.cpp:60-110) for groups of 3,
// generalised to groups of 4.  A necessary condition only: it drops matrices that no
// complete matrix extends, so the complete matrices found are the same with it.
inline bool split_into_groups(unsigned set, const uint32_t *free, int k);

// take `need` more members of a group (pairwise unmet, from cand), then split the rest
inline bool pick_members(unsigned set, unsigned cand, const uint32_t *free, int k, int need) {
    if (!need)
        return split_into_groups(set, free, k);
    while (cand) {
        const int w = ctz32(cand);
        cand &= cand - 1u;
        if (pick_members(set & ~(1u << w), cand & free[w], free, k, need - 1))
            return true;
    }
    return false;
}

inline bool split_into_groups(unsigned set, const uint32_t *free, int k) {
    if (!set)
        return true;
    const int v = ctz32(set);
    const unsigned rest = set & ~(1u << v);
    return pick_members(rest, rest & free[v], free, k, k - 1);
}

inline bool links_complete(const uint32_t *used, int np, int g) {
    const unsigned all = (1u << np) - 1u;
    uint32_t free[16];
    for (int x = 0; x < np; ++x)
        free[x] = all & ~used[x] & ~(1u << x);
    for (int x = 0; x < np; ++x)
        if (free[x] && !split_into_groups(free[x], free, g - 1))
            return false;
    return true;
}

// The rounds that may follow a parent of d rounds: every partition of the np players
// into groups of g that repeats no pair of an earlier round, written in result() form
// (players ascending inside a group, groups ordered by their first player), whose second
// entry (the first partner of player 0) is above the parent's last one, so that the rounds
// stay ordered by their second entry, and after which the unmet pairs still split into
// groups (links_complete).  Appended to out as parent + round.
struct RoundBuilder {
    int np, g, d;
    int second;            // the first partner of player 0 (the round's second entry)
    bool links;            // apply links_complete to the children
    const uint8_t *parent;
    uint32_t used[16];
    uint8_t row[16];
    std::vector<uint8_t> *out;

    void emit() {
        uint32_t u[16];
        std::memcpy(u, used, sizeof(u));
        for (int q = 0; q < np; q += g)
            for (int e = 0; e < g; ++e)
                for (int f = e + 1; f < g; ++f) {
                    u[row[q + e]] |= 1u << row[q + f];
                    u[row[q + f]] |= 1u << row[q + e];
                }
        if (links && !links_complete(u, np, g))
            return;
        out->insert(out->end(), parent, parent + (size_t)d * np);
        out->insert(out->end(), row, row + np);
    }
    // position pos starts a group: its first player is the lowest one not taken
    void group(unsigned taken, int pos) {
        if (pos == np) {
            emit();
            return;
        }
        const int a = ctz32(~taken);
        row[pos] = (uint8_t)a;
        const int minp = a == 0 ? parent[(size_t)(d - 1) * np + 1] + 1 : a + 1;
        const unsigned all = (1u << np) - 1u;
        partner(taken | (1u << a), pos + 1, 1, all & ~(taken | (1u << a)) & ~used[a], minp);
    }
    // the k-th member of the group at positions pos-k .. : a player of `allowed` >= minp
    void partner(unsigned taken, int pos, int k, unsigned allowed, int minp) {
        if (k == g) {
            group(taken, pos);
            return;
        }
        unsigned m = allowed & ~((1u << minp) - 1u);
        if (pos == 1)
            m &= 1u << second;
        while (m) {
            const int p = ctz32(m);
            m &= m - 1u;
            row[pos] = (uint8_t)p;
            partner(taken | (1u << p), pos + 1, k + 1, allowed & ~used[p] & ~(1u << p), p + 1);
        }
    }
    void run() {
        std::memset(used, 0, sizeof(used));
        for (int r = 0; r < d; ++r)
            for (int q = 0; q < np; q += g)
                for (int e = 0; e < g; ++e)
                    for (int f = e + 1; f < g; ++f) {
                        const int x = parent[(size_t)r * np + q + e], y = parent[(size_t)r * np + q + f];
                        used[x] |= 1u << y;
                        used[y] |= 1u << x;
                    }
        group(0u, 0);
    }
};

}  // namespace kenum
}  // namespace canon
