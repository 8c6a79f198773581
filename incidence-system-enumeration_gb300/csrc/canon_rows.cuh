// canon_rows.cuh -- the admissible next rows of a partial BIBD incidence matrix,
// as host and device code (the device enumerator runs it one thread per parent;
// a host build of the same code is tested against the oracle's enumeration).
//
// The next row is chosen as a number of 1s per column orbit of the parent (the
// row solutions that CRowSolution / CInSysSolver enumerate, Source/RowSolution.h,
// Source/InSysSolver.h): r ones in total, lambda in common with every row above,
// no column above k, columns that need every remaining row forced to 1, and no
// earlier row i that the new row beats after a swap: exchanging rows i and n and
// moving the new row's 1s first inside every column orbit of rows 0..i-1 leaves
// rows 0..i-1 as they are, so a greater row i there means a greater matrix and
// the child is not canonical.  Inside each orbit the 1s come first, so every
// child is again in orbit normal form.
//
// Automorphisms of the parent prune children too (the grouping of row solutions by
// the parent's automorphism group, CRowSolution::sortSolutionsByGroup(),
// Source/RowSolution.h:325-383, with the group built by CPermutStorage::constructGroup()
// and the orbit representative found by findSolutionIndex(), Source/PermutStorage.h:
// 183-335).  An automorphism of the parent permutes its rows by sigma and its column
// orbits along: the orbit whose columns hold 1s in the rows of a set P goes to the
// orbit of the rows sigma(P).  Applied to a child it keeps the parent and moves the
// new row's 1s from orbit to orbit, giving an isomorphic child; if that child's row
// is greater (read orbit by orbit, more 1s first), the child is not the greatest of
// its class and cannot be canonical.  Each automorphism given and its inverse are
// tried; a subset of the group prunes less but never wrongly.
#pragma once
#include <cstddef>
#include <cstdint>

#ifdef __CUDACC__
#define CANON_HD __host__ __device__
#else
#define CANON_HD
#endif

namespace canon {
namespace rows {

struct Params {
    int v, b, r, k, lambda;
};

// What children() writes for child j < out_cap: nothing, the whole child at
// out[j*(n+1) .. j*(n+1)+n] (the parent's rows, then the new row), or the new
// row alone at out[j].
enum Emit { COUNT = 0, CHILD = 1, NEW_ROW = 2 };

// at most this many automorphisms of a parent prune its children
constexpr int AUT_GENS = 8;

// one byte per row (rows 0-7 in w[0], 8-15 in w[1])
constexpr uint64_t B64 = 0x4040404040404040ull;    // 64 in every byte
constexpr uint64_t HIB = 0x8080808080808080ull;    // the high bit of every byte
constexpr uint64_t LOW7 = 0x7F7F7F7F7F7F7F7Full;
constexpr uint64_t ONE8 = 0x0101010101010101ull;
struct Bytes16 {
    uint64_t w[2];
    // += / -= v times the 0/1 bytes of m (v <= 63: no byte leaves 0..127)
    CANON_HD void add(const Bytes16 &m, unsigned v) {
        w[0] += m.w[0] * v;
        w[1] += m.w[1] * v;
    }
    CANON_HD void sub(const Bytes16 &m, unsigned v) {
        w[0] -= m.w[0] * v;
        w[1] -= m.w[1] * v;
    }
};

// bit j of m (j < 8) -> byte j, as 0 or 1
CANON_HD inline uint64_t spread8(unsigned m) {
    const uint64_t v = ((uint64_t)(m & 0xFFu) * 0x0101010101010101ull) & 0x8040201008040201ull;
    return (((v + 0x7F7F7F7F7F7F7F7Full) | v) >> 7) & 0x0101010101010101ull;
}
// bit i of m (i < 16) -> byte i of the two words
CANON_HD inline Bytes16 spread16(unsigned m) { return Bytes16{{spread8(m & 0xFFu), spread8((m >> 8) & 0xFFu)}}; }

// Children of one parent with n rows (bit c of word i = row i, column c), in a
// fixed order: orbits left to right, more 1s first.  Returns their number.
// gens: ngens automorphisms of the parent as row permutations (nibble i = the row
// that goes to position i), or none.
template <int EMIT>
CANON_HD uint32_t children(const Params &d, const uint64_t *parent, int n, uint64_t *out, uint32_t out_cap,
                           const uint64_t *gens = nullptr, int ngens = 0) {
    const int b = d.b, k = d.k;
    uint8_t start[64], len[64], weight[64];
    uint8_t split[64];      // the first row in which orbit q differs from orbit q-1
    uint16_t ones[64];
    int norb = 0;
    int s = 0;
    for (int c = 1; c <= b; ++c) {
        bool same = c < b;
        for (int i = 0; same && i < n; ++i)
            if (((parent[i] >> c) & 1u) != ((parent[i] >> (c - 1)) & 1u))
                same = false;
        if (!same) {
            int first = 0;
            while (norb && first < n && ((parent[first] >> s) & 1u) == ((parent[first] >> (s - 1)) & 1u))
                ++first;
            split[norb] = (uint8_t)first;
            start[norb] = (uint8_t)s;
            len[norb] = (uint8_t)(c - s);
            int w = 0;
            unsigned om = 0;
            for (int i = 0; i < n; ++i)
                if ((parent[i] >> s) & 1u) {
                    ++w;
                    om |= 1u << i;
                }
            weight[norb] = (uint8_t)w;
            ones[norb] = (uint16_t)om;
            ++norb;
            s = c;
        }
    }
    // the orbit map of every automorphism: orbit q (1s in the rows of ones[q]) goes to
    // the orbit with 1s in the rows sigma(ones[q])
    uint8_t omap[AUT_GENS][64];
    int na = 0;
    for (int a = 0; a < ngens && a < AUT_GENS; ++a) {
        const uint64_t sg = gens[a];
        bool good = true;
        for (int t = 0; t < norb && good; ++t) {
            unsigned img = 0;
            for (int i = 0; i < n; ++i)
                if ((ones[t] >> i) & 1u)
                    img |= 1u << ((sg >> (4 * i)) & 15u);
            int u = 0;
            while (u < norb && ones[u] != img)
                ++u;
            if (u == norb)
                good = false;      // not an automorphism of this parent: not used
            else
                omap[na][t] = (uint8_t)u;
        }
        if (good)
            ++na;
    }
    // hi/lo: the most / least 1s orbit q can take (full orbits none, orbits whose
    // columns need every remaining row all).  Per row i, with one byte per row in two
    // 64-bit words (rows 0-7, 8-15): LAM = the 1s row i still needs in common with the
    // new row, plus 64; RC / RN = the sums of hi / lo over the orbits from the current
    // one on that meet row i.  A value xv for orbit q is admissible when every row
    // keeps RN - lo[q] <= lam - xv <= RC - hi[q] (rows in the orbit; the others keep
    // RN <= lam <= RC), tested for all rows at once: bytes stay in 0..127, so
    // ((a | 0x80) - b) has its byte's high bit set exactly when a >= b.  A row whose
    // lambda can no longer be met ends the branch at once.
    const int rem_rows = d.v - n - 1;
    uint8_t hi[64], lo[64];
    // rows 0..n-1 need lambda (byte 64 + lambda), rows past n nothing (byte 64)
    const unsigned rows_mask = (n >= 16) ? 0xFFFFu : ((1u << n) - 1u);
    Bytes16 rc{{0, 0}}, rn{{0, 0}};
    Bytes16 lamb{{spread8(rows_mask & 0xFFu) * (uint64_t)d.lambda + B64,
                  spread8(rows_mask >> 8) * (uint64_t)d.lambda + B64}};
    int ca = 0, cn = 0;
    for (int q = 0; q < norb; ++q) {
        hi[q] = (weight[q] >= k) ? 0 : len[q];
        lo[q] = (k - weight[q] > rem_rows) ? len[q] : 0;
        ca += hi[q];
        cn += lo[q];
        const Bytes16 m = spread16(ones[q]);
        rc.add(m, hi[q]);
        rn.add(m, lo[q]);
    }
    // iterative depth-first search over the orbits: x[q] the 1s given to orbit q,
    // nxt[q] the next value to try, left[q] the 1s still to place before orbit q,
    // tied bit q: the row equals row n-1 on the orbits before q
    uint8_t x[64], nxt[64], mn[64], left[65];
    // of the orbit q being filled: 1 in the bytes of the rows it meets, and RN - lo[q] + 64,
    // RC - hi[q] + 64
    Bytes16 mq{{0, 0}}, lo64{{0, 0}}, up64{{0, 0}};
    uint64_t tied = 1;
    uint32_t count = 0;
    int q = 0;
    left[0] = (uint8_t)d.r;
    // The walk is a state machine that takes one step per iteration -- set up an orbit,
    // try one value, back up one orbit, or test a leaf -- so that the threads of a warp,
    // which walk different parents, stay in step instead of each looping over its own
    // run of rejected values.  The children come in the order of the plain depth-first
    // walk.
    enum : int { ENTER = 0, TRY = 1, BACK = 2 };
    int state = ENTER;
    for (;;) {
        if (state == ENTER) {
            if (q == norb) {
                bool ok = left[q] == 0 && lamb.w[0] == B64 && lamb.w[1] == B64;
                // the swap test against every row i >= 1 (the orbits of level i are
                // runs of orbits not split by rows 0..i-1; row 0 has the same weight)
                for (int i = 1; ok && i < n; ++i) {
                    int c = 0, ri = 0;
                    for (int t = 0; t <= norb; ++t) {
                        if (t == norb || (t > 0 && split[t] < i)) {
                            if (c > ri)
                                ok = false;
                            if (c != ri || t == norb)
                                break;
                            c = ri = 0;
                        }
                        c += x[t];
                        ri += ((ones[t] >> i) & 1u) ? len[t] : 0;
                    }
                }
                // an automorphism of the parent (or its inverse) that makes the row greater
                for (int a = 0; ok && a < na; ++a) {
                    for (int dir = 0; dir < 2 && ok; ++dir) {
                        for (int t = 0; t < norb; ++t) {
                            // dir 0: image row y[omap[t]] = x[t]; dir 1: y[t] = x[omap[t]]
                            int yt;
                            if (dir) {
                                yt = x[omap[a][t]];
                            } else {
                                yt = -1;
                                for (int u = 0; u < norb; ++u)
                                    if (omap[a][u] == t)
                                        yt = x[u];
                            }
                            if (yt != x[t]) {
                                if (yt > x[t])
                                    ok = false;
                                break;
                            }
                        }
                    }
                }
                if (ok) {
                    if (EMIT != COUNT && count < out_cap) {
                        uint64_t row = 0;
                        for (int t = 0; t < norb; ++t)
                            if (x[t])
                                row |= ((1ull << x[t]) - 1ull) << start[t];
                        if (EMIT == CHILD) {
                            uint64_t *dst = out + (size_t)count * (n + 1);
                            for (int i = 0; i < n; ++i)
                                dst[i] = parent[i];
                            dst[n] = row;
                        } else {
                            out[count] = row;
                        }
                    }
                    ++count;
                }
                if (q == 0)
                    break;
                --q;
                mq = spread16(ones[q]);
                ca += hi[q];
                cn += lo[q];
                rc.add(mq, hi[q]);
                rn.add(mq, lo[q]);
                lo64 = rn;
                lo64.sub(mq, lo[q]);
                lo64.w[0] += B64;
                lo64.w[1] += B64;
                up64 = rc;
                up64.sub(mq, hi[q]);
                up64.w[0] += B64;
                up64.w[1] += B64;
                state = TRY;
                continue;
            }
            mq = spread16(ones[q]);
            const int lf = left[q];
            const int ca1 = ca - hi[q], cn1 = cn - lo[q];      // orbits after q
            int minx = lo[q], maxx = hi[q];
            if (maxx > lf)
                maxx = lf;
            if (minx < lf - ca1)
                minx = lf - ca1;
            if (maxx > lf - cn1)
                maxx = lf - cn1;
            if (((tied >> q) & 1u) && !((ones[q] >> (n - 1)) & 1u) && maxx > 0)
                maxx = 0;
            mn[q] = (uint8_t)(minx < 0 ? 0 : minx);
            nxt[q] = (uint8_t)(maxx + 1);          // values maxx .. minx, tried downwards
            x[q] = 0xFF;                           // nothing applied yet
            if (maxx < minx)
                nxt[q] = mn[q];                    // empty range
            lo64 = rn;
            lo64.sub(mq, lo[q]);
            lo64.w[0] += B64;
            lo64.w[1] += B64;
            up64 = rc;
            up64.sub(mq, hi[q]);
            up64.w[0] += B64;
            up64.w[1] += B64;
            state = TRY;
            continue;
        }
        if (state == TRY) {
            // undo the value applied at level q, then try the next one
            if (x[q] != 0xFF) {
                lamb.add(mq, x[q]);
                x[q] = 0xFF;
            }
            if (nxt[q] > mn[q]) {
                const int xv = --nxt[q];
                Bytes16 l = lamb;
                l.sub(mq, (unsigned)xv);
                // per row, with the 1s left after this orbit (left'), the capacities of the
                // later orbits (ca', cn') and their parts that meet row i (RC', RN'):
                //   RN' <= lam' <= RC'                  (byte high bits of a and bb)
                //   RC' - lam' <= ca' - left'           (the 1s outside row i's orbits fit)
                //   lam' - RN' <= left' - cn'           (and fill what must be filled)
                const int lf1 = left[q] - xv;
                const uint64_t k2 = ONE8 * (uint64_t)(ca - hi[q] - lf1) | HIB;
                const uint64_t k3 = ONE8 * (uint64_t)(lf1 - (cn - lo[q])) | HIB;
                uint64_t g = HIB;
#pragma unroll
                for (int w = 0; w < 2; ++w) {
                    const uint64_t a = (up64.w[w] | HIB) - l.w[w];      // 128 + RC' - lam'
                    const uint64_t bb = (l.w[w] | HIB) - lo64.w[w];     // 128 + lam' - RN'
                    g &= a & bb & (k2 - (a & LOW7)) & (k3 - (bb & LOW7));
                }
                if (g == HIB) {
                    lamb = l;
                    x[q] = (uint8_t)xv;
                    left[q + 1] = (uint8_t)(left[q] - xv);
                    // still equal to row n-1: its value on the orbit taken everywhere
                    const bool prev1 = (ones[q] >> (n - 1)) & 1u;
                    if (((tied >> q) & 1u) && xv == (prev1 ? len[q] : 0))
                        tied |= 1ull << (q + 1);
                    else
                        tied &= ~(1ull << (q + 1));
                    ca -= hi[q];
                    cn -= lo[q];
                    rc.sub(mq, hi[q]);
                    rn.sub(mq, lo[q]);
                    ++q;
                    state = ENTER;
                }
                continue;
            }
            state = BACK;
        }
        // no value left at orbit q: back up one orbit
        if (q == 0)
            break;
        --q;
        mq = spread16(ones[q]);
        ca += hi[q];
        cn += lo[q];
        rc.add(mq, hi[q]);
        rn.add(mq, lo[q]);
        lo64 = rn;
        lo64.sub(mq, lo[q]);
        lo64.w[0] += B64;
        lo64.w[1] += B64;
        up64 = rc;
        up64.sub(mq, hi[q]);
        up64.w[0] += B64;
        up64.w[1] += B64;
        state = TRY;
    }
    return count;
}

}  // namespace rows
}  // namespace canon
