// canon_report.cpp -- the reference's result tables, written from enumeration results.
//
// BIBD runs end with the |Aut(D)| table that CGroupsInfo::printGroupInfo()
// writes (Source/GroupsInfo.cpp:72-150, counters of Source/GroupsInfo.h:4-11),
// in the layout of the committed result files Results/BIBDs/V = v/<v>_<k>_<l>.txt.
// k-system runs end with the |Aut(M)| x cycle-type table of MatrixDB
// (k-Factorization/TripleSys/Include/MatrixDB.h, DescrStorage::reportResult and
// MatrixDB::printRecord), whose cycle descriptors are those of
// alldata::matrixStatOutput() (Source/p1fCheck.cpp:499-515) over the cycle sets
// that collectCyclesAndPath() keeps sorted (Source/p1fCheck.cpp:77-117), in the
// layout of k-Factorization/Results/Complete_graphs/<n>/.../K_Results.txt.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/canon_gb300.h"

namespace {

void add(std::string &s, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    s += buf;
}

size_t emit(const std::string &s, char *buf, size_t cap) {
    if (buf && cap) {
        const size_t n = std::min(cap - 1, s.size());
        std::memcpy(buf, s.data(), n);
        buf[n] = '\0';
    }
    return s.size();
}

// counters of one group order: designs, simple, transitive, simple and transitive
struct Counts {
    unsigned long long nd = 0, ns = 0, ndt = 0, nst = 0;
};

// cycle lengths (ascending) of the union of two perfect matchings given as rounds
// in result() form (pairs of players)
std::vector<uint8_t> cycle_type(const uint8_t *a, const uint8_t *b, unsigned np) {
    uint8_t pa[16], pb[16];
    for (unsigned i = 0; i < np; i += 2) {
        pa[a[i]] = a[i + 1];
        pa[a[i + 1]] = a[i];
        pb[b[i]] = b[i + 1];
        pb[b[i + 1]] = b[i];
    }
    std::vector<uint8_t> lens;
    unsigned seen = 0;
    for (unsigned s = 0; s < np; ++s) {
        if (seen & (1u << s))
            continue;
        unsigned x = s, len = 0;
        bool first = true;
        do {
            seen |= 1u << x;
            ++len;
            x = first ? pa[x] : pb[x];
            first = !first;
        } while (x != s || !first);
        lens.push_back((uint8_t)len);
    }
    std::sort(lens.begin(), lens.end());
    return lens;
}

}  // namespace

extern "C" {

size_t canon_report_bibd(uint32_t v, uint32_t b, uint32_t r, uint32_t k, uint32_t lambda, uint32_t n,
                         const uint64_t *aut, const uint8_t *simple, const uint8_t *transitive,
                         uint64_t fully_constructed, double seconds, char *buf, size_t cap) {
    std::map<uint64_t, Counts> by_order;
    Counts total;
    for (uint32_t i = 0; i < n; ++i) {
        Counts &c = by_order[aut[i]];
        const bool s = simple && simple[i], t = transitive && transitive[i];
        ++c.nd;
        c.ns += s;
        c.ndt += t;
        c.nst += s && t;
        ++total.nd;
        total.ns += s;
        total.ndt += t;
        total.nst += s && t;
    }
    std::string out;
    add(out, "BIBD(%3u, %3u, %2u, %2u, %2u)\n\n", v, b, r, k, lambda);
    const std::string rule = "    " + std::string(79, '_') + "\n";
    out += "        |Aut(D)|          Nd:             Ns:            Ndt:            Nst:\n";
    out += rule;
    for (const auto &e : by_order)
        add(out, "    %10llu%16llu%16llu%16llu%16llu\n", (unsigned long long)e.first, e.second.nd, e.second.ns,
            e.second.ndt, e.second.nst);
    out += rule;
    add(out, "        Total:%16llu%16llu%16llu%16llu\n\n", total.nd, total.ns, total.ndt, total.nst);
    const unsigned long long fc = (unsigned long long)fully_constructed;
    add(out, "%10llu matri%s constructed in %5.2f\n", total.nd, total.nd == 1 ? "x" : "ces", seconds);
    add(out, "%10llu matri%s no replicated blocks\n", total.ns, total.ns == 1 ? "x has" : "ces have");
    add(out, "%10llu matri%s fully constructed\n", fc, fc == 1 ? "x was" : "ces were");
    return emit(out, buf, cap);
}

size_t canon_ksys_cycles(uint32_t np, uint32_t rounds, const uint8_t *matrix, char *buf, size_t cap) {
    // cycle sets in increasing order of their length lists, each with the number
    // of round pairs that give it
    std::map<std::vector<uint8_t>, unsigned> sets;
    if (np >= 4 && np <= 16 && !(np & 1u))
        for (uint32_t d2 = 1; d2 < rounds; ++d2)
            for (uint32_t d1 = 0; d1 < d2; ++d1)
                ++sets[cycle_type(matrix + d1 * np, matrix + d2 * np, np)];
    std::string out;
    for (const auto &e : sets) {
        add(out, "%u(", e.second);
        for (size_t j = 0; j < e.first.size(); ++j)
            add(out, j ? ":%u" : "%u", (unsigned)e.first[j]);
        out += ") ";
    }
    return emit(out, buf, cap);
}

size_t canon_report_ksys(uint32_t np, uint32_t rounds, uint32_t n, const uint8_t *matrices, const uint64_t *aut,
                         char *buf, size_t cap) {
    // records ordered by |Aut(M)|, then by descriptor (strcmp), as
    // DescrStorage::addObjDescriptor() inserts them
    std::map<std::pair<uint64_t, std::string>, unsigned long long> rec;
    for (uint32_t i = 0; i < n; ++i) {
        char d[512];
        canon_ksys_cycles(np, rounds, matrices + (size_t)i * rounds * np, d, sizeof(d));
        ++rec[{aut[i], std::string(d)}];
    }
    std::string out;
    const std::string rule = "     " + std::string(60, '-') + "\n";
    add(out, "     Factorization of K(%u)\n", np);
    out += rule;
    out += "       |Aut(M)|:  # of matrices:          Cycles:\n";
    out += rule;
    unsigned long long total = 0;
    for (const auto &e : rec) {
        add(out, "     %8llu      %8llu        %-34s\n", (unsigned long long)e.first.first, e.second,
            e.first.second.c_str());
        total += e.second;
    }
    out += rule;
    add(out, "     %11s%11llu\n", "Total:", total);
    out += rule;
    out += "\n\n";
    return emit(out, buf, cap);
}

}  // extern "C"
