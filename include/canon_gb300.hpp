// canon_gb300.hpp -- header-only C++ adapter over the C ABI (canon_gb300.h).
//
// Mirrors the checker surface the reference's enumerators call, so that a
// maintainer can swap the check of Source/Enumerator.cpp:364 / :446-447 and of
// k-Factorization/TripleSys/Source/checkCurrentResult.cpp:91 for the GPU one:
//
//   GpuCanonicityChecker::TestCanonicity(nRowMax, rows, outInfo)
//       ~ CCanonicityChecker<uchar,uchar>::TestCanonicity(nRowMax, pCanonParam, outInfo)
//         Source/CanonicityChecker.h:58,255-586; permRow() :61, groupOrder()
//         GroupOrder.h:54, permStorage() :63-64, rowToChange() CanonicityChecker.cpp:320-330
//   GpuCanonicityChecker::CanonizeMatrix(rows)
//       ~ CMatrixCanonChecker::CanonizeMatrix(0), Source/MatrixCanonChecker.cpp:420-564
//   GpuKSysChecker::cnvCheckNew(nrows, result)
//       ~ alldata::cnvCheckNew(0, nrows), k-Factorization/TripleSys/Source/cnv.cpp:211;
//         m_playerIndex and orderOfGroup() (Include/groupInfo.h:121-125)
//
// The batch methods (queue + sync) are the intended way to use the GPU: the
// enumerator collects every partial matrix of a level, checks them in one
// canon_sync() and then continues on the canonical ones.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "canon_gb300.h"

namespace canon_gb300 {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string &msg) : std::runtime_error(msg), code(code) {}
    int code;
};

// t_canonOutInfo, Source/CanonicityChecker.h:27-32
enum OutInfo : unsigned { t_saveNothing = 0, t_saveRowPermutations = 1, t_saveRowToChange = 4 };

class Context {
public:
    explicit Context(int device = 0, uint32_t max_items = 1u << 16, uint32_t aut_cap = 64) {
        canon_cfg cfg{};
        cfg.device = device;
        cfg.max_items = max_items;
        cfg.aut_cap = aut_cap;
        ctx_ = canon_create(&cfg);
        if (!ctx_)
            throw Error(CANON_ENODEV, "canon_create failed");
    }
    ~Context() { canon_destroy(ctx_); }
    Context(const Context &) = delete;
    Context &operator=(const Context &) = delete;
    canon_ctx *get() const { return ctx_; }
    void check(int rc) const {
        if (rc != CANON_OK)
            throw Error(rc, canon_last_error(ctx_));
    }
    // queue incidence matrices (rows: n*v words, bit c = column c)
    void submitBIBD(const uint64_t *rows, uint32_t n, uint32_t v, uint32_t b, uint32_t flags,
                    const uint8_t *nrows = nullptr) {
        canon_bibd_batch bt{n, v, b, flags, rows, nrows};
        check(canon_submit_bibd(ctx_, &bt));
    }
    // queue k-system matrices (rounds of pairs in the reference's result() form)
    void submitKSys(const uint8_t *data, uint32_t n, uint32_t np, uint32_t rounds, uint32_t flags,
                    const uint8_t *nrows = nullptr, uint32_t groupSize = 2) {
        canon_ksys_batch bt{n, np, rounds, flags, data, nrows};
        check(groupSize == 2 ? canon_submit_ksys(ctx_, &bt) : canon_submit_ksys_groups(ctx_, &bt, groupSize));
    }
    const canon_results &sync() {
        check(canon_sync(ctx_, &res_));
        return res_;
    }
    const canon_results &results() const { return res_; }

private:
    canon_ctx *ctx_ = nullptr;
    canon_results res_{};
};

// pack a row-major 0/1 byte matrix (the reference's CMatrixData rows) into words
inline std::vector<uint64_t> packRows(const uint8_t *matrix, uint32_t nrows, uint32_t ncols) {
    std::vector<uint64_t> w(nrows, 0);
    for (uint32_t r = 0; r < nrows; ++r)
        for (uint32_t c = 0; c < ncols; ++c)
            if (matrix[r * ncols + c])
                w[r] |= 1ull << c;
    return w;
}

class GpuCanonicityChecker {
public:
    GpuCanonicityChecker(Context &ctx, uint32_t nRow, uint32_t nCol) : ctx_(ctx), nRow_(nRow), nCol_(nCol) {}

    // One TestCanonicity() call; `matrix` is the row-major byte matrix of the
    // enumerator (columns in orbit normal form, as MakeRow() builds them).
    bool TestCanonicity(uint32_t nRowMax, const uint8_t *matrix, unsigned outInfo = t_saveNothing) {
        auto rows = packRows(matrix, nRowMax, nCol_);
        const uint32_t flags = (outInfo & t_saveRowPermutations) ? CANON_COMPLETE : 0u;
        ctx_.submitBIBD(rows.data(), 1, nRowMax, nCol_, flags | CANON_SAVE_AUTS);
        const canon_results &r = ctx_.sync();
        if (r.status[0] & CANON_ST_BADINPUT)
            throw Error(CANON_EINVAL, "matrix is not in column-orbit normal form");
        nRowMax_ = nRowMax;
        return r.canonical[0] != 0;
    }
    const uint8_t *permRow() const { return ctx_.results().witness; }
    uint8_t rowToChange() const { return ctx_.results().row_to_change[0]; }
    uint64_t groupOrder() const { return ctx_.results().aut[0]; }
    // PermutStorage layout: numPerm x lenPerm bytes, slot 0 the identity
    uint32_t numPerm() const { return ctx_.results().n_auts[0]; }
    uint32_t lenPerm() const { return ctx_.results().len_aut[0]; }
    const uint8_t *getPermutByIndex(uint32_t i) const { return ctx_.results().auts + i * 64u; }

    // CanonizeMatrix(0) in place on packed rows (all nRow rows filled)
    uint64_t CanonizeMatrix(uint64_t *rows) {
        uint64_t aut[2] = {0, 0};
        ctx_.check(canon_canonize_bibd(ctx_.get(), 1, nRow_, nCol_, rows, aut));
        return aut[0];
    }

private:
    Context &ctx_;
    uint32_t nRow_, nCol_, nRowMax_ = 0;
};

class GpuKSysChecker {
public:
    // groupSize: m_groupSize of the alldata object (2, 3 or 4)
    GpuKSysChecker(Context &ctx, uint32_t numPlayers, uint32_t groupSize = 2)
        : ctx_(ctx), np_(numPlayers), g_(groupSize) {}
    bool cnvCheckNew(uint32_t nrows, const uint8_t *result) {
        ctx_.submitKSys(result, 1, np_, nrows, CANON_SAVE_AUTS, nullptr, g_);
        const canon_results &r = ctx_.sync();
        if (r.status[0] & CANON_ST_BADINPUT)
            throw Error(CANON_EINVAL, "rounds are not in the result() form");
        return r.canonical[0] != 0;
    }
    int32_t playerIndex() const { return ctx_.results().player_index[0]; }
    uint64_t orderOfGroup() const { return ctx_.results().aut[0]; }
    const uint8_t *groupObject(uint32_t i) const { return ctx_.results().auts + i * 64u; }

private:
    Context &ctx_;
    uint32_t np_, g_;
};

// RAII owner of the reference's plugin handle (createCanonizer / runCanonizer /
// releaseCanonizer, k-Factorization/Utils/Include/CDTools.h:9-11).
class Canonizer {
public:
    Canonizer(int v, int k) : h_(createCanonizer(v, k)) {
        if (!h_)
            throw Error(CANON_EINVAL, "createCanonizer failed (k = 2 with even v in 6..16, k = 3 with v = 9 or 15, "
                                      "k = 4 with v = 16; a GPU)");
    }
    ~Canonizer() { releaseCanonizer(h_); }
    Canonizer(const Canonizer &) = delete;
    Canonizer &operator=(const Canonizer &) = delete;
    // the canonical binary matrix of the first iDay rounds (all when iDay <= 0), owned here
    const unsigned char *run(const unsigned char *pMatrix, int k, int iDay = 0) {
        return runCanonizer(h_, pMatrix, k, iDay);
    }

private:
    void *h_;
};

}  // namespace canon_gb300
