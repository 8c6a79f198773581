"""The reference's plugin (createCanonizer / runCanonizer / releaseCanonizer,
k-Factorization/Utils/Include/CDTools.h:9-11) and the batched canonical binary matrix
of k-systems on the GPU, against the oracle's restatement of the reference path
(convertToBinaryMatrix + CanonizeMatrix with the day classes): every 1-factorization
of K6 and K8 with all days (the days may be permuted), K10 prefixes of 2..8 days (the
day order is fixed by the colours), random relabelings of each, and the complete K10
factorizations through invariance under relabelings of players, days and pairs."""
import numpy as np
import pytest

import cases
import ise_gb300 as G
import oracle

pytestmark = pytest.mark.gpu


def relabel(R, rng, np_, shuffle_days):
    p = rng.permutation(np_)
    rounds = []
    for row in R:
        pairs = sorted(tuple(sorted((int(p[row[i]]), int(p[row[i + 1]])))) for i in range(0, np_, 2))
        rounds.append([x for pr in pairs for x in pr])
    order = rng.permutation(len(rounds)) if shuffle_days else np.arange(len(rounds))
    return np.array([rounds[i] for i in order], np.uint8)


@pytest.mark.parametrize("np_", [6, 8])
def test_batched_all_days_match_the_oracle(ctx, np_):
    rng = np.random.default_rng(np_)
    found, _ = oracle.ksys_enumerate(np_)
    mats = [R for R, _ in found] + [relabel(R, rng, np_, True) for R, _ in found]
    out, aut = ctx.canonize_ksys_binary(np.stack(mats), np_, np_ - 1)
    for i, (R, a) in enumerate(found):
        ref, _ = oracle.ksys_binary_canonize(R, np_)
        assert np.array_equal(out[i], ref) and np.array_equal(out[len(found) + i], ref)
        assert aut[i] == a and aut[len(found) + i] == a      # |Aut| of the factorization


def test_plugin_on_k10_prefixes_matches_the_oracle():
    rng = np.random.default_rng(10)
    k10 = cases.load_k10()
    can = G.Canonizer(10, 2)
    try:
        for R, _ in k10[::11]:
            for d in (2, 3, 5, 8):
                ref, _ = oracle.ksys_binary_canonize(R[:d], 10, 2, d)
                got = can.run(R, d)          # the first d rounds, as runCanonizer(h, result(0), k, iDay)
                assert got is not None and np.array_equal(got, ref), d
                X = relabel(R[:d], rng, 10, False)
                assert np.array_equal(can.run(X, d), ref)
        # invalid day counts are refused with NULL, as the reference returns nothing useful
        assert can.run(k10[0][0], 1) is None and can.run(k10[0][0], 10) is None
    finally:
        can.close()


def test_complete_k10_is_invariant_and_separates_the_396(ctx):
    """All 396 complete 1-factorizations of K10 (all 9 days): relabelled copies give the
    same canonical binary matrix, different factorizations give different ones, and
    the labelings reaching the form number |Aut| of the factorization."""
    rng = np.random.default_rng(396)
    k10 = cases.load_k10()
    mats = np.stack([R for R, _ in k10] + [relabel(R, rng, 10, True) for R, _ in k10])
    out, aut = ctx.canonize_ksys_binary(mats, 10, 9)
    n = len(k10)
    assert np.array_equal(out[:n], out[n:])
    assert len({o.tobytes() for o in out[:n]}) == n
    assert [int(a) for a in aut[:n]] == [a for _, a in k10]
    # the plugin's full-day call gives the batched result
    can = G.Canonizer(10, 2)
    try:
        for i in range(0, n, 99):
            assert np.array_equal(can.run(k10[i][0]), out[i])
    finally:
        can.close()


def test_groups_of_3_and_4_match_the_oracle(ctx):
    """Groups of 3 and 4 (canon_canonize_ksys_binary_groups and the plugin with k = 3, 4):
    the 7 Kirkman triple systems of 15 players and relabelled copies, all days (|Aut(M)|
    as the labelings reaching the form) and prefixes through runCanonizer; the resolution
    of AG(2,4) (groups of 4) from the enumeration."""
    rng = np.random.default_rng(15)
    kts = cases.load_kts15()
    mats = [R for R, _ in kts] + [cases.ksys_relabel_random(R, rng, g=3) for R, _ in kts]
    out, aut = ctx.canonize_ksys_binary(np.stack(mats), 15, 7, k=3)
    for i, (R, a) in enumerate(kts):
        ref, _ = oracle.ksys_binary_canonize(R, 15, 3)
        assert np.array_equal(out[i], ref) and np.array_equal(out[len(kts) + i], ref)
        assert aut[i] == a and aut[len(kts) + i] == a
    can = G.Canonizer(15, 3)
    try:
        for R, _ in kts[::3]:
            for d in (2, 3, 5, 6):
                ref, _ = oracle.ksys_binary_canonize(R[:d], 15, 3, d)
                assert np.array_equal(can.run(R, d), ref), d
            assert np.array_equal(can.run(R), oracle.ksys_binary_canonize(R, 15, 3)[0])
        assert can.run(kts[0][0], 1) is None and can.run(kts[0][0], 8) is None
    finally:
        can.close()
    found, _ = ctx.enumerate_ksys_groups(16, 4)
    R = found[0][0]
    out, aut = ctx.canonize_ksys_binary(R[None], 16, 5, k=4)
    assert np.array_equal(out[0], oracle.ksys_binary_canonize(R, 16, 4)[0]) and aut[0] == 5760
    can = G.Canonizer(16, 4)
    try:
        assert np.array_equal(can.run(R, 3), oracle.ksys_binary_canonize(R[:3], 16, 4, 3)[0])
    finally:
        can.close()
    for v, k in [(12, 3), (12, 4), (15, 5)]:
        with pytest.raises(G.CanonError):
            G.Canonizer(v, k)
