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
