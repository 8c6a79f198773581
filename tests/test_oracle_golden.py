"""The CPU oracle against the reference's published known answers (no GPU)."""
import collections
import json
import os

import numpy as np
import pytest

import cases
import oracle

HIST = json.load(open(os.path.join(cases.GOLDEN, "bibd_histograms.json")))
FAST = ["7,7,3,3,1", "7,14,6,3,2", "9,12,4,3,1", "13,26,6,3,1", "8,14,7,4,3", "11,11,5,5,2",
        "10,15,6,4,2", "9,18,8,4,3"]


@pytest.mark.parametrize("key", FAST)
def test_bibd_enumeration_matches_reference_histogram(key):
    v, b, r, k, lam = map(int, key.split(","))
    found = cases.bibd_designs(v, b, r, k, lam)
    hist = collections.Counter(a for _, a in found)
    assert dict(hist) == {int(a): c for a, c in HIST[key].items()}


def test_sts15_fixture_is_canonical_with_reference_histogram():
    sts = cases.load_sts15()
    assert len(sts) == 80
    hist = collections.Counter()
    for M, aut in sts:
        res = oracle.bibd_test(M)
        assert res["canonical"] and res["aut"] == aut
        hist[aut] += 1
    assert dict(hist) == {int(a): c for a, c in HIST["15,35,7,3,1"].items()}
    assert len({M.tobytes() for M, _ in sts}) == 80


def test_k10_golden_matrices_are_canonical_with_reference_aut():
    k10 = cases.load_k10()
    assert len(k10) == 396
    for R, aut in k10[::9]:
        res = oracle.ksys_test(R)
        assert res["canonical"] and res["n_aut"] == aut


def test_k8_enumeration_counts():
    found, _ = oracle.ksys_enumerate(8)
    # six non-isomorphic 1-factorizations of K8
    assert len(found) == 6
    found6, _ = oracle.ksys_enumerate(6)
    assert len(found6) == 1 and found6[0][1] == 120


def test_aut_is_isomorphism_invariant_full_search():
    rng = np.random.default_rng(5)
    sts = cases.load_sts15()
    for M, aut in sts[::16]:
        P = cases.permute_normalize(M, rng)
        res = oracle.bibd_test(P, oracle.SAVE_ROW_PERM | oracle.FULL_AUT)
        assert res["aut"] == aut


def test_canonize_reaches_the_fixture_form():
    rng = np.random.default_rng(7)
    sts = cases.load_sts15()
    canon = {M.tobytes(): a for M, a in sts}
    for M, aut in sts[::20]:
        P = M[rng.permutation(15)][:, rng.permutation(35)]
        C, a, calls = oracle.bibd_canonize(P)
        assert C.tobytes() in canon and a == aut


def test_relabelled_k10_is_rejected_unless_equal():
    rng = np.random.default_rng(3)
    k10 = cases.load_k10()
    canon = {R.tobytes() for R, _ in k10}
    for R, aut in k10[:40]:
        X = cases.ksys_relabel_random(R, rng)
        res = oracle.ksys_test(X)
        assert res["canonical"] == (X.tobytes() in canon)


def test_kirkman_golden_matrices_are_canonical_with_reference_aut():
    """The oracle's cnvCheckNew() restatement with groups of 3 (the general path: relabel,
    sort inside the groups, groups by first player, rounds by second entry) on the 7
    Kirkman triple systems of k-Factorization/Results/Complete_graphs/15/15x7x3: each is
    canonical with the reference's |Aut(M)|, after trying all 5! x 3!^5 x 7 - 1
    relabelings; relabelled copies are rejected."""
    import concurrent.futures as cf
    kts = cases.load_kts15()
    assert sorted(a for _, a in kts) == [12, 12, 21, 24, 24, 168, 168]
    with cf.ThreadPoolExecutor(max(1, min(7, os.cpu_count() or 1))) as ex:
        outs = list(ex.map(lambda R: oracle.ksys_test(R, g=3), [R for R, _ in kts]))
    for (R, aut), o in zip(kts, outs):
        assert o["canonical"] and o["n_aut"] == aut
        assert o["candidates"] == 120 * 6 ** 5 * 7 - 1
    rng = np.random.default_rng(15)
    rejected = 0
    for R, _ in kts:
        X = cases.ksys_relabel_random(R, rng, g=3)
        if not np.array_equal(X, R):
            rejected += not oracle.ksys_test(X, g=3)["canonical"]
    assert rejected >= 5
