"""The oracle's restatement of GroupOrder.h against the reference's own
CGroupOrder<T>, compiled in place from the reference tree (this container only)."""
import os
import subprocess

import numpy as np
import pytest

import cases
import oracle

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(REPO, "oracle", "_ref", "libref_grouporder.so")


@pytest.fixture(scope="module")
def ref():
    # the recipe finds the reference tree (ISE_REFERENCE_ROOT or its default) and
    # builds nothing where it is absent, e.g. on a machine without the reference
    root = os.environ.get("ISE_REFERENCE_ROOT")
    subprocess.run(["sh", os.path.join(REPO, "oracle", "build_ref.sh")] + ([root] if root else []), check=True,
                   capture_output=True)
    if not os.path.exists(REF_LIB):
        pytest.skip("reference tree not present")
    yield REF_LIB
    oracle.use_reference_group_order(None)


def _run(M, flags, ref_path):
    oracle.use_reference_group_order(None)
    a = oracle.bibd_test(M, flags, perm_cap=256)
    oracle.use_reference_group_order(ref_path)
    b = oracle.bibd_test(M, flags, perm_cap=256)
    oracle.use_reference_group_order(None)
    return a, b


def _same(a, b):
    assert a.keys() == b.keys()
    for k in a:
        if isinstance(a[k], np.ndarray):
            assert np.array_equal(a[k], b[k]), k
        else:
            assert a[k] == b[k], k


def test_sts15_complete_partial_full(ref):
    rng = np.random.default_rng(11)
    sts = cases.load_sts15()
    for i in range(40):
        M = oracle.rows_to_matrix(oracle.sts_random_rows(15, 99, i), 35)
        if i % 2:
            M = sts[i % 80][0][rng.permutation(15)]
        for nr in (15, 5, 8, 11):
            X = oracle.bibd_normalize(M[:nr])
            base = (oracle.SAVE_ROW_PERM | oracle.SAVE_ROW_TO_CHANGE) if nr == 15 else 0
            for extra in (0, oracle.FULL_AUT):
                _same(*_run(X, base | extra, ref))


def test_small_designs_all_prefixes(ref):
    rng = np.random.default_rng(12)
    for params in [(8, 14, 7, 4, 3), (11, 11, 5, 5, 2), (7, 14, 6, 3, 2), (13, 26, 6, 3, 1)]:
        for M, _ in cases.bibd_designs(*params):
            for _ in range(3):
                P = cases.permute_normalize(M, rng)
                for nr in range(2, P.shape[0] + 1):
                    X = oracle.bibd_normalize(P[:nr])
                    flags = (oracle.SAVE_ROW_PERM | oracle.SAVE_ROW_TO_CHANGE |
                             oracle.SAVE_AUT_ROWS) if nr == P.shape[0] else 0
                    _same(*_run(X, flags | oracle.FULL_AUT, ref))
