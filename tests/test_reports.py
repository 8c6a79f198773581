"""The result-table writers (canon_report.cpp) against the reference's committed
result files, on designs from the oracle (host only, no GPU)."""
import re

import numpy as np
import pytest

import cases
import oracle

# BIBD parameter sets whose oracle enumeration takes well under a second
SMALL = ["6,10,5,3,2", "6,20,10,3,4", "6,30,15,3,6", "7,7,3,3,1", "7,14,6,3,2", "7,21,9,3,3",
         "7,28,12,3,4", "8,14,7,4,3", "9,12,4,3,1", "9,18,8,4,3", "9,24,8,3,2", "10,15,6,4,2",
         "11,11,5,5,2", "13,13,4,4,1", "13,26,6,3,1", "15,15,7,7,3", "16,16,6,6,2", "16,20,5,4,1"]


@pytest.fixture(scope="module")
def G():
    import conftest
    conftest.build_native()
    import ise_gb300
    return ise_gb300


def test_k10_table_is_the_reference_table(G):
    """The 396 canonical 1-factorizations of K10 with their |Aut(M)| give K_Results.txt's
    table line for line: group orders, counts and cycle descriptors."""
    k10 = cases.load_k10()
    text = G.report_ksys([M for M, _ in k10], [a for _, a in k10])
    with open(cases.os.path.join(cases.GOLDEN, "k10_results_table.txt")) as f:
        assert text == f.read()


def test_ksys_cycle_descriptor(G):
    # K4: the three rounds pairwise form one 4-cycle
    M = np.array([[0, 1, 2, 3], [0, 2, 1, 3], [0, 3, 1, 2]], np.uint8)
    assert G.ksys_cycles(M) == "3(4) "
    # K6 with two rounds only: one pair of rounds
    M = np.array([[0, 1, 2, 3, 4, 5], [0, 2, 1, 3, 4, 5]], np.uint8)
    assert G.ksys_cycles(M) == "1(2:4) "


@pytest.mark.parametrize("key", SMALL)
def test_bibd_table_counts(G, key):
    """Nd / Ns / Ndt / Nst per group order of the oracle's enumeration equal the
    reference's result file; in the current layout the whole text block does."""
    ref = cases.load_result_tables()[key]
    params = tuple(map(int, key.split(",")))
    designs, _ = oracle.bibd_enumerate(*params)
    simple = [cases.simple_design(M) for M, _ in designs]
    trans = [cases.oracle_transitive(M) for M, _ in designs]
    assert cases.table_rows(designs, simple, trans) == ref["rows"]
    text = G.report_bibd(params, [a for _, a in designs], simple, trans,
                         fully_constructed=ref.get("fully_constructed", 0), seconds=ref.get("seconds", 0.0))
    if ref["wide"]:
        # one older file prints the run time without its field width
        norm = lambda t: re.sub(r"constructed in +", "constructed in ", t)
        assert norm(text) == norm(ref["text"])
    total = next(l for l in text.splitlines() if l.strip().startswith("Total:"))
    assert [int(x) for x in total.split()[1:]] == ref["total"]


def test_report_buffer_truncates_like_snprintf(G):
    import ctypes
    L = G.load_library()
    aut = np.array([1, 1, 6], np.uint64)
    full = L.canon_report_bibd(7, 7, 3, 3, 1, 3, aut.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                               None, None, 0, 0.0, None, 0)
    buf = ctypes.create_string_buffer(16)
    n = L.canon_report_bibd(7, 7, 3, 3, 1, 3, aut.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)),
                            None, None, 0, 0.0, buf, 16)
    assert n == full and len(buf.value) == 15 and buf.value.startswith(b"BIBD(")
