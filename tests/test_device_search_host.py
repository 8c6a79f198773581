"""The BIBD kernel's search (canon_bibd_core.cuh) compiled for the host and checked
against the oracle: catches logic errors of the device code on the CPU."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import cases
import conftest
import oracle

import ise_gb300 as G

SRC = os.path.join(conftest.REPO, "tests", "host_build", "canon_bibd_host.cpp")
OUT = os.path.join(conftest.REPO, "tests", "host_build", "_build", "libcanon_bibd_host.so")
CUDA_INC = "/usr/local/cuda/include"

COMPLETE, RAW, FULL_AUT, AUT_CANON, REFERENCE_ORDER = 0x1, 0x2, 0x4, 0x10, 0x20


@pytest.fixture(scope="module")
def host():
    if not os.path.isdir(CUDA_INC):
        pytest.skip("CUDA headers not found")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", CUDA_INC, SRC, "-o", OUT],
                   check=True)
    return ctypes.CDLL(OUT)


def run(L, rows, n, b, flags):
    rows = np.ascontiguousarray(rows, np.uint64)
    u8, u64 = ctypes.c_uint8, ctypes.c_uint64
    can, st, rr, w, tr = u8(), u8(), u8(), u64(), u64()
    aut = (u64 * 2)()
    L.emu_check(rows.ctypes.data_as(ctypes.POINTER(u64)), n, b, flags, u64(1 << 24), ctypes.byref(can),
                ctypes.byref(st), ctypes.byref(rr), ctypes.byref(w), aut, ctypes.byref(tr))
    return dict(canonical=bool(can.value), status=st.value, reject_row=rr.value,
                witness=bytes((w.value >> (4 * i)) & 15 for i in range(n)),
                aut=aut[0] | (aut[1] << 64), trials=tr.value)


def expected(M, flags):
    X = oracle.bibd_normalize(M) if flags & RAW else M
    f = (oracle.SAVE_ROW_PERM | oracle.SAVE_ROW_TO_CHANGE) if flags & COMPLETE else 0
    o = oracle.bibd_test(X, f | (oracle.FULL_AUT if flags & FULL_AUT else 0))
    if flags & AUT_CANON and not o["canonical"]:
        _, o["aut"], _ = oracle.bibd_canonize(X)
    return o


def compare(L, M, flags):
    n, b = M.shape
    import ise_gb300 as G
    e = run(L, G.pack_rows(M), n, b, flags)
    o = expected(M, flags)
    assert e["status"] == 0
    assert e["canonical"] == o["canonical"]
    if flags & REFERENCE_ORDER:
        assert e["trials"] == o["trials"]
    if not o["canonical"]:
        assert e["witness"] == o["witness"] and e["reject_row"] == o["reject_row"]
    if o["canonical"] or flags & (FULL_AUT | AUT_CANON):
        assert e["aut"] == o["aut"]


FLAGS = [COMPLETE | RAW, COMPLETE | RAW | FULL_AUT, COMPLETE | RAW | AUT_CANON]


@pytest.mark.parametrize("flags", FLAGS + [f | REFERENCE_ORDER for f in FLAGS])
def test_sts15_random(host, flags):
    for i in range(8 if flags & FULL_AUT and flags & REFERENCE_ORDER else 30):
        compare(host, oracle.rows_to_matrix(oracle.sts_random_rows(15, 808, i), 35), flags)


def test_sts15_canonical_fixture_aut(host):
    for M, aut in cases.load_sts15():
        import ise_gb300 as G
        e = run(host, G.pack_rows(M), 15, 35, COMPLETE)
        assert e["canonical"] and e["aut"] == aut


def maxsearch(L, rows, n, b, prune):
    u64 = ctypes.c_uint64
    rows = np.ascontiguousarray(rows, np.uint64)
    out = np.zeros(n, np.uint64)
    leaves, nodes, imp, fr = u64(), u64(), ctypes.c_uint8(), ctypes.c_uint()
    rc = L.emu_maxsearch(rows.ctypes.data_as(ctypes.POINTER(u64)), n, b, out.ctypes.data_as(ctypes.POINTER(u64)),
                         ctypes.byref(leaves), ctypes.byref(nodes), ctypes.byref(imp), int(prune), ctypes.byref(fr))
    assert rc == 0
    return dict(rows=out, aut=leaves.value, nodes=nodes.value, improved=bool(imp.value), first_rows=fr.value)


def test_lex_max_search_gives_canonical_form(host):
    import ise_gb300 as G
    canon = {M.tobytes(): a for M, a in cases.load_sts15()}
    for i in range(25):
        rows = oracle.sts_random_rows(15, 4242, i)
        for prune in (False, True):
            r = maxsearch(host, rows, 15, 35, prune)
            C = G.unpack_rows(r["rows"], 35)
            Co, ao, _ = oracle.bibd_canonize(oracle.rows_to_matrix(rows, 35))
            assert np.array_equal(C, Co) and r["aut"] == ao == canon[C.tobytes()]


def _same_search_results(L, rows, n, b):
    full = maxsearch(L, rows, n, b, False)
    pruned = maxsearch(L, rows, n, b, True)
    for k in ("aut", "improved", "first_rows"):
        assert pruned[k] == full[k], (k, pruned[k], full[k])
    assert np.array_equal(pruned["rows"], full["rows"])
    assert pruned["nodes"] <= full["nodes"]
    return full, pruned


def test_automorphism_pruning_keeps_every_output(host):
    """The pruned lex-max search gives the canonical form, |Aut|, the verdict and the
    first-row orbit of the unpruned one, on canonical designs (large groups: up to
    20160), their row/column-permuted copies and partial matrices of both."""
    import ise_gb300 as G
    rng = np.random.default_rng(5)
    sts = cases.load_sts15()
    ratio = {}
    for M, aut in sts:
        full, pruned = _same_search_results(host, G.pack_rows(M), 15, 35)
        assert full["aut"] == aut and not full["improved"]
        ratio[aut] = full["nodes"] / pruned["nodes"]
        P = cases.permute_normalize(M, rng)
        _same_search_results(host, G.pack_rows(P), 15, 35)
        for k in (4, 7, 10, 13):
            _same_search_results(host, G.pack_rows(oracle.bibd_normalize(P[:k])), k, 35)
    assert ratio[20160] > 20          # PG(3,2): the pruned search visits far fewer nodes
    for params in [(8, 14, 7, 4, 3), (11, 11, 5, 5, 2), (13, 26, 6, 3, 1), (9, 12, 4, 3, 1)]:
        v, b = params[0], params[1]
        for M, _ in cases.bibd_designs(*params):
            _same_search_results(host, G.pack_rows(M), v, b)
            for _ in range(3):
                P = cases.permute_normalize(M, rng)
                for k in range(2, v + 1):
                    _same_search_results(host, G.pack_rows(oracle.bibd_normalize(P[:k])), k, b)


def test_partial_prefixes(host):
    rng = np.random.default_rng(21)
    sts = cases.load_sts15()
    for M, _ in sts[::7]:
        P = cases.permute_normalize(M, rng)
        for k in (3, 6, 9, 12):
            compare(host, oracle.bibd_normalize(P[:k]), 0)
            compare(host, oracle.bibd_normalize(P[:k]), FULL_AUT)
            compare(host, oracle.bibd_normalize(P[:k]), REFERENCE_ORDER)
    for params in [(8, 14, 7, 4, 3), (11, 11, 5, 5, 2), (7, 14, 6, 3, 2)]:
        for M, _ in cases.bibd_designs(*params):
            for _ in range(3):
                P = cases.permute_normalize(M, rng)
                for k in range(2, P.shape[0] + 1):
                    f = COMPLETE if k == P.shape[0] else 0
                    compare(host, oracle.bibd_normalize(P[:k]), f)
                    compare(host, oracle.bibd_normalize(P[:k]), f | FULL_AUT)


def test_trial_budget_ends_the_search_with_a_timeout_status(host):
    import ise_gb300 as G
    M = cases.load_sts15()[0][0]
    rows = np.ascontiguousarray(G.pack_rows(M), np.uint64)
    u8, u64 = ctypes.c_uint8, ctypes.c_uint64
    for flags in (COMPLETE, COMPLETE | REFERENCE_ORDER):
        can, st, rr, w, tr = u8(), u8(), u8(), u64(), u64()
        aut = (u64 * 2)()
        host.emu_check(rows.ctypes.data_as(ctypes.POINTER(u64)), 15, 35, flags, u64(4), ctypes.byref(can),
                       ctypes.byref(st), ctypes.byref(rr), ctypes.byref(w), aut, ctypes.byref(tr))
        assert st.value & 2 and not can.value


def _split_result(L, rows, n, b):
    """The search split into one thread per first row, combined as the split kernel does."""
    u64 = ctypes.c_uint64
    rows = np.ascontiguousarray(rows, np.uint64)
    improved, total0, deep = False, 0, None
    for j in range(n):
        leaves, orb0, imp = u64(), ctypes.c_uint(), ctypes.c_uint8()
        assert L.emu_maxsearch_root(rows.ctypes.data_as(ctypes.POINTER(u64)), n, b, 1 << j, ctypes.byref(leaves),
                                    ctypes.byref(orb0), ctypes.byref(imp)) == 0
        improved |= bool(imp.value)
        total0 += orb0.value
        if j == 0:
            deep = leaves.value // max(orb0.value, 1)
    return improved, (0 if improved else total0 * deep)


def _split2_result(L, rows, n, b):
    """The search split into one thread per (first row, second row), combined as
    the two-level split kernel does."""
    u64 = ctypes.c_uint64
    rows = np.ascontiguousarray(rows, np.uint64)
    improved, in_orbit0, in_orbit1, deep = False, set(), 0, None
    for j in range(n):
        for k in range(n):
            leaves, o0, o1, imp = u64(), ctypes.c_uint(), ctypes.c_uint(), ctypes.c_uint8()
            assert L.emu_maxsearch_root2(rows.ctypes.data_as(ctypes.POINTER(u64)), n, b, 1 << j, 1 << k,
                                         ctypes.byref(leaves), ctypes.byref(o0), ctypes.byref(o1),
                                         ctypes.byref(imp)) == 0
            improved |= bool(imp.value)
            if j != 0 and o0.value:
                in_orbit0.add(j)
            if j == 0 and k >= 2:
                in_orbit1 += o1.value
            if (j, k) == (0, 1):
                deep = leaves.value
    return improved, (0 if improved else (1 + len(in_orbit0)) * (1 + in_orbit1) * deep)


def test_search_split_by_first_two_rows_combines_to_the_whole(host):
    """One thread per (first row, second row): |Aut| = |orbit of row 0| x |orbit of
    row 1 under the stabilizer of row 0| x the identity thread's product below."""
    import ise_gb300 as G
    rng = np.random.default_rng(12)
    todo = []
    for M, _ in cases.load_sts15()[::7]:
        todo.append((G.pack_rows(M), 35))
        P = cases.permute_normalize(M, rng)
        for k in (4, 8, 12):
            todo.append((G.pack_rows(oracle.bibd_normalize(P[:k])), 35))
    for params in [(8, 14, 7, 4, 3), (13, 26, 6, 3, 1), (9, 12, 4, 3, 1)]:
        for M, _ in cases.bibd_designs(*params):
            todo.append((G.pack_rows(M), params[1]))
            P = cases.permute_normalize(M, rng)
            for k in range(3, params[0] + 1, 3):
                todo.append((G.pack_rows(oracle.bibd_normalize(P[:k])), params[1]))
    for i in range(6):
        todo.append((oracle.sts_random_rows(15, 78, i), 35))
    for rows, b in todo:
        n = len(rows)
        full = maxsearch(host, rows, n, b, True)
        imp, aut = _split2_result(host, rows, n, b)
        assert imp == full["improved"]
        if not imp:
            assert aut == full["aut"], (n, aut, full["aut"])


def test_search_split_by_first_row_combines_to_the_whole(host):
    """One thread per first row (the enumerator's small-batch check): the verdict is
    the OR of the threads', |Aut| = (rows found in the orbit of row 0) x (the
    identity thread's product below level 0) -- equal to the unsplit search."""
    import ise_gb300 as G
    rng = np.random.default_rng(8)
    cases_ = []
    for M, _ in cases.load_sts15()[::3]:
        cases_.append((G.pack_rows(M), 35))
        P = cases.permute_normalize(M, rng)
        for k in (5, 9, 12, 15):
            cases_.append((G.pack_rows(oracle.bibd_normalize(P[:k])), 35))
    for params in [(8, 14, 7, 4, 3), (11, 11, 5, 5, 2), (13, 26, 6, 3, 1), (9, 12, 4, 3, 1)]:
        for M, _ in cases.bibd_designs(*params):
            cases_.append((G.pack_rows(M), params[1]))
            P = cases.permute_normalize(M, rng)
            for k in range(3, params[0] + 1, 2):
                cases_.append((G.pack_rows(oracle.bibd_normalize(P[:k])), params[1]))
    for i in range(10):
        cases_.append((oracle.sts_random_rows(15, 77, i), 35))
    for rows, b in cases_:
        n = len(rows)
        full = maxsearch(host, rows, n, b, True)
        imp, aut = _split_result(host, rows, n, b)
        assert imp == full["improved"]
        if not imp:
            assert aut == full["aut"]


def _search(fn, rows, n, b, order0=0xFEDCBA9876543210, mode=0):
    u64 = ctypes.c_uint64
    leaves, nodes, imp = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint8()
    rc = fn(rows.ctypes.data_as(ctypes.POINTER(u64)), n, b, ctypes.c_uint64(order0), ctypes.byref(leaves),
            ctypes.byref(nodes), ctypes.byref(imp), mode)
    assert rc == 0
    return leaves.value, nodes.value, imp.value


def _conv_vs_max(L, rows, n, b, order0=0xFEDCBA9876543210, aut_only=0):
    return [_search(L.emu_conv_search, rows, n, b, order0, 0),
            _search(L.emu_maxsearch_order, rows, n, b, order0, aut_only)]


def test_restart_and_aut_of_m_give_the_same_verdict_and_order(host):
    """The converged lex-max pass restarts on its bound once it is a complete greater
    matrix (after RESTART_AFTER nodes, or always); the thread-per-matrix pass falls back
    to keeping the bound at M after CLIMB_CAP nodes.  Every mode gives the verdict and
    |Aut| of the plain climb, with far fewer nodes on relabelled matrices of large
    groups; the 80 STS(15) classes relabelled at random, and partial matrices."""
    rng = np.random.default_rng(80)
    worst = {"climb": 0, "restart": 0, "cap": 0}
    for M, aut in cases.load_sts15():
        X = cases.permute_normalize(M, rng)
        r = np.ascontiguousarray(G.pack_rows(X), np.uint64)
        climb, mclimb = _conv_vs_max(host, r, 15, 35)
        assert climb == mclimb and climb[0] == aut
        for mode in (1, 2):
            a = _search(host.emu_conv_search, r, 15, 35, mode=mode)
            assert a[0] == aut and a[2] == climb[2]
            m = _search(host.emu_maxsearch_order, r, 15, 35, mode=mode)
            assert m[0] == aut and m[2] == climb[2]
        # verdict only: stops at the first greater node, the verdict is the climb's
        vo = _search(host.emu_conv_search, r, 15, 35, mode=3)
        assert vo[2] == climb[2] and (vo[2] or vo[0] == aut)
        worst["climb"] = max(worst["climb"], climb[1])
        worst["restart"] = max(worst["restart"], _search(host.emu_conv_search, r, 15, 35, mode=1)[1])
        worst["cap"] = max(worst["cap"], _search(host.emu_maxsearch_order, r, 15, 35, mode=2)[1])
        for k in (4, 7, 10):
            p = np.ascontiguousarray(r[:k])
            c2 = _search(host.emu_conv_search, p, k, 35)
            for mode in (1, 2):
                a2 = _search(host.emu_conv_search, p, k, 35, mode=mode)
                assert a2[0] == c2[0] and a2[2] == c2[2]
            v2 = _search(host.emu_conv_search, p, k, 35, mode=3)
            assert v2[2] == c2[2] and (v2[2] or v2[0] == c2[0])
            m2 = _search(host.emu_maxsearch_order, p, k, 35, mode=1)
            assert m2[0] == c2[0] and m2[2] == c2[2]
    # both bound the longest search (the relabelled PG(3,2): 151,636 nodes climbing)
    assert worst["restart"] < worst["climb"] and worst["cap"] < worst["climb"]
    print(worst)


def test_converged_layout_walks_the_same_tree(host):
    """The converged search (canon_bibd_conv.cuh) visits exactly the nodes of
    max_search() and gives the same verdict and |Aut|, in the plain order and under a
    first-row order, on complete and partial matrices of several shapes."""
    rng = np.random.default_rng(77)
    cases_ = [np.stack([oracle.sts_random_rows(15, 99, i) for i in range(40)])]
    sts = cases.load_sts15()
    cases_.append(np.stack([G.pack_rows(M) for M, _ in sts]))
    for rows in cases_:
        for r in rows:
            r = np.ascontiguousarray(r, np.uint64)
            a, m = _conv_vs_max(host, r, 15, 35)
            assert a == m
            order = rng.permutation(15)
            o0 = sum(int(x) << (4 * q) for q, x in enumerate(order))
            a, m = _conv_vs_max(host, r, 15, 35, o0)
            assert a == m
            for k in (5, 9, 12):
                p = np.ascontiguousarray(r[:k])
                a, m = _conv_vs_max(host, p, k, 35)
                assert a == m
    u64 = ctypes.c_uint64
    for params in ((8, 14, 7, 4, 3), (11, 11, 5, 5, 2), (13, 26, 6, 3, 1), (7, 14, 6, 3, 2)):
        for M, _ in cases.bibd_designs(*params):
            X = cases.permute_normalize(M, rng)
            r = np.ascontiguousarray(G.pack_rows(X), np.uint64)
            for k in range(2, params[0] + 1):
                p = np.ascontiguousarray(r[:k])
                a, m = _conv_vs_max(host, p, k, params[1])
                assert a == m, (params, k)
                # walking more columns than the matrix has (the widest item of a mixed
                # launch) changes nothing
                leaves, nodes, imp = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint8()
                assert host.emu_conv_search_bt(p.ctypes.data_as(ctypes.POINTER(u64)), k, params[1], 35,
                                               ctypes.c_uint64(0xFEDCBA9876543210), ctypes.byref(leaves),
                                               ctypes.byref(nodes), ctypes.byref(imp), 0) == 0
                assert (leaves.value, nodes.value, imp.value) == a, (params, k)


def test_converged_layout_with_four_and_six_count_planes(host):
    """The node step counts with 3, 4 or 6 bit planes by the matrix's greatest row
    weight (<= 7, <= 15, more).  Heavier rows take the 4- and 6-plane paths: the
    BIBD(9,18,8,4,3) designs (weight 8) and their prefixes, and random 0/1 matrices of
    weights around 12 and 20, must walk the same tree as max_search()."""
    rng = np.random.default_rng(78)
    for M, _ in cases.bibd_designs(9, 18, 8, 4, 3):
        X = cases.permute_normalize(M, rng)
        r = np.ascontiguousarray(G.pack_rows(X), np.uint64)
        for k in (3, 6, 9):
            a, m = _conv_vs_max(host, np.ascontiguousarray(r[:k]), k, 18)
            assert a == m, k
    for v, b, dens in ((10, 24, 0.5), (8, 40, 0.5), (6, 63, 0.45)):
        for _ in range(6):
            X = (rng.random((v, b)) < dens).astype(np.uint8)
            X[:, 0] = 1                      # no empty matrix
            r = np.ascontiguousarray(G.pack_rows(X), np.uint64)
            w = int(X.sum(axis=1).max())
            assert w > 7
            a, m = _conv_vs_max(host, r, v, b)
            assert a == m, (v, b, w)
