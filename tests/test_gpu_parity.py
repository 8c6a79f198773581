"""CUDA path against the CPU oracle on the same seeded inputs (bit-exact)."""
import numpy as np
import pytest

import cases
import ise_gb300 as G
import oracle

pytestmark = pytest.mark.gpu

COMPLETE = oracle.SAVE_ROW_PERM | oracle.SAVE_ROW_TO_CHANGE


def oracle_bibd(M, gflags):
    f = COMPLETE if gflags & G.COMPLETE else 0
    if gflags & G.FULL_AUT:
        f |= oracle.FULL_AUT
    if gflags & G.SAVE_AUTS and gflags & G.COMPLETE:
        f |= oracle.SAVE_AUT_ROWS
    X = oracle.bibd_normalize(M) if gflags & G.RAW else M
    o = oracle.bibd_test(X, f, perm_cap=64 if gflags & G.SAVE_AUTS else 0)
    if gflags & G.AUT_CANON and not o["canonical"]:
        _, o["aut"], _ = oracle.bibd_canonize(X)
    return o


def compare_bibd(ctx, mats, gflags, v, b):
    rows = np.zeros((len(mats), v), np.uint64)
    nrows = np.zeros(len(mats), np.uint8)
    for i, M in enumerate(mats):
        rows[i, :M.shape[0]] = G.pack_rows(M)
        nrows[i] = M.shape[0]
    ctx.submit_bibd(rows, v, b, gflags, nrows)
    r = ctx.sync()
    assert r["n"] == len(mats)
    for i, M in enumerate(mats):
        o = oracle_bibd(M, gflags)
        n = M.shape[0]
        assert r["status"][i] == 0, (i, r["status"][i])
        assert bool(r["canonical"][i]) == o["canonical"], i
        if gflags & (G.REFERENCE_ORDER | G.SAVE_AUTS):
            assert int(r["trials"][i]) == o["trials"], i
        if not o["canonical"]:
            assert int(r["reject_row"][i]) == o["reject_row"], i
            assert bytes(r["witness"][i][:n]) == o["witness"], i
            if gflags & G.COMPLETE:
                assert int(r["row_to_change"][i]) == o["row_to_change"], i
        if o["canonical"] or gflags & (G.FULL_AUT | G.AUT_CANON):
            assert r["aut"][i] == o["aut"], (i, r["aut"][i], o["aut"])
        if gflags & G.SAVE_AUTS:
            k = int(r["n_auts"][i])
            assert k == o["n_perm"], i
            ln = int(r["len_aut"][i])
            kk = min(k, 64)
            assert np.array_equal(r["auts_raw"][i][:kk, :ln], o["perms"][:kk, :ln]), i
    return r


def test_sts15_complete_raw_full_aut(ctx):
    mats = [oracle.rows_to_matrix(oracle.sts_random_rows(15, 2024, i), 35) for i in range(12)]
    sts = cases.load_sts15()
    mats += [M for M, _ in sts[::5]]
    compare_bibd(ctx, mats, G.COMPLETE | G.RAW | G.FULL_AUT, 15, 35)
    compare_bibd(ctx, mats, G.COMPLETE | G.RAW | G.FULL_AUT | G.REFERENCE_ORDER, 15, 35)


def test_sts15_complete_aut_by_canonization(ctx):
    mats = [oracle.rows_to_matrix(oracle.sts_random_rows(15, 4048, i), 35) for i in range(128)]
    sts = cases.load_sts15()
    mats += [M for M, _ in sts[1::3]]
    r = compare_bibd(ctx, mats, G.COMPLETE | G.RAW | G.AUT_CANON, 15, 35)
    fixture = {a for _, a in sts}
    assert all(a in fixture for a in r["aut"])
    compare_bibd(ctx, mats[:40], G.COMPLETE | G.RAW | G.AUT_CANON | G.REFERENCE_ORDER, 15, 35)


def test_sts15_complete_reference_semantics(ctx):
    rng = np.random.default_rng(1)
    sts = cases.load_sts15()
    mats = [cases.permute_normalize(M, rng) for M, _ in sts[:40]] + [M for M, _ in sts[40:]]
    compare_bibd(ctx, mats, G.COMPLETE, 15, 35)
    compare_bibd(ctx, mats, G.COMPLETE | G.REFERENCE_ORDER, 15, 35)


def test_partial_matrices_mixed_shapes_with_automorphisms(ctx):
    rng = np.random.default_rng(2)
    sts = cases.load_sts15()
    groups = {(15, 35): [], (8, 14): [], (11, 11): [], (13, 26): []}
    for M, _ in sts[::4]:
        P = cases.permute_normalize(M, rng) if rng.integers(2) else M
        k = int(rng.integers(2, 16))
        groups[(15, 35)].append(oracle.bibd_normalize(P[:k]))
    for params, key in [((8, 14, 7, 4, 3), (8, 14)), ((11, 11, 5, 5, 2), (11, 11)),
                        ((13, 26, 6, 3, 1), (13, 26))]:
        for M, _ in cases.bibd_designs(*params):
            for _ in range(6):
                P = cases.permute_normalize(M, rng) if rng.integers(3) else M
                k = int(rng.integers(2, M.shape[0] + 1))
                groups[key].append(oracle.bibd_normalize(P[:k]))
    for (v, b), mats in groups.items():
        compare_bibd(ctx, mats, G.SAVE_AUTS, v, b)
        compare_bibd(ctx, mats, G.SAVE_AUTS | G.FULL_AUT, v, b)
        compare_bibd(ctx, mats, 0, v, b)
        compare_bibd(ctx, mats, G.FULL_AUT, v, b)


def test_complete_small_designs_save_row_automorphisms(ctx):
    rng = np.random.default_rng(4)
    mats = []
    for params in [(7, 7, 3, 3, 1), (8, 14, 7, 4, 3), (11, 11, 5, 5, 2), (7, 14, 6, 3, 2),
                   (9, 12, 4, 3, 1)]:
        for M, _ in cases.bibd_designs(*params):
            mats_p = [M] + [cases.permute_normalize(M, rng) for _ in range(3)]
            v, b = M.shape
            compare_bibd(ctx, mats_p, G.COMPLETE | G.SAVE_AUTS | G.FULL_AUT, v, b)


def test_canonize_matches_oracle_and_fixture(ctx):
    sts = cases.load_sts15()
    canon = {M.tobytes(): a for M, a in sts}
    raw = np.stack([oracle.sts_random_rows(15, 77, i) for i in range(64)])
    rows, auts = ctx.canonize_bibd(raw, 15, 35)
    for i in range(64):
        C = G.unpack_rows(rows[i], 35)
        Co, ao, _ = oracle.bibd_canonize(oracle.rows_to_matrix(raw[i], 35))
        assert np.array_equal(C, Co)
        assert C.tobytes() in canon and auts[i] == ao == canon[C.tobytes()]


def test_generator_matches_oracle_stream(ctx):
    n = 256
    d = ctx.alloc(n * 15 * 8)
    try:
        ctx.generate_sts_device(n, 15, 123456789, False, d)
        got = ctx.d2h(np.zeros(n * 15, np.uint64), d).reshape(n, 15)
    finally:
        ctx.free(d)
    for i in range(n):
        assert np.array_equal(got[i], oracle.sts_random_rows(15, 123456789, i)), i


def test_device_entry_point_matches_batched_path(ctx):
    n = 200
    d_rows = ctx.alloc(n * 15 * 8)
    d_can = ctx.alloc(n)
    d_wit = ctx.alloc(n * 16)
    d_aut = ctx.alloc(n * 16)
    d_st = ctx.alloc(n)
    try:
        ctx.generate_sts_device(n, 15, 5, True, d_rows)
        ctx.check_bibd_device(n, 15, 35, G.COMPLETE | G.RAW | G.AUT_CANON, d_rows, d_can, d_wit, d_aut, d_st)
        ctx.stream_sync()
        rows = ctx.d2h(np.zeros(n * 15, np.uint64), d_rows).reshape(n, 15)
        can = ctx.d2h(np.zeros(n, np.uint8), d_can)
        wit = ctx.d2h(np.zeros(n * 16, np.uint8), d_wit).reshape(n, 16)
        aut = ctx.d2h(np.zeros(2 * n, np.uint64), d_aut).reshape(n, 2)
        st = ctx.d2h(np.zeros(n, np.uint8), d_st)
    finally:
        for p in (d_rows, d_can, d_wit, d_aut, d_st):
            ctx.free(p)
    assert not st.any()
    sts = {M.tobytes(): a for M, a in cases.load_sts15()}
    for i in range(n):
        M = oracle.rows_to_matrix(rows[i], 35)
        o = oracle_bibd(M, G.COMPLETE | G.RAW | G.AUT_CANON)
        assert bool(can[i]) == o["canonical"]
        assert int(aut[i][0]) == o["aut"]
        if not o["canonical"]:
            assert bytes(wit[i][:15]) == o["witness"]
        if i % 2:
            assert M.tobytes() in sts and bool(can[i])


def test_ksys_golden_k10_complete(ctx):
    k10 = cases.load_k10()
    data = np.stack([R for R, _ in k10])
    ctx.submit_ksys(data, 10, 9, G.SAVE_AUTS)
    r = ctx.sync()
    for i, (R, aut) in enumerate(k10):
        assert r["canonical"][i] and r["aut"][i] == aut, i
    for i in range(0, 396, 37):
        o = oracle.ksys_test(k10[i][0], aut_cap=64)
        k = int(r["n_auts"][i])
        assert k == min(o["n_aut"], 64)
        assert np.array_equal(r["auts_raw"][i][:k, :10], o["auts"][:k])
        assert int(r["trials"][i]) == o["candidates"]


def test_ksys_relabelled_and_partial(ctx):
    rng = np.random.default_rng(9)
    k10 = cases.load_k10()
    mats, nrows = [], []
    for R, _ in k10[::3]:
        X = cases.ksys_relabel_random(R, rng) if rng.integers(2) else R
        k = int(rng.integers(2, 10))
        P = X[:k] if k < 9 else X
        if k < 9 and rng.integers(2):
            P = cases.ksys_relabel_random(P, rng)
        pad = np.zeros((9, 10), np.uint8)
        pad[:k] = P
        mats.append(pad)
        nrows.append(k)
    ctx.submit_ksys(np.stack(mats), 10, 9, 0, np.array(nrows, np.uint8))
    r = ctx.sync()
    for i, (M, k) in enumerate(zip(mats, nrows)):
        o = oracle.ksys_test(M[:k])
        assert r["status"][i] == 0, i
        assert bool(r["canonical"][i]) == o["canonical"], i
        assert int(r["player_index"][i]) == o["player_index"], (i, r["player_index"][i], o["player_index"])
        assert int(r["trials"][i]) == o["candidates"], i
        if o["canonical"]:
            assert r["aut"][i] == o["n_aut"], i


def test_edge_cases(ctx):
    # empty batch
    r = ctx.sync()
    assert r["n"] == 0
    # a single row, one column, maximum width, and a non-normal matrix
    one = np.array([[1]], np.uint8)
    wide = np.zeros((2, 63), np.uint8)
    wide[0, :32] = 1
    wide[1, :16] = 1
    wide[1, 32:48] = 1
    compare_bibd(ctx, [one], G.COMPLETE, 1, 1)
    compare_bibd(ctx, [wide], G.COMPLETE | G.FULL_AUT, 2, 63)
    bad = np.array([[0, 1, 1]], np.uint8)
    ctx.submit_bibd(G.pack_rows(bad), 1, 3, 0)
    r = ctx.sync()
    assert r["status"][0] & G.ST_BADINPUT
    # invalid arguments are rejected on the host
    with pytest.raises(G.CanonError):
        ctx.submit_bibd(np.zeros(17, np.uint64), 17, 10, 0)
    with pytest.raises(G.CanonError):
        ctx.submit_bibd(np.zeros(2, np.uint64), 2, 64, 0)
    # malformed k-system rounds are flagged per item
    R = cases.load_k10()[0][0].copy()
    R[1, 0], R[1, 1] = R[1, 1], R[1, 0]
    ctx.submit_ksys(R, 10, 9, 0)
    r = ctx.sync()
    assert r["status"][0] & G.ST_BADINPUT


def test_trial_budget_reports_timeout_not_a_hang():
    ctx = G.Context(max_items=64, aut_cap=1, max_trials=4)
    try:
        M = cases.load_sts15()[0][0]
        ctx.submit_bibd(G.pack_rows(M), 15, 35, G.COMPLETE)
        with pytest.raises(G.CanonError) as e:
            ctx.sync()
        assert e.value.code == G.CANON_ETIMEOUT
        ctx.submit_bibd(G.pack_rows(M), 15, 35, G.COMPLETE)
        r = ctx.sync(allow_timeout=True)
        assert r["status"][0] & G.ST_TIMEOUT and not r["canonical"][0]
    finally:
        ctx.close()


def test_mixed_batch_one_persistent_launch(ctx):
    """Incidence matrices of three shapes and k-systems in one sync (the fused kernel)."""
    rng = np.random.default_rng(17)
    sts = cases.load_sts15()
    groups = []
    for params, cnt in [((15, 35, 7, 3, 1), 24), ((8, 14, 7, 4, 3), 16), ((11, 11, 5, 5, 2), 12)]:
        designs = [M for M, _ in sts] if params[0] == 15 else [M for M, _ in cases.bibd_designs(*params)]
        v, b = params[0], params[1]
        mats = []
        for _ in range(cnt):
            M = designs[int(rng.integers(len(designs)))]
            P = M[rng.permutation(v)][:, rng.permutation(b)]
            k = int(rng.integers(3, v + 1))
            mats.append(P[:k])
        groups.append((v, b, mats))
    k10 = cases.load_k10()
    kmats, knr = [], []
    for _ in range(20):
        R = cases.ksys_relabel_random(k10[int(rng.integers(396))][0], rng)
        k = int(rng.integers(3, 10))
        pad = np.zeros((9, 10), np.uint8)
        pad[:k] = R[:k]
        kmats.append(pad)
        knr.append(k)
    for v, b, mats in groups:
        rows = np.zeros((len(mats), v), np.uint64)
        nr = np.zeros(len(mats), np.uint8)
        for i, M in enumerate(mats):
            rows[i, :M.shape[0]] = G.pack_rows(M)
            nr[i] = M.shape[0]
        ctx.submit_bibd(rows, v, b, G.RAW | G.FULL_AUT, nr)
    ctx.submit_ksys(np.stack(kmats), 10, 9, 0, np.array(knr, np.uint8))
    r = ctx.sync()
    i = 0
    for v, b, mats in groups:
        for M in mats:
            o = oracle_bibd(M, G.RAW | G.FULL_AUT)
            assert r["status"][i] == 0
            assert bool(r["canonical"][i]) == o["canonical"], i
            assert r["aut"][i] == o["aut"], i
            if not o["canonical"]:
                assert bytes(r["witness"][i][:M.shape[0]]) == o["witness"], i
            i += 1
    for M, k in zip(kmats, knr):
        o = oracle.ksys_test(M[:k])
        assert bool(r["canonical"][i]) == o["canonical"] and int(r["player_index"][i]) == o["player_index"], i
        i += 1


def test_queue_survives_a_refused_batch_and_a_canonisation(ctx):
    """Batches are copied to the GPU when they are queued: a batch refused for a bad
    row count leaves the queue as it was, and canon_canonize_bibd (which borrows the
    device staging) between submit and sync makes the sync copy the queue again."""
    sts = cases.load_sts15()
    rng = np.random.default_rng(5)
    mats = [sts[int(rng.integers(80))][0][rng.permutation(15)][:, rng.permutation(35)] for _ in range(12)]
    rows = np.stack([G.pack_rows(M) for M in mats])
    nr = np.full(12, 15, np.uint8)
    ref = compare_bibd(ctx, mats, G.COMPLETE | G.RAW, 15, 35)
    ctx.submit_bibd(rows[:6], 15, 35, G.COMPLETE | G.RAW, nr[:6])
    bad = nr[6:].copy()
    bad[3] = 16
    with pytest.raises(G.CanonError):
        ctx.submit_bibd(rows[6:], 15, 35, G.COMPLETE | G.RAW, bad)
    ctx.submit_bibd(rows[6:], 15, 35, G.COMPLETE | G.RAW, nr[6:])
    canon_rows, _ = ctx.canonize_bibd(rows[:4], 15, 35)
    assert canon_rows.shape[0] == 4
    r = ctx.sync()
    assert r["n"] == 12
    assert np.array_equal(r["canonical"], ref["canonical"])
    assert np.array_equal(r["witness"], ref["witness"])
    assert r["aut"] == ref["aut"]
