"""The k-system check with every matrix's candidates split over warps
(canon_set_ksys_segment) against the one-warp-per-matrix check and the oracle:
verdict, status, m_playerIndex, relabelings tried and |Aut| must be identical for
every segment size, on complete, relabelled and partial K10 matrices, K8 matrices
in the same sync, and an ill-formed item; and the K10 enumeration must give the
same designs in the same order with the same relabelings tried."""
import numpy as np
import pytest

import cases
import ise_gb300 as G
import oracle

pytestmark = pytest.mark.gpu

FIELDS = ["canonical", "status", "player_index", "trials", "aut", "reject_row", "row_to_change"]


def batch(seed):
    rng = np.random.default_rng(seed)
    k10 = cases.load_k10()
    mats, nrows = [], []
    for R, _ in k10[::2]:
        X = cases.ksys_relabel_random(R, rng) if rng.integers(2) else R
        k = int(rng.integers(2, 10))
        P = X if k == 9 else X[:k]
        if k < 9 and rng.integers(2):
            P = cases.ksys_relabel_random(P, rng)
        pad = np.zeros((9, 10), np.uint8)
        pad[:k] = P
        mats.append(pad)
        nrows.append(k)
    bad = mats[3].copy()
    bad[1, 0], bad[1, 1] = bad[1, 1], bad[1, 0]    # a pair out of order: ill formed
    mats.append(bad)
    nrows.append(9)
    k8, _ = oracle.ksys_enumerate(8)
    return np.stack(mats), np.array(nrows, np.uint8), np.stack([R for R, _ in k8])


def run(ctx, seg, mats, nrows, k8):
    ctx.set_ksys_segment(seg)
    ctx.submit_ksys(mats, 10, 9, 0, nrows)
    ctx.submit_ksys(k8, 8, 7, 0)
    return ctx.sync()


def test_split_check_equals_one_warp_per_matrix_and_the_oracle(ctx):
    mats, nrows, k8 = batch(31)
    try:
        whole = run(ctx, G.KSYS_WHOLE, mats, nrows, k8)
        for seg in [32, 256, 1000, 4096, 0]:
            r = run(ctx, seg, mats, nrows, k8)
            for f in FIELDS:
                assert np.array_equal(np.asarray(r[f]), np.asarray(whole[f])), (seg, f)
    finally:
        ctx.set_ksys_segment(0)
    n = len(nrows)
    assert whole["status"][n - 1] & G.ST_BADINPUT
    for i in list(range(0, n - 1, 7)):
        o = oracle.ksys_test(mats[i][:nrows[i]])
        assert bool(whole["canonical"][i]) == o["canonical"], i
        assert int(whole["player_index"][i]) == o["player_index"], i
        assert int(whole["trials"][i]) == o["candidates"], i
        if o["canonical"]:
            assert whole["aut"][i] == o["n_aut"], i
    for j in range(len(k8)):
        assert whole["canonical"][n + j]


def test_k10_enumeration_is_the_same_under_every_split(ctx):
    runs = []
    try:
        for seg in [G.KSYS_WHOLE, 256, 0]:
            ctx.set_ksys_segment(seg)
            found, st = ctx.enumerate_ksys(10)
            runs.append(([(R.tobytes(), a) for R, a in found], int(st.trials), int(st.checks)))
    finally:
        ctx.set_ksys_segment(0)
    assert len(runs[0][0]) == 396
    assert runs[1] == runs[0] and runs[2] == runs[0]


def _enum(ctx, np_):
    found, st = ctx.enumerate_ksys(np_)
    return [(R.tobytes(), a) for R, a in found], int(st.trials), int(st.checks), list(st.level_checks)


def test_captured_graph_enumeration_equals_level_by_level():
    """canon_enumerate_ksys replays one captured CUDA graph (level sizes in device
    memory); CANON_OPT_NO_GRAPH runs level by level.  Same designs in the same order,
    same relabelings tried and per-level checks, for K6, K8 and K10; a context whose
    item capacity is below K10's largest level (4,092) overflows the graph's buffers,
    falls back to the level-by-level run, and replays a 4x larger graph next time."""
    plain = G.Context(max_items=1 << 16, aut_cap=4, options=G.OPT_NO_GRAPH)
    graph = G.Context(max_items=1 << 16, aut_cap=4)
    small = G.Context(max_items=1024, aut_cap=4)
    try:
        for np_ in (6, 8, 10):
            ref = _enum(plain, np_)
            assert _enum(graph, np_) == ref, np_
            assert _enum(graph, np_) == ref, np_          # the cached graph, replayed
        ref10 = _enum(plain, 10)
        assert len(ref10[0]) == 396
        l0 = small.kernel_launches()
        assert _enum(small, 10) == ref10                  # overflow: level by level
        l1 = small.kernel_launches()
        assert _enum(small, 10) == ref10                  # 4,096 fits: the graph
        l2 = small.kernel_launches()
        assert l1 - l0 != l2 - l1
    finally:
        plain.close()
        graph.close()
        small.close()
