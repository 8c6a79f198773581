"""Config 3 at its full size: the 2,097,152-item uneven mix (partial STS(15),
BIBD(8,14,7,4,3), BIBD(11,11,5,5,2) and K10 1-factorizations, each made by
seeded random backtracking of its filled rows) checked in one persistent launch
through the C ABI, and every 128th item of every shape compared with the oracle:
verdict, witness and rejecting row of the rejected, |Aut| of the canonical
(incidence matrices); verdict, player index, relabelings tried and |Aut|
(k-systems)."""
import concurrent.futures as cf
import os

import numpy as np
import pytest

import ise_gb300 as G
import oracle
from ise_gb300 import workloads

pytestmark = pytest.mark.gpu

STRIDE = 128


def _oracle_bibd(M):
    return oracle.bibd_test(oracle.bibd_normalize(M), oracle.SAVE_NOTHING)


def test_config3_full_mix_sample_matches_oracle():
    batches = workloads.config3_mix()
    n = sum(len(bt["nrows"]) for bt in batches)
    assert n == workloads.MIX_ITEMS
    ctx = G.Context(max_items=n + 16, max_words=16 * n, aut_cap=1)
    try:
        workloads.submit_mix(ctx, batches)
        r = ctx.sync(raw=True)
    finally:
        ctx.close()
    assert r["n"] == n and not r["status"].any()
    # the verdict-only sync (CANON_OPT_VERDICT_SYNC) returns the same verdicts
    ctx = G.Context(max_items=n + 16, max_words=16 * n, aut_cap=1, options=G.OPT_VERDICT_SYNC)
    try:
        workloads.submit_mix(ctx, batches)
        rv = ctx.sync(raw=True)
    finally:
        ctx.close()
    assert np.array_equal(rv["canonical"], r["canonical"]) and np.array_equal(rv["status"], r["status"])
    off = 0
    with cf.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        for bt in batches:
            cnt = len(bt["nrows"])
            idx = np.arange(0, cnt, STRIDE)
            if bt["kind"] == "bibd":
                b = bt["b"]
                mats = [oracle.rows_to_matrix(bt["data"][i, :bt["nrows"][i]], b) for i in idx]
                for i, M, o in zip(idx, mats, ex.map(_oracle_bibd, mats)):
                    j = off + i
                    assert bool(r["canonical"][j]) == o["canonical"], (bt["name"], i)
                    if o["canonical"]:
                        assert int(r["aut"][j, 0]) == o["aut"] and r["aut"][j, 1] == 0, (bt["name"], i)
                    else:
                        assert int(r["reject_row"][j]) == o["reject_row"], (bt["name"], i)
                        assert bytes(r["witness"][j][:M.shape[0]]) == o["witness"], (bt["name"], i)
            else:
                mats = [bt["data"][i, :bt["nrows"][i]] for i in idx]
                for i, o in zip(idx, ex.map(oracle.ksys_test, mats)):
                    j = off + i
                    assert bool(r["canonical"][j]) == o["canonical"], (bt["name"], i)
                    assert int(r["player_index"][j]) == o["player_index"], (bt["name"], i)
                    assert int(r["trials"][j]) == o["candidates"], (bt["name"], i)
                    if o["canonical"]:
                        assert int(r["aut"][j, 0]) == o["n_aut"], (bt["name"], i)
            off += cnt
