"""canon_check_bibd_noalloc: the check for callers that cannot allocate device
memory (a host whose device memory belongs to another allocator or a fixed
arena, latency paths that cannot take cudaMalloc's device synchronisation).
It is called through the C ABI and must give exactly what the batched entry
point (canon_submit_bibd + canon_sync) gives, on two calls in a row, which also
shows that the shared static scratch is reset between calls; the free device
memory must not change across a call.  Collected last so that a run stopping at
the first failure has run everything else already."""
import ctypes

import numpy as np
import pytest

import cases
import ise_gb300 as G
import oracle

pytestmark = pytest.mark.gpu

FIELDS = [("canonical", 1, np.uint8), ("status", 1, np.uint8), ("reject_row", 1, np.uint8),
          ("row_to_change", 1, np.uint8), ("player_index", 4, np.int32), ("witness", 16, np.uint8),
          ("aut", 16, np.uint64), ("trials", 8, np.uint64), ("n_auts", 2, np.uint16),
          ("len_aut", 1, np.uint8)]


def batch(seed):
    rng = np.random.default_rng(seed)
    sts = cases.load_sts15()
    mats = [oracle.bibd_normalize(oracle.rows_to_matrix(oracle.sts_random_rows(15, seed, i), 35))
            for i in range(24)]
    mats += [M for M, _ in sts[::6]]
    rows = np.zeros((len(mats) * 2, 15), np.uint64)
    nrows = np.zeros(len(mats) * 2, np.uint8)
    for i, M in enumerate(mats):
        rows[2 * i] = G.pack_rows(M)
        nrows[2 * i] = 15
        k = int(rng.integers(3, 15))
        P = oracle.bibd_normalize(M[:k])
        rows[2 * i + 1, :k] = G.pack_rows(P)
        nrows[2 * i + 1] = k
    return rows, nrows


def run_noalloc(ctx, rows, nrows, flags, aut_cap=16, pass_nrows=True):
    import torch
    n = len(rows)
    lib = G.load_library()
    d_rows = ctx.alloc(rows.nbytes)
    d_nrows = ctx.alloc(n)
    ctx.h2d(d_rows, rows)
    ctx.h2d(d_nrows, nrows)
    ptrs = {name: ctx.alloc(n * size) for name, size, _ in FIELDS}
    ptrs["auts"] = ctx.alloc(n * aut_cap * 64)
    try:
        out = G.DeviceOutputs(**{k: ptrs[k] for k in ptrs}, aut_cap=aut_cap)
        free = []
        # the same call twice: the first may load the kernels' code (lazy module
        # loading); around the second the free device memory must not change
        for _ in range(2):
            torch.cuda.synchronize()
            free.append(torch.cuda.mem_get_info()[0])
            rc = lib.canon_check_bibd_noalloc(n, 15, 35, flags, d_rows, d_nrows if pass_nrows else None,
                                              ctypes.byref(out), 1 << 24, None)
            assert rc == G.CANON_OK
            # launched on the default stream, which the context's (non-blocking) stream does not wait for
            torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free[1], "the call changed the free device memory"
    except Exception:
        for p in list(ptrs.values()) + [d_rows, d_nrows]:
            ctx.free(p)
        raise
    res = {}
    for name, size, dt in FIELDS:
        host = np.zeros(n * size, np.uint8)
        ctx.d2h(host, ptrs[name])
        res[name] = host.view(dt)
    auts = np.zeros(n * aut_cap * 64, np.uint8)
    ctx.d2h(auts, ptrs["auts"])
    res["auts"] = auts.reshape(n, aut_cap, 64)
    for p in list(ptrs.values()) + [d_rows, d_nrows]:
        ctx.free(p)
    return res


def run_batched(ctx, rows, nrows, flags):
    ctx.submit_bibd(rows, 15, 35, flags, nrows)
    return ctx.sync()


@pytest.mark.parametrize("flags", [0, G.COMPLETE | G.AUT_CANON, G.SAVE_AUTS])
def test_noalloc_matches_batched_entry_point_twice(flags):
    ctx = G.Context(max_items=1024, aut_cap=16, max_trials=1 << 24)
    try:
        for call in range(2):
            rows, nrows = batch(1000 + call)
            got = run_noalloc(ctx, rows, nrows, flags)
            ref = run_batched(ctx, rows, nrows, flags)
            n = len(nrows)
            assert np.array_equal(got["canonical"], ref["canonical"].astype(np.uint8)), call
            assert np.array_equal(got["status"], ref["status"]), call
            assert np.array_equal(got["reject_row"], ref["reject_row"]), call
            assert np.array_equal(got["row_to_change"], ref["row_to_change"]), call
            assert np.array_equal(got["witness"].reshape(n, 16), ref["witness"]), call
            assert [int(a) | (int(b) << 64) for a, b in got["aut"].reshape(n, 2)] == ref["aut"], call
            assert np.array_equal(got["trials"], ref["trials"]), call
            if flags & G.SAVE_AUTS:
                assert np.array_equal(got["n_auts"], ref["n_auts"]), call
                for i in range(n):
                    k, ln = min(int(ref["n_auts"][i]), 16), int(ref["len_aut"][i])
                    assert np.array_equal(got["auts"][i][:k, :ln], ref["auts_raw"][i][:k, :ln]), (call, i)
    finally:
        ctx.close()


def test_noalloc_flags_bad_row_counts_per_matrix_and_takes_null_counts():
    """A filled-row count of 0 or above v marks that matrix CANON_ST_BADINPUT and
    leaves the others checked; without counts every matrix has all v rows."""
    ctx = G.Context(max_items=1024, aut_cap=16, max_trials=1 << 24)
    try:
        rows, nrows = batch(2024)
        full = rows[nrows == 15]
        bad = nrows.copy()
        bad[1], bad[4] = 0, 16
        got = run_noalloc(ctx, rows, bad, 0)
        assert got["status"][1] == G.ST_BADINPUT and got["status"][4] == G.ST_BADINPUT
        assert got["canonical"][1] == 0 and got["canonical"][4] == 0
        keep = np.ones(len(bad), bool)
        keep[[1, 4]] = False
        ref = run_batched(ctx, rows[keep], nrows[keep], 0)
        assert np.array_equal(got["canonical"][keep], ref["canonical"].astype(np.uint8))
        assert np.array_equal(got["witness"].reshape(-1, 16)[keep], ref["witness"])
        got = run_noalloc(ctx, full, np.full(len(full), 15, np.uint8), G.COMPLETE, pass_nrows=False)
        ref = run_batched(ctx, full, None, G.COMPLETE)
        assert np.array_equal(got["canonical"], ref["canonical"].astype(np.uint8))
        assert np.array_equal(got["witness"].reshape(-1, 16), ref["witness"])
    finally:
        ctx.close()


def test_noalloc_refuses_batches_beyond_the_scratch():
    lib = G.load_library()
    out = G.DeviceOutputs()
    rc = lib.canon_check_bibd_noalloc(G.NOALLOC_MAX_ITEMS + 1, 15, 35, 0, 1, None, ctypes.byref(out), 0, None)
    assert rc == G.CANON_ESIZE
