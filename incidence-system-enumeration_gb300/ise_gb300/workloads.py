"""Seeded inputs of the benchmark configurations, shared by bench.py and the tests.

config3_mix(): the uneven batch of one persistent check launch -- 2,097,152
partial matrices: 40% STS(15) with 5-15 rows, 30% BIBD(8,14,7,4,3) with 4-8
rows, 20% BIBD(11,11,5,5,2) with 4-11 rows, 10% 1-factorizations of K10 with
3-9 rounds.  Each item is made by seeded random backtracking of its filled rows
(canon_generate_partial_bibd / canon_generate_partial_ksys), uniform over the row
counts, so the batch holds the dead-end partial matrices that an orderly
enumerator meets as well as prefixes of complete designs.
"""
import numpy as np

from . import RAW, generate_partial_bibd, generate_partial_ksys

# (share, kind, (v, b, r, k, lambda) or np, min rows filled, max rows filled)
MIX_SHAPES = [
    (0.40, "bibd", (15, 35, 7, 3, 1), 5, 15),
    (0.30, "bibd", (8, 14, 7, 4, 3), 4, 8),
    (0.20, "bibd", (11, 11, 5, 5, 2), 4, 11),
    (0.10, "ksys", 10, 3, 9),
]
MIX_ITEMS = 2_097_152
MIX_FLAGS_BIBD = RAW          # partial check (t_saveNothing) of arbitrary 0/1 rows
MIX_FLAGS_KSYS = 0


def config3_mix(n_total=MIX_ITEMS, seed=20241206):
    """The batches of the uneven mix, in submission order: a list of dicts with
    kind, name, shape, data (rows or round bytes), nrows, flags, and the number of
    items taken from a complete design (STS(15) with 14-15 rows)."""
    batches = []
    for i, (share, kind, params, lo, hi) in enumerate(MIX_SHAPES):
        cnt = int(round(share * n_total))
        s = seed + 7919 * (i + 1)
        if kind == "bibd":
            rows, nrows, from_complete = generate_partial_bibd(params, cnt, s, lo, hi)
            batches.append(dict(kind="bibd", name="BIBD(%d,%d,%d,%d,%d)" % params, params=params, v=params[0],
                                b=params[1], data=rows, nrows=nrows, flags=MIX_FLAGS_BIBD,
                                from_complete=from_complete))
        else:
            data, nrows = generate_partial_ksys(params, cnt, s, lo, hi)
            batches.append(dict(kind="ksys", name="K%d" % params, params=(params,), v=params, b=params - 1,
                                data=data, nrows=nrows, flags=MIX_FLAGS_KSYS, from_complete=0))
    return batches


def submit_mix(ctx, batches):
    for bt in batches:
        if bt["kind"] == "bibd":
            ctx.submit_bibd(bt["data"], bt["v"], bt["b"], bt["flags"], bt["nrows"])
        else:
            ctx.submit_ksys(bt["data"], bt["v"], bt["b"], bt["flags"], bt["nrows"])
    return sum(len(bt["nrows"]) for bt in batches)


def mix_input_bytes(batches):
    return int(sum(bt["data"].nbytes + bt["nrows"].nbytes for bt in batches))


__all__ = ["MIX_SHAPES", "MIX_ITEMS", "config3_mix", "submit_mix", "mix_input_bytes"]
