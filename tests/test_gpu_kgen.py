"""The GPU check of k-systems with groups of 3 or 4 (canon_submit_ksys_groups) against
the oracle's cnvCheckNew() restatement and the reference's Kirkman results: the 7
Kirkman triple systems of 15 players are canonical with the reference's |Aut(M)| after
all 5! x 3!^5 x 7 - 1 relabelings; prefixes, relabelled copies and random partial
systems with groups of 3 and 4 give the oracle's verdict, m_playerIndex and relabelings
tried, under every work split; ill-formed items and refused batches fail as stated."""
import numpy as np
import pytest

import cases
import ise_gb300 as G
import oracle

pytestmark = pytest.mark.gpu

FIELDS = ["canonical", "status", "player_index", "trials", "aut"]


def expect(R, g):
    o = oracle.ksys_test(R, g=g)
    return dict(canonical=o["canonical"], player_index=o["player_index"],
                aut=o["n_aut"] if o["canonical"] else 0, trials=o["candidates"])


def got(r, i):
    return dict(canonical=bool(r["canonical"][i]), player_index=int(r["player_index"][i]),
                aut=int(r["aut"][i]), trials=int(r["trials"][i]))


def test_kirkman_systems_are_canonical_with_reference_aut(ctx):
    kts = cases.load_kts15()
    mats = np.stack([R for R, _ in kts])
    assert ctx.submit_ksys_groups(mats, 15, 7, 3) == 7
    r = ctx.sync()
    for i, (_, aut) in enumerate(kts):
        assert r["status"][i] == 0
        assert got(r, i) == dict(canonical=True, player_index=7 * 15 - 4, aut=aut, trials=120 * 6 ** 5 * 7 - 1)


def mixed_batch(seed):
    """(matrices padded to the batch's rounds, filled rounds, group size) per shape."""
    rng = np.random.default_rng(seed)
    kts = cases.load_kts15()
    out = {}
    mats, nrows = [], []
    for i, (R, _) in enumerate(kts):
        k = int(rng.integers(2, 8))
        for X in (R[:1 + i % 4], cases.ksys_relabel_random(R, rng, g=3),
                  cases.ksys_relabel_keep_round0(R[:k], rng, g=3), cases.ksys_relabel_random(R[:k], rng, g=3)):
            pad = np.zeros((7, 15), np.uint8)
            pad[:X.shape[0]] = X
            mats.append(pad)
            nrows.append(X.shape[0])
    # random partial systems of 15 players, until two of them lower m_playerIndex
    n15 = n_pi = 0
    while n15 < 40 or (n_pi < 2 and n15 < 800):
        X = cases.ksys_random_partial(15, 3, 3 + n15 % 2, rng)
        if X is None:
            continue
        n15 += 1
        lowers = oracle.ksys_test(X, g=3)["player_index"] != X.shape[0] * 15 - 4
        if n15 > 40 and not lowers:
            continue
        n_pi += lowers
        pad = np.zeros((7, 15), np.uint8)
        pad[:X.shape[0]] = X
        mats.append(pad)
        nrows.append(X.shape[0])
    bad = mats[1].copy()
    bad[1, [0, 1]] = bad[1, [1, 0]]       # players out of order inside a group: ill formed
    mats.append(bad)
    nrows.append(7)
    out[(15, 7, 3)] = (np.stack(mats), np.array(nrows, np.uint8))
    for np_, g, nr in [(9, 3, 4), (12, 3, 4), (16, 4, 3)]:
        mats, nrows = [], []
        for t in range(24):
            X = cases.ksys_random_partial(np_, g, 2 + t % (nr - 1), rng)
            if X is None:
                continue
            if t % 3 == 0:
                X = cases.ksys_relabel_keep_round0(X, rng, g=g)
            pad = np.zeros((nr, np_), np.uint8)
            pad[:X.shape[0]] = X
            mats.append(pad)
            nrows.append(X.shape[0])
        out[(np_, nr, g)] = (np.stack(mats), np.array(nrows, np.uint8))
    return out


def run(ctx, seg, shapes):
    ctx.set_ksys_segment(seg)
    for (np_, nr, g), (mats, nrows) in shapes.items():
        ctx.submit_ksys_groups(mats, np_, nr, g, 0, nrows)
    return ctx.sync()


def test_groups_of_3_and_4_equal_the_oracle_under_every_split(ctx):
    shapes = mixed_batch(3)
    try:
        first = run(ctx, 0, shapes)
        for seg in [G.KSYS_WHOLE, 32, 4096]:
            r = run(ctx, seg, shapes)
            for f in FIELDS:
                assert np.array_equal(np.asarray(r[f]), np.asarray(first[f])), (seg, f)
    finally:
        ctx.set_ksys_segment(0)
    i = 0
    n_pi = n_canon = 0
    for (np_, nr, g), (mats, nrows) in shapes.items():
        for X, k in zip(mats, nrows):
            if np_ == 15 and i == len(shapes[(15, 7, 3)][0]) - 1:
                assert first["status"][i] & G.ST_BADINPUT
                assert not first["canonical"][i]
            else:
                assert first["status"][i] == 0, i
                w = expect(X[:k], g)
                assert got(first, i) == w, (i, np_, g, k)
                n_pi += w["player_index"] != k * np_ - g - 1
                n_canon += w["canonical"]
            i += 1
    assert i == first["n"]
    assert n_canon >= 3 and n_pi >= 1


def test_refused_batches(ctx):
    kts = cases.load_kts15()
    R = kts[0][0][None]
    with pytest.raises(G.CanonError):
        ctx.submit_ksys_groups(R, 15, 7, 5)
    with pytest.raises(G.CanonError):
        ctx.submit_ksys_groups(np.zeros((1, 3, 14), np.uint8), 14, 3, 3)
    ctx.submit_ksys_groups(R, 15, 7, 3)
    k8, _ = oracle.ksys_enumerate(8)
    with pytest.raises(G.CanonError):
        ctx.submit_ksys(k8[0][0][None], 8, 7)
    r = ctx.sync()
    assert r["n"] == 1 and r["canonical"][0]
    # the queue takes group-size-2 batches again after the sync
    ctx.submit_ksys_groups(k8[0][0][None], 8, 7, 2)
    r = ctx.sync()
    assert r["n"] == 1 and r["canonical"][0]


def test_enumeration_gives_the_reference_kirkman_systems(ctx):
    """Orderly generation of k-systems with groups of 3 (canon_enumerate_ksys_groups: the
    next rounds of every canonical parent built on the host, checked on the GPU) gives
    the 7 Kirkman triple systems of 15 players of the reference's K_OrderedMatrices.txt,
    matrix for matrix, with its |Aut(M)|."""
    found, st = ctx.enumerate_ksys_groups(15, 3)
    kts = cases.load_kts15()
    assert sorted((R.tobytes(), a) for R, a in found) == sorted((R.tobytes(), a) for R, a in kts)
    assert st.designs == 7 and st.level_checks[6] == 8


def covers_every_pair_once(R, g):
    n = R.shape[1]
    seen = np.zeros((n, n), int)
    for row in R:
        for q in range(0, n, g):
            grp = row[q:q + g]
            for a in grp:
                for b in grp:
                    if a != b:
                        seen[a, b] += 1
    return bool((seen + np.eye(n, dtype=int) == 1).all())


def test_enumeration_of_the_affine_planes_of_order_3_and_4(ctx):
    """The resolvable designs with blocks of 3 on 9 points and of 4 on 16 are the affine
    planes AG(2,3) and AG(2,4), each with one resolution: one system each, with |Aut| the
    order of the affine semilinear group, 9 x 48 = 432 and 16 x 180 x 2 = 5760."""
    found, _ = ctx.enumerate_ksys_groups(9, 3)
    assert len(found) == 1 and found[0][1] == 432
    R = found[0][0]
    assert covers_every_pair_once(R, 3)
    o = oracle.ksys_test(R, g=3)
    assert o["canonical"] and o["n_aut"] == 432
    found, _ = ctx.enumerate_ksys_groups(16, 4)
    assert len(found) == 1 and found[0][1] == 5760
    assert covers_every_pair_once(found[0][0], 4)


def test_enumeration_routes_and_refusals(ctx):
    a, _ = ctx.enumerate_ksys_groups(8, 2)
    b, _ = ctx.enumerate_ksys(8)
    assert [(R.tobytes(), x) for R, x in a] == [(R.tobytes(), x) for R, x in b]
    for np_, g in [(12, 3), (12, 4), (18, 3), (15, 5)]:
        with pytest.raises(G.CanonError):
            ctx.enumerate_ksys_groups(np_, g)


def test_automorphisms_stored_as_the_oracle_stores_them(ctx):
    """CANON_SAVE_AUTS with groups of 3: the automorphisms of a canonical matrix are the
    oracle's CGroupInfo set (sorted relabelings, identity first); beyond aut_cap the item
    reports CANON_ST_PERM_OVF with aut_cap of them stored; a rejected matrix stores none."""
    kts = cases.load_kts15()
    big = G.Context(max_items=1024, aut_cap=200)
    try:
        picks = [next(R for R, a in kts if a == 12), next(R for R, a in kts if a == 168), kts[0][0][:2],
                 kts[3][0][:3]]
        rng = np.random.default_rng(5)
        rejected = cases.ksys_relabel_random(kts[2][0], rng, g=3)
        for X in picks + [rejected]:
            big.submit_ksys_groups(X[None], 15, X.shape[0], 3, G.SAVE_AUTS)
            r = big.sync()
            o = oracle.ksys_test(X, g=3, aut_cap=256)
            assert bool(r["canonical"][0]) == o["canonical"]
            if not o["canonical"]:
                assert r["n_auts"][0] == 0 and r["aut"][0] == 0
                continue
            n = o["n_aut"]
            assert r["aut"][0] == n and r["status"][0] == (G.ST_PERM_OVF if n > 200 else 0)
            if n <= 200:
                assert r["n_auts"][0] == n
                got = r["auts_raw"][0][:n, :15]
                assert np.array_equal(got, o["auts"]), X.shape
    finally:
        big.close()
