"""The host side of the enumeration of k-systems with groups of 3 or 4
(incidence-system-enumeration_gb300/csrc/canon_kenum_rounds.h), compiled for the host:
the next rounds of a parent against a plain Python enumeration of the partitions into
groups that repeat no pair (result() form, ordered by second entry), in the same order,
and the links test (checkLinksV, k-Factorization/TripleSys/Source/checkLinksV.cpp) against
a Python restatement of its condition and against completability of small systems."""
import ctypes
import itertools
import os
import subprocess

import numpy as np
import pytest

import cases
import conftest

SRC = os.path.join(conftest.REPO, "tests", "host_build", "canon_kenum_host.cpp")
OUT = os.path.join(conftest.REPO, "tests", "host_build", "_build", "libcanon_kenum_host.so")


@pytest.fixture(scope="module")
def lib():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", SRC, "-o", OUT], check=True)
    L = ctypes.CDLL(OUT)
    L.emu_kenum_children.restype = ctypes.c_uint64
    L.emu_kenum_children.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_uint64]
    L.emu_kenum_links.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    return L


def children(L, P, g, links):
    P = np.ascontiguousarray(P, np.uint8)
    d, n = P.shape
    cnt = L.emu_kenum_children(P.ctypes.data, d, n, g, int(links), None, 0)
    out = np.zeros((cnt, d + 1, n), np.uint8)
    L.emu_kenum_children(P.ctypes.data, d, n, g, int(links), out.ctypes.data, cnt)
    return out


def used_pairs(P, g):
    s = set()
    for row in P:
        for q in range(0, len(row), g):
            for a, b in itertools.combinations(row[q:q + g], 2):
                s.add((int(a), int(b)))
                s.add((int(b), int(a)))
    return s


def py_rounds(P, g):
    """Every next round in result() form with second entry above the parent's last,
    in increasing order of the round's bytes (the builder's order)."""
    n = P.shape[1]
    used = used_pairs(P, g)
    prev2 = int(P[-1][1])
    out = []

    def rec(avail, cur):
        if not avail:
            out.append(list(cur))
            return
        a = min(avail)
        rest = sorted(avail - {a})
        for grp in itertools.combinations(rest, g - 1):
            if a == 0 and grp[0] <= prev2:
                continue
            members = (a,) + grp
            if any((x, y) in used for x, y in itertools.combinations(members, 2)):
                continue
            rec(avail - set(members), cur + list(members))

    rec(set(range(n)), [])
    return out


def py_links(P, g):
    n = P.shape[1]
    used = used_pairs(P, g)
    free = {x: {y for y in range(n) if y != x and (x, y) not in used} for x in range(n)}

    def split(s):
        if not s:
            return True
        v = min(s)
        rest = s - {v}
        for grp in itertools.combinations(sorted(rest & free[v]), g - 2):
            if all(b in free[a] for a, b in itertools.combinations(grp, 2)):
                if split(rest - set(grp)):
                    return True
        return False

    return all(split(free[x]) for x in range(n) if free[x])


@pytest.mark.parametrize("np_,g", [(9, 3), (15, 3), (16, 4), (12, 3)])
def test_first_level_equals_the_python_enumeration(lib, np_, g):
    P = np.arange(np_, dtype=np.uint8)[None, :]
    got = children(lib, P, g, False)
    want = py_rounds(P, g)
    assert [list(c[-1]) for c in got] == want
    assert (got[:, 0] == P[0]).all()
    if (np_, g) == (15, 3):
        assert len(want) == 132192


def test_deeper_levels_and_the_links_test(lib):
    rng = np.random.default_rng(9)
    kts = cases.load_kts15()
    seen = 0
    for R, _ in kts[::2]:
        for d in (2, 3, 4, 5):
            P = R[:d]
            got = children(lib, P, 3, False)
            want = py_rounds(P, 3)
            assert [list(c[-1]) for c in got] == want, d
            # the links test keeps exactly the children whose unmet pairs still split
            kept = children(lib, P, 3, True)
            flags = [py_links(c, 3) for c in got]
            assert [list(c[-1]) for c in kept] == [list(c[-1]) for c, f in zip(got, flags) if f], d
            # the next round of the Kirkman system itself always passes
            assert any(np.array_equal(c[-1], R[d]) for c in kept)
            seen += len(got)
        for _ in range(20):
            k = int(rng.integers(1, 7))
            X = cases.ksys_relabel_random(R[:k], rng, g=3)
            assert lib.emu_kenum_links(np.ascontiguousarray(X).ctypes.data, k, 15, 3) == int(py_links(X, 3))
    assert seen > 0


def test_links_test_against_completability(lib):
    """On 9 players in groups of 3 a partial system passes the links test whenever some
    completion exists (a necessary condition), checked by brute-force completion."""
    rng = np.random.default_rng(3)
    checked = 0
    for t in range(40):
        X = cases.ksys_random_partial(9, 3, 2 + t % 2, rng)
        if X is None:
            continue
        completable = False
        stack = [X]
        while stack and not completable:
            P = stack.pop()
            if P.shape[0] == 4:
                completable = True
                break
            for r in py_rounds(P, 3) if P.shape[0] > 0 else []:
                stack.append(np.vstack([P, np.array(r, np.uint8)[None, :]]))
        ok = lib.emu_kenum_links(np.ascontiguousarray(X).ctypes.data, X.shape[0], 9, 3)
        if completable:
            assert ok == 1
        checked += 1
    assert checked > 0


def test_orderly_enumeration_of_nine_players_in_triples(lib):
    """The whole orderly generation with groups of 3 on 9 players, on the CPU: the host
    round builder with its links test, the oracle's cnvCheckNew() as the check.  One
    system results, AG(2,3) with its 4 parallel classes, |Aut| = 9 x 48 = 432 -- the result
    the GPU enumeration gives (tests/test_gpu_kgen.py)."""
    import oracle
    level = [np.arange(9, dtype=np.uint8)[None, :]]
    found = []
    for d in range(1, 4):
        nxt = []
        for P in level:
            for C in children(lib, P, 3, 2 * (4 - (d + 1)) <= 3):
                o = oracle.ksys_test(C, g=3)
                if not o["canonical"]:
                    continue
                if d + 1 == 4:
                    found.append((C, o["n_aut"]))
                else:
                    nxt.append(C)
        level = nxt
    assert len(found) == 1 and found[0][1] == 432
    R = found[0][0]
    pairs = used_pairs(R, 3)
    assert len(pairs) == 9 * 8      # every pair of players meets exactly once


def test_orderly_enumeration_of_sixteen_players_in_fours(lib):
    """The same on 16 players in groups of 4 (about 50 s on 8 host threads): one system,
    the resolution of AG(2,4), with |Aut| = 16 x 180 x 2 = 5760 (the affine semilinear
    group) -- a known answer that pins the oracle's check with groups of 4, and the result
    of the GPU enumeration."""
    import concurrent.futures as cf
    import oracle
    level = [np.arange(16, dtype=np.uint8)[None, :]]
    found = []
    with cf.ThreadPoolExecutor(max(1, min(8, os.cpu_count() or 1))) as ex:
        for d in range(1, 5):
            cands = [C for P in level for C in children(lib, P, 4, 2 * (5 - (d + 1)) <= 4)]
            res = list(ex.map(lambda C: oracle.ksys_test(C, g=4), cands))
            nxt = []
            for C, o in zip(cands, res):
                if o["canonical"]:
                    (found.append((C, o["n_aut"])) if d + 1 == 5 else nxt.append(C))
            level = nxt
    assert len(found) == 1 and found[0][1] == 5760
    assert len(used_pairs(found[0][0], 4)) == 16 * 15
