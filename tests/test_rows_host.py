"""The device enumerator's row generator (canon_rows.cuh), compiled for the host and
driven level by level with the oracle as the checker: it must give the oracle's
depth-first enumeration (designs and |Aut|) and the reference's result tables."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import cases
import conftest
import oracle

SRC = os.path.join(conftest.REPO, "tests", "host_build", "canon_rows_host.cpp")
OUT = os.path.join(conftest.REPO, "tests", "host_build", "_build", "libcanon_rows_host.so")
FAMILIES = ["7,7,3,3,1", "7,14,6,3,2", "6,30,15,3,6", "8,14,7,4,3", "9,12,4,3,1", "9,18,8,4,3",
            "10,15,6,4,2", "11,11,5,5,2", "13,13,4,4,1", "13,26,6,3,1", "16,20,5,4,1"]


@pytest.fixture(scope="module")
def gen():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", SRC, "-o", OUT], check=True)
    L = ctypes.CDLL(OUT)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    L.rows_children.argtypes = [ctypes.c_int] * 5 + [u64p, ctypes.c_int, u64p, ctypes.c_uint32]
    L.rows_children.restype = ctypes.c_uint32
    return L


def children(L, params, parent):
    n = len(parent)
    p = np.ascontiguousarray(parent, np.uint64)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    cnt = L.rows_children(*params, p.ctypes.data_as(u64p), n, None, 0)
    out = np.zeros(max(cnt, 1) * (n + 1), np.uint64)
    assert L.rows_children(*params, p.ctypes.data_as(u64p), n, out.ctypes.data_as(u64p), cnt) == cnt
    return out[: cnt * (n + 1)].reshape(cnt, n + 1)


def unpack(words, b):
    return ((np.asarray(words, np.uint64)[:, None] >> np.arange(b, dtype=np.uint64)) & 1).astype(np.uint8)


@pytest.mark.parametrize("key", FAMILIES)
def test_level_enumeration_equals_oracle(gen, key):
    params = tuple(map(int, key.split(",")))
    v, b, r = params[:3]
    level = [np.array([(1 << r) - 1], np.uint64)]
    for m in range(2, v + 1):
        nxt = []
        for parent in level:
            for child in children(gen, params, parent):
                M = unpack(child, b)
                flags = (oracle.SAVE_ROW_PERM | oracle.SAVE_ROW_TO_CHANGE) if m == v else 0
                o = oracle.bibd_test(M, flags)
                if o["canonical"]:
                    nxt.append((child, o["aut"]))
        level = [c for c, _ in nxt]
    got = {unpack(c, b).tobytes(): a for c, a in nxt}
    ref, _ = oracle.bibd_enumerate(*params)
    assert got == {M.tobytes(): a for M, a in ref}
    tab = cases.load_result_tables()[key]
    designs = [(unpack(c, b), a) for c, a in nxt]
    assert cases.table_rows(designs, [cases.simple_design(M) for M, _ in designs],
                            [cases.oracle_transitive(M) for M, _ in designs]) == tab["rows"]


def test_children_are_normal_and_non_increasing(gen):
    """Every child is in orbit normal form and its new row is not greater than the
    row above it (read column 0 first)."""
    params = (15, 35, 7, 3, 1)
    rng = np.random.default_rng(3)
    sts = cases.load_sts15()
    for M, _ in sts[::9]:
        P = cases.permute_normalize(M, rng)
        for k in (3, 6, 9):
            parent = np.array([int("".join(str(x) for x in row[::-1]), 2) for row in P[:k]], np.uint64)
            for child in children(gen, params, parent):
                C = unpack(child, 35)
                assert oracle.bibd_is_normal(C)
                assert tuple(C[-1]) <= tuple(C[-2])


def children_aut(L, params, parent, gens):
    n = len(parent)
    p = np.ascontiguousarray(parent, np.uint64)
    g = np.ascontiguousarray(gens, np.uint64)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    f = L.rows_children_aut
    f.argtypes = [ctypes.c_int] * 5 + [u64p, ctypes.c_int, u64p, ctypes.c_uint32, u64p, ctypes.c_int]
    f.restype = ctypes.c_uint32
    gp = g.ctypes.data_as(u64p) if len(g) else None
    cnt = f(*params, p.ctypes.data_as(u64p), n, None, 0, gp, len(g))
    out = np.zeros(max(cnt, 1) * (n + 1), np.uint64)
    assert f(*params, p.ctypes.data_as(u64p), n, out.ctypes.data_as(u64p), cnt, gp, len(g)) == cnt
    return out[: cnt * (n + 1)].reshape(cnt, n + 1)


def row_automorphisms(M):
    """The row automorphisms that the oracle's TestCanonicity finds (t_outRowPermute),
    nibble-packed: nibble i = the row that goes to position i."""
    o = oracle.bibd_test(M, oracle.SAVE_ROW_PERM | oracle.SAVE_AUT_ROWS, perm_cap=64)
    perms = o["perms"][1:] if len(o["perms"]) else []
    return [sum(int(x) << (4 * i) for i, x in enumerate(p)) for p in perms]


@pytest.mark.parametrize("key", ["7,14,6,3,2", "8,14,7,4,3", "9,12,4,3,1", "10,15,6,4,2", "13,26,6,3,1",
                                 "16,20,5,4,1"])
def test_automorphism_pruning_keeps_the_designs_and_drops_candidates(gen, key):
    """Children that an automorphism of their parent maps to a greater child are not
    generated: the same designs, with fewer candidates to check."""
    params = tuple(map(int, key.split(",")))
    v, b, r = params[:3]
    level = [np.array([(1 << r) - 1], np.uint64)]
    cand_plain = cand_aut = 0
    for m in range(2, v + 1):
        nxt = []
        for parent in level:
            gens = row_automorphisms(unpack(parent, b)) if len(parent) > 1 else []
            cand_plain += len(children(gen, params, parent))
            kids = children_aut(gen, params, parent, gens)
            cand_aut += len(kids)
            for child in kids:
                M = unpack(child, b)
                flags = (oracle.SAVE_ROW_PERM | oracle.SAVE_ROW_TO_CHANGE) if m == v else 0
                o = oracle.bibd_test(M, flags)
                if o["canonical"]:
                    nxt.append((child, o["aut"]))
        level = [c for c, _ in nxt]
    got = {unpack(c, b).tobytes(): a for c, a in nxt}
    ref, _ = oracle.bibd_enumerate(*params)
    assert got == {M.tobytes(): a for M, a in ref}
    assert cand_aut <= cand_plain
    print(key, cand_plain, cand_aut)


def _orbits(parent, n, b):
    """The parent's column orbits: (start, len, rows with 1s as a bit set, split row)."""
    cols = [sum(((int(parent[i]) >> c) & 1) << i for i in range(n)) for c in range(b)]
    orbs, s = [], 0
    for c in range(1, b + 1):
        if c == b or cols[c] != cols[c - 1]:
            split = 0
            if orbs:
                while split < n and ((cols[s] >> split) & 1) == ((cols[s - 1] >> split) & 1):
                    split += 1
            orbs.append((s, c - s, cols[s], split))
            s = c
    return orbs


def _brute_children(params, parent):
    """Every admissible next row by brute force over the 1s per orbit, with the
    generator's rules written out: weight r, lambda with every row, no column above k,
    columns that need every remaining row, not above row n-1, and the swap test."""
    import itertools
    v, b, r, k, lam = params
    n = len(parent)
    orbs = _orbits(parent, n, b)
    rem = v - n - 1
    rngs = []
    for _, ln, om, _ in orbs:
        w = bin(om).count("1")
        hi = 0 if w >= k else ln
        lo = ln if k - w > rem else 0
        rngs.append(range(lo, hi + 1))
    prev = [ln if (om >> (n - 1)) & 1 else 0 for _, ln, om, _ in orbs]
    out = []
    for x in itertools.product(*[list(rg)[::-1] for rg in rngs]):
        if sum(x) != r:
            continue
        if any(sum(x[t] for t, o in enumerate(orbs) if (o[2] >> i) & 1) != lam for i in range(n)):
            continue
        if list(x) > prev:
            continue
        ok = True
        for i in range(1, n):
            c = ri = 0
            for t in range(len(orbs) + 1):
                if t == len(orbs) or (t > 0 and orbs[t][3] < i):
                    if c > ri:
                        ok = False
                    if c != ri or t == len(orbs):
                        break
                    c = ri = 0
                c += x[t]
                ri += orbs[t][1] if (orbs[t][2] >> i) & 1 else 0
            if not ok:
                break
        if ok:
            row = 0
            for t, (st, _, _, _) in enumerate(orbs):
                row |= ((1 << x[t]) - 1) << st
            out.append(row)
    return out


@pytest.mark.parametrize("key,levels", [("8,14,7,4,3", 6), ("10,15,6,4,2", 6), ("13,26,8,4,2", 4),
                                        ("12,22,11,6,5", 4)])
def test_children_equal_the_rules_by_brute_force(gen, key, levels):
    """The generator's depth-first search with its bounds (per-row lambda windows, the
    1s that must fit outside every row's orbits, the swap test run orbit by orbit) gives
    exactly the rows that the rules admit, in the same order (orbits left to right,
    more 1s first)."""
    params = tuple(map(int, key.split(",")))
    v, b, r = params[:3]
    level = [np.array([(1 << r) - 1], np.uint64)]
    for m in range(2, levels + 1):
        nxt = []
        for parent in level[:60]:
            kids = children(gen, params, parent)
            assert [int(c[-1]) for c in kids] == _brute_children(params, parent), (key, m)
            nxt.extend(kids)
        level = nxt
