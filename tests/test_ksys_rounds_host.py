"""The device round generator of the k-system enumerator (canon_ksys_rounds.cuh),
compiled for the host: every admissible next round of a partial 1-factorization,
in the order the enumerator writes them, and -- with the oracle as the checker --
a level-by-level enumeration of K8 that gives the oracle's depth-first result (the
device enumerator runs this generator level by level; its K10 run is compared with
the reference's 396 matrices in the GPU suite)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import cases
import conftest
import oracle

SRC = os.path.join(conftest.REPO, "tests", "host_build", "canon_ksys_rounds_host.cpp")
OUT = os.path.join(conftest.REPO, "tests", "host_build", "_build", "libcanon_ksys_rounds_host.so")


@pytest.fixture(scope="module")
def gen():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", SRC, "-o", OUT], check=True)
    L = ctypes.CDLL(OUT)
    L.emu_ksys_children.restype = ctypes.c_uint32
    L.emu_ksys_children.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    return L


def children(L, np_, parent):
    d = parent.shape[0]
    p = np.ascontiguousarray(parent, np.uint8)
    cnt = L.emu_ksys_children(np_, p.ctypes.data, d, None)
    out = np.zeros((cnt, d + 1, np_), np.uint8)
    assert L.emu_ksys_children(np_, p.ctypes.data, d, out.ctypes.data) == cnt
    return out


def brute_rounds(np_, parent):
    """Every perfect matching with unused pairs and player 0 meeting d+1, as sorted rounds."""
    d = parent.shape[0]
    used = {tuple(sorted((int(r[i]), int(r[i + 1])))) for r in parent for i in range(0, np_, 2)}
    found = []

    def rec(rest, pairs):
        if not rest:
            found.append([x for pr in sorted(pairs) for x in pr])
            return
        a = rest[0]
        for c in rest[1:]:
            if (a, c) in used or (a == 0 and c != d + 1):
                continue
            rec([x for x in rest if x not in (a, c)], pairs + [(a, c)])

    rec(list(range(np_)), [])
    return sorted(found)


def test_next_rounds_are_every_admissible_matching(gen):
    rng = np.random.default_rng(5)
    for np_ in (6, 8, 10, 12):
        parent = np.arange(np_, dtype=np.uint8)[None, :]
        for _ in range(np_ - 2):
            kids = children(gen, np_, parent)
            got = sorted(k[-1].tolist() for k in kids)
            assert got == brute_rounds(np_, parent)
            # the parent is copied in front of every child, in the walk's order
            assert all(np.array_equal(k[:-1], parent) for k in kids)
            assert [k[-1].tolist() for k in kids] == sorted(k[-1].tolist() for k in kids)
            if not len(kids):
                break
            parent = kids[int(rng.integers(len(kids)))]


def test_level_by_level_enumeration_matches_the_oracle_on_k8(gen):
    level = [np.arange(8, dtype=np.uint8)[None, :]]
    for _ in range(6):
        nxt = []
        for P in level:
            for K in children(gen, 8, P):
                if oracle.ksys_test(K)["canonical"]:
                    nxt.append(K)
        level = nxt
    ref, _ = oracle.ksys_enumerate(8)
    assert len(level) == len(ref) == 6
    assert sorted(M.tobytes() for M in level) == sorted(np.asarray(M, np.uint8).tobytes() for M, _ in ref)


def test_children_split_by_the_second_pair_concatenate_to_the_whole(gen):
    """The device walks a parent in parts, one per partner of the second pair; taken in
    increasing partner order the parts are the parent's children in their order."""
    gen.emu_ksys_children_part.restype = ctypes.c_uint32
    gen.emu_ksys_children_part.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_int]
    for np_ in (6, 8, 10):
        found, _ = oracle.ksys_enumerate(np_) if np_ < 10 else (cases.load_k10(), None)
        mats = [R for R, _ in found]
        for R in mats[:: max(1, len(mats) // 12)]:
            for d in range(1, np_ - 1):
                parent = np.ascontiguousarray(R[:d], np.uint8)
                whole = children(gen, np_, parent)
                parts = []
                for s in range(np_):
                    cnt = gen.emu_ksys_children_part(np_, parent.ctypes.data, d, None, s)
                    out = np.zeros((cnt, d + 1, np_), np.uint8)
                    assert gen.emu_ksys_children_part(np_, parent.ctypes.data, d, out.ctypes.data, s) == cnt
                    parts.append(out)
                joined = np.concatenate(parts) if parts else whole[:0]
                assert np.array_equal(joined, whole), (np_, d)
