"""The canonical binary matrix of a k-system (runCanonizer(), Source/CDTools.cpp:5-52):
the device search (canon_kbin_core.cuh) compiled for the host against the oracle's
restatement of the reference path (convertToBinaryMatrix + CanonizeMatrix with the day
classes), on every 1-factorization of K6 and K8 (all days: the days may be permuted)
and on prefixes of K10 1-factorizations (fewer days: the day order is fixed), each
also under random relabelings, which must not change the result."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import cases
import conftest
import oracle

SRC = os.path.join(conftest.REPO, "tests", "host_build", "canon_kbin_host.cpp")
OUT = os.path.join(conftest.REPO, "tests", "host_build", "_build", "libcanon_kbin_host.so")


@pytest.fixture(scope="module")
def kb():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", SRC, "-o", OUT], check=True)
    L = ctypes.CDLL(OUT)
    u64p = ctypes.POINTER(ctypes.c_uint64)
    L.emu_kbin.argtypes = [u64p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, u64p,
                           u64p, u64p]
    return L


def binary_rows(R, np_, days):
    """convertToBinaryMatrix: player p, column d*g + j = group j of day d"""
    g = np_ // 2
    rows = np.zeros(np_, np.uint64)
    for d in range(days):
        for j in range(g):
            for p in R[d][2 * j: 2 * j + 2]:
                rows[p] |= np.uint64(1) << np.uint64(d * g + j)
    return rows


def run(L, R, np_, days, free):
    g = np_ // 2
    rows = binary_rows(R, np_, days)
    out = np.zeros(np_, np.uint64)
    leaves, nodes = ctypes.c_uint64(), ctypes.c_uint64()
    u64p = ctypes.POINTER(ctypes.c_uint64)
    assert L.emu_kbin(rows.ctypes.data_as(u64p), np_, days * g, g, days, int(free), out.ctypes.data_as(u64p),
                      ctypes.byref(leaves), ctypes.byref(nodes)) == 0
    b = days * g
    return ((out[:, None] >> np.arange(b, dtype=np.uint64)) & np.uint64(1)).astype(np.uint8), leaves.value


def relabel(R, rng, np_, shuffle_days):
    p = rng.permutation(np_)
    rounds = []
    for row in R:
        pairs = sorted(tuple(sorted((int(p[row[i]]), int(p[row[i + 1]])))) for i in range(0, np_, 2))
        rounds.append([x for pr in pairs for x in pr])
    order = rng.permutation(len(rounds)) if shuffle_days else np.arange(len(rounds))
    return np.array([rounds[i] for i in order], np.uint8)


@pytest.mark.parametrize("np_", [6, 8])
def test_all_days_match_the_oracle(kb, np_):
    rng = np.random.default_rng(np_)
    found, _ = oracle.ksys_enumerate(np_)
    for R, aut in found:
        ref, _ = oracle.ksys_binary_canonize(R, np_)
        got, leaves = run(kb, R, np_, np_ - 1, True)
        assert np.array_equal(got, ref)
        assert leaves == aut           # the labelings that reach the form: |Aut| of the factorization
        X = relabel(R, rng, np_, True)
        got2, _ = run(kb, X, np_, np_ - 1, True)
        assert np.array_equal(got2, ref)


def test_k10_prefixes_match_the_oracle(kb):
    rng = np.random.default_rng(10)
    k10 = cases.load_k10()
    for R, _ in k10[::20]:
        for d in (2, 3, 5, 8):
            ref, _ = oracle.ksys_binary_canonize(R[:d], 10, 2, d)
            got, _ = run(kb, R[:d], 10, d, False)
            assert np.array_equal(got, ref), d
            # relabelled players (the day order stays: it is fixed by the colours)
            X = relabel(R[:d], rng, 10, False)
            assert np.array_equal(oracle.ksys_binary_canonize(X, 10, 2, d)[0], ref)
            assert np.array_equal(run(kb, X, 10, d, False)[0], ref)


def binary_rows_k(R, np_, days, k):
    """convertToBinaryMatrix with groups of k: column d*g + j = group j of day d"""
    g = np_ // k
    rows = np.zeros(np_, np.uint64)
    for d in range(days):
        for j in range(g):
            for p in R[d][k * j: k * j + k]:
                rows[p] |= np.uint64(1) << np.uint64(d * g + j)
    return rows


def run_k(L, R, np_, days, free, k):
    g = np_ // k
    rows = binary_rows_k(R, np_, days, k)
    out = np.zeros(np_, np.uint64)
    leaves, nodes = ctypes.c_uint64(), ctypes.c_uint64()
    u64p = ctypes.POINTER(ctypes.c_uint64)
    assert L.emu_kbin(rows.ctypes.data_as(u64p), np_, days * g, g, days, int(free), out.ctypes.data_as(u64p),
                      ctypes.byref(leaves), ctypes.byref(nodes)) == 0
    b = days * g
    return ((out[:, None] >> np.arange(b, dtype=np.uint64)) & np.uint64(1)).astype(np.uint8), leaves.value


def test_kirkman_systems_match_the_oracle_with_groups_of_3(kb):
    """The same search on the 7 Kirkman triple systems of 15 players (groups of 3, 5
    columns a day): every prefix of 2..6 days (day order fixed) and the complete systems
    (days permuted), against the oracle's restatement; the labelings reaching the form
    of a complete system are its |Aut(M)|, and relabelled copies reach the same form."""
    rng = np.random.default_rng(3)
    for R, aut in cases.load_kts15():
        for d in (2, 4, 6):
            ref, _ = oracle.ksys_binary_canonize(R[:d], 15, 3, d)
            assert np.array_equal(run_k(kb, R[:d], 15, d, False, 3)[0], ref), d
        ref, _ = oracle.ksys_binary_canonize(R, 15, 3)
        got, leaves = run_k(kb, R, 15, 7, True, 3)
        assert np.array_equal(got, ref) and leaves == aut
        X = cases.ksys_relabel_random(R, rng, g=3)
        assert np.array_equal(run_k(kb, X, 15, 7, True, 3)[0], ref)
