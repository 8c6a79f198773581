"""The relabeling step of the GPU check of k-systems with groups of 3 or 4
(incidence-system-enumeration_gb300/csrc/canon_kgen.cuh), compiled for the host and run
over every relabeling in the reference's order, against the oracle's cnvCheckNew()
restatement (k-Factorization/TripleSys/Source/cnv.cpp:211-351, kmSupport.cpp:220-356):
the 7 Kirkman triple systems of 15 players, their prefixes, relabelled copies, random
partial systems with groups of 3 and 4 (some of them lowering m_playerIndex)."""
import concurrent.futures as cf
import ctypes
import os
import subprocess

import numpy as np
import pytest

import cases
import conftest
import oracle

SRC = os.path.join(conftest.REPO, "tests", "host_build", "canon_kgen_host.cpp")
OUT = os.path.join(conftest.REPO, "tests", "host_build", "_build", "libcanon_kgen_host.so")


@pytest.fixture(scope="module")
def emu():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", SRC, "-o", OUT], check=True)
    L = ctypes.CDLL(OUT)
    L.emu_kgen_check.restype = ctypes.c_int

    def run(R, g):
        R = np.ascontiguousarray(R, np.uint8)
        nr, n = R.shape
        c, p = ctypes.c_int(), ctypes.c_int()
        a, k = ctypes.c_uint64(), ctypes.c_uint64()
        rc = L.emu_kgen_check(R.ctypes.data_as(ctypes.c_void_p), nr, n, g, ctypes.byref(c), ctypes.byref(p),
                              ctypes.byref(a), ctypes.byref(k))
        assert rc == 0
        return dict(canonical=bool(c.value), player_index=p.value, n_aut=a.value, candidates=k.value)
    return run


def expect(R, g):
    o = oracle.ksys_test(R, g=g)
    # |Aut| is reported for canonical matrices only (the search stops at a rejection)
    return dict(canonical=o["canonical"], player_index=o["player_index"],
                n_aut=o["n_aut"] if o["canonical"] else 0, candidates=o["candidates"])


def test_kirkman_systems_are_canonical_with_reference_aut(emu):
    kts = cases.load_kts15()
    with cf.ThreadPoolExecutor(max(1, min(7, os.cpu_count() or 1))) as ex:
        outs = list(ex.map(lambda R: emu(R, 3), [R for R, _ in kts]))
    for (R, aut), o in zip(kts, outs):
        assert o == dict(canonical=True, player_index=7 * 15 - 3 - 1, n_aut=aut,
                         candidates=120 * 6 ** 5 * 7 - 1)


def test_kirkman_prefixes_and_relabelled_copies(emu):
    kts = cases.load_kts15()
    rng = np.random.default_rng(2024)
    jobs = []
    for R, _ in kts[::3]:
        for k in (1, 2, 4, 6):
            jobs.append(R[:k])
    for R, _ in kts:
        jobs.append(cases.ksys_relabel_random(R, rng, g=3))
        for k in (2, 3, 5, 7):
            jobs.append(cases.ksys_relabel_keep_round0(R[:k], rng, g=3))
            jobs.append(cases.ksys_relabel_random(R[:k], rng, g=3))
    with cf.ThreadPoolExecutor(max(1, min(8, os.cpu_count() or 1))) as ex:
        got = list(ex.map(lambda X: emu(X, 3), jobs))
        want = list(ex.map(lambda X: expect(X, 3), jobs))
    assert got == want
    assert any(w["canonical"] for w in want) and any(not w["canonical"] for w in want)


@pytest.mark.parametrize("np_,g,nrs", [(9, 3, (2, 3, 4)), (12, 3, (2, 3, 4)), (15, 3, (3, 4)), (16, 4, (2, 3))])
def test_random_partial_systems(emu, np_, g, nrs):
    rng = np.random.default_rng(np_ * 10 + g)
    n_pi = 0
    for t in range(400 if np_ == 15 else 60):
        X = cases.ksys_random_partial(np_, g, nrs[t % len(nrs)], rng)
        if X is None:
            continue
        w = expect(X, g)
        assert emu(X, g) == w, X
        n_pi += w["player_index"] != X.shape[0] * np_ - g - 1
        if np_ == 15 and t >= 60 and n_pi:
            break
    if np_ == 15:
        # setPlayerIndex() lowers m_playerIndex on some of them
        assert n_pi >= 1


@pytest.mark.parametrize("np_,g", [(6, 3), (8, 4), (12, 4), (16, 4)])
def test_single_round_every_relabeling_is_an_automorphism(emu, np_, g):
    R = np.arange(np_, dtype=np.uint8)[None, :]
    o = emu(R, g)
    ng = np_ // g
    total = int(np.prod(np.arange(1, ng + 1))) * int(np.prod(np.arange(1, g + 1))) ** ng
    assert o == dict(canonical=True, player_index=np_ - g - 1, n_aut=total, candidates=total - 1)
    if np_ <= 12:
        assert expect(R, g) == o
