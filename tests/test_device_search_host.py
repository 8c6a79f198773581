"""The BIBD kernel's search (canon_bibd_core.cuh) compiled for the host and checked
against the oracle: catches logic errors of the device code on the CPU."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import cases
import conftest
import oracle

SRC = os.path.join(conftest.REPO, "tests", "host_build", "canon_bibd_host.cpp")
OUT = os.path.join(conftest.REPO, "tests", "host_build", "_build", "libcanon_bibd_host.so")
CUDA_INC = "/usr/local/cuda/include"

COMPLETE, RAW, FULL_AUT, AUT_CANON = 0x1, 0x2, 0x4, 0x10


@pytest.fixture(scope="module")
def host():
    if not os.path.isdir(CUDA_INC):
        pytest.skip("CUDA headers not found")
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I", CUDA_INC, SRC, "-o", OUT],
                   check=True)
    return ctypes.CDLL(OUT)


def run(L, rows, n, b, flags):
    rows = np.ascontiguousarray(rows, np.uint64)
    u8, u64 = ctypes.c_uint8, ctypes.c_uint64
    can, st, rr, w, tr = u8(), u8(), u8(), u64(), u64()
    aut = (u64 * 2)()
    L.emu_check(rows.ctypes.data_as(ctypes.POINTER(u64)), n, b, flags, u64(1 << 24), ctypes.byref(can),
                ctypes.byref(st), ctypes.byref(rr), ctypes.byref(w), aut, ctypes.byref(tr))
    return dict(canonical=bool(can.value), status=st.value, reject_row=rr.value,
                witness=bytes((w.value >> (4 * i)) & 15 for i in range(n)),
                aut=aut[0] | (aut[1] << 64), trials=tr.value)


def expected(M, flags):
    X = oracle.bibd_normalize(M) if flags & RAW else M
    f = (oracle.SAVE_ROW_PERM | oracle.SAVE_ROW_TO_CHANGE) if flags & COMPLETE else 0
    o = oracle.bibd_test(X, f | (oracle.FULL_AUT if flags & FULL_AUT else 0))
    if flags & AUT_CANON and not o["canonical"]:
        _, o["aut"], _ = oracle.bibd_canonize(X)
    return o


def compare(L, M, flags):
    n, b = M.shape
    import ise_gb300 as G
    e = run(L, G.pack_rows(M), n, b, flags)
    o = expected(M, flags)
    assert e["status"] == 0
    assert e["canonical"] == o["canonical"]
    assert e["trials"] == o["trials"]
    if not o["canonical"]:
        assert e["witness"] == o["witness"] and e["reject_row"] == o["reject_row"]
    if o["canonical"] or flags & (FULL_AUT | AUT_CANON):
        assert e["aut"] == o["aut"]


@pytest.mark.parametrize("flags", [COMPLETE | RAW, COMPLETE | RAW | FULL_AUT, COMPLETE | RAW | AUT_CANON])
def test_sts15_random(host, flags):
    for i in range(12 if flags & FULL_AUT else 30):
        compare(host, oracle.rows_to_matrix(oracle.sts_random_rows(15, 808, i), 35), flags)


def test_partial_prefixes(host):
    rng = np.random.default_rng(21)
    sts = cases.load_sts15()
    for M, _ in sts[::7]:
        P = cases.permute_normalize(M, rng)
        for k in (3, 6, 9, 12):
            compare(host, oracle.bibd_normalize(P[:k]), 0)
            compare(host, oracle.bibd_normalize(P[:k]), FULL_AUT)
    for params in [(8, 14, 7, 4, 3), (11, 11, 5, 5, 2), (7, 14, 6, 3, 2)]:
        for M, _ in cases.bibd_designs(*params):
            for _ in range(3):
                P = cases.permute_normalize(M, rng)
                for k in range(2, P.shape[0] + 1):
                    compare(host, oracle.bibd_normalize(P[:k]), COMPLETE if k == P.shape[0] else 0)
