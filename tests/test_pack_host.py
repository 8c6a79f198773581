"""The packing of a queued batch's work descriptors (canon_submit_bibd / canon_submit_ksys,
incidence-system-enumeration_gb300/csrc/canon_pack.h), compiled for the host: descriptors in
a stable order of filled rows (so a warp's matrices run the same loops; outputs keep the
submission order through each descriptor's output index), every matrix copied once, and a
batch with a row count outside [1, maxr] refused."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import conftest

SRC = os.path.join(conftest.REPO, "tests", "host_build", "canon_pack_host.cpp")
OUT = os.path.join(conftest.REPO, "tests", "host_build", "_build", "libcanon_pack_host.so")


@pytest.fixture(scope="module")
def lib():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-shared", "-fPIC", SRC, "-o", OUT], check=True)
    L = ctypes.CDLL(OUT)
    L.emu_pack.argtypes = [ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p]
    return L


def pack(L, nrows, maxr, n=None):
    n = len(nrows) if nrows is not None else n
    order = np.zeros(n, np.uint32)
    rows = np.zeros(n, np.uint32)
    copied = np.zeros(n, np.uint8)
    nr = None if nrows is None else np.ascontiguousarray(nrows, np.uint8)
    ok = L.emu_pack(n, None if nr is None else nr.ctypes.data, maxr, order.ctypes.data, rows.ctypes.data,
                    copied.ctypes.data)
    return ok, order, rows, copied


@pytest.mark.parametrize("n", [1, 100, 65535, 65536, 300001])
def test_stable_order_of_filled_rows(lib, n):
    rng = np.random.default_rng(n)
    nrows = rng.integers(1, 16, size=n).astype(np.uint8)
    ok, order, rows, copied = pack(lib, nrows, 15)
    assert ok == 1
    assert np.array_equal(order, np.argsort(nrows, kind="stable"))
    assert np.array_equal(rows, np.sort(nrows))
    assert (copied == 1).all()


def test_all_rows_filled_keeps_the_submission_order(lib):
    ok, order, rows, copied = pack(lib, None, 15, n=200000)
    assert ok == 1 and np.array_equal(order, np.arange(200000)) and (rows == 15).all()


@pytest.mark.parametrize("bad", [0, 16, 255])
def test_out_of_range_row_count_refuses_the_batch(lib, bad):
    nrows = np.full(100000, 7, np.uint8)
    nrows[77777] = bad
    ok, _, _, _ = pack(lib, nrows, 15)
    assert ok == 0
