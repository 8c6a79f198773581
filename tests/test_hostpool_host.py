"""The persistent pool of host threads that packs batches and builds enumeration levels
(incidence-system-enumeration_gb300/csrc/canon_hostpool.h), compiled for the host: every
job of a call runs exactly once, ranges cover their interval exactly, and calls from
several host threads at once are serialised without losing or repeating a job."""
import ctypes
import os
import subprocess

import pytest

import conftest

SRC = os.path.join(conftest.REPO, "tests", "host_build", "canon_hostpool_host.cpp")
OUT = os.path.join(conftest.REPO, "tests", "host_build", "_build", "libcanon_hostpool_host.so")


@pytest.fixture(scope="module")
def pool():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-shared", "-fPIC", SRC, "-o", OUT], check=True)
    L = ctypes.CDLL(OUT)
    L.emu_pool_run.restype = ctypes.c_long
    L.emu_pool_run.argtypes = [ctypes.c_uint, ctypes.c_uint, ctypes.c_uint]
    L.emu_pool_ranges.restype = ctypes.c_long
    L.emu_pool_ranges.argtypes = [ctypes.c_ulonglong]
    L.emu_pool_threads.restype = ctypes.c_uint
    return L


def test_every_job_runs_once(pool):
    assert 1 <= pool.emu_pool_threads() <= 16
    for n in (1, 2, 3, 16, 17, 64, 1000):
        assert pool.emu_pool_run(n, 20, 1) == 0, n


def test_calls_from_several_threads(pool):
    assert pool.emu_pool_run(37, 50, 4) == 0


@pytest.mark.parametrize("n", [0, 1, 5, 15, 16, 63, 64, 65, 1000, 123457])
def test_ranges_cover_once(pool, n):
    assert pool.emu_pool_ranges(n) == 0
