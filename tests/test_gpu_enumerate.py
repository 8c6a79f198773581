"""Frontier-batched enumeration with the GPU check (configs 1 and 5) against the
reference's known answers."""
import collections
import json
import os

import numpy as np
import pytest

import cases
import oracle

pytestmark = pytest.mark.gpu

HIST = json.load(open(os.path.join(cases.GOLDEN, "bibd_histograms.json")))


@pytest.mark.parametrize("key", ["7,7,3,3,1", "7,14,6,3,2", "9,12,4,3,1", "13,26,6,3,1", "8,14,7,4,3",
                                 "11,11,5,5,2", "10,15,6,4,2", "9,18,8,4,3"])
def test_bibd_enumeration_histograms(ctx, key):
    v, b, r, k, lam = map(int, key.split(","))
    found, st = ctx.enumerate_bibd(v, b, r, k, lam)
    hist = collections.Counter(a for _, a in found)
    assert dict(hist) == {int(a): c for a, c in HIST[key].items()}
    assert st.designs == len(found) and st.checks > 0


def test_sts13_designs_equal_oracle_enumeration(ctx):
    found, _ = ctx.enumerate_bibd(13, 26, 6, 3, 1)
    ref, _ = oracle.bibd_enumerate(13, 26, 6, 3, 1)
    assert {M.tobytes(): a for M, a in found} == {M.tobytes(): a for M, a in ref}


def test_sts15_enumeration_gives_the_80_fixture_designs(ctx):
    found, st = ctx.enumerate_bibd(15, 35, 7, 3, 1)
    fixture = {M.tobytes(): a for M, a in cases.load_sts15()}
    assert {M.tobytes(): a for M, a in found} == fixture


def test_k10_enumeration_gives_the_reference_matrices(ctx):
    found, st = ctx.enumerate_ksys(10)
    gold = {R.tobytes(): a for R, a in cases.load_k10()}
    assert len(found) == 396
    assert {R.tobytes(): a for R, a in found} == gold


def test_small_complete_graphs(ctx):
    f6, _ = ctx.enumerate_ksys(6)
    assert [a for _, a in f6] == [120]
    f8, _ = ctx.enumerate_ksys(8)
    ref8, _ = oracle.ksys_enumerate(8)
    assert {R.tobytes(): a for R, a in f8} == {R.tobytes(): a for R, a in ref8}
