"""Seeded test inputs shared by the parity tests (built on the CPU)."""
import os

import numpy as np

import oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_sts15():
    out = []
    with open(os.path.join(GOLDEN, "sts15_canonical.txt")) as f:
        for line in f:
            if line.startswith("#"):
                continue
            parts = line.split()
            M = np.array([[int(ch) for ch in row] for row in parts[1:]], np.uint8)
            out.append((M, int(parts[0])))
    return out


def load_k10():
    out = []
    with open(os.path.join(GOLDEN, "k10_canonical.txt")) as f:
        for line in f:
            if line.startswith("#"):
                continue
            aut, rest = line.split(" ", 1)
            rows = [[int(x) for x in r.split()] for r in rest.split("|")]
            out.append((np.array(rows, np.uint8), int(aut)))
    return out


def permute_normalize(M, rng):
    """Random row + column permutation of M, columns brought to normal form."""
    P = M[rng.permutation(M.shape[0])][:, rng.permutation(M.shape[1])]
    return oracle.bibd_normalize(P)


def bibd_designs(v, b, r, k, lam):
    found, _ = oracle.bibd_enumerate(v, b, r, k, lam)
    return found


def ksys_sorted_form(R):
    """Bring rounds (pairs) to the reference's result() form: pairs ascending,
    ordered by first player, rounds ordered by their second entry."""
    out = []
    for row in R:
        pairs = sorted(tuple(sorted((int(row[i]), int(row[i + 1])))) for i in range(0, len(row), 2))
        out.append([x for p in pairs for x in p])
    out.sort(key=lambda r: r[1])
    return np.array(out, np.uint8)


def ksys_relabel_random(R, rng):
    """Random relabeling of a complete/partial k-system that maps a random round onto
    round 0 = (0 1)(2 3)..., then the sorted form."""
    nr, n = R.shape
    d = int(rng.integers(nr))
    pairs = [(int(R[d][i]), int(R[d][i + 1])) for i in range(0, n, 2)]
    order = rng.permutation(len(pairs))
    lab = np.zeros(n, np.int64)
    for new_g, gi in enumerate(order):
        a, b = pairs[gi]
        if rng.integers(2):
            a, b = b, a
        lab[a], lab[b] = 2 * new_g, 2 * new_g + 1
    return ksys_sorted_form(lab[R])
