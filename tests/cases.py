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


def load_kts15():
    """The 7 canonical Kirkman triple systems on 15 points (rounds of 5 groups of 3)."""
    return load_k10("kts15_canonical.txt")


def load_k10(name="k10_canonical.txt"):
    out = []
    with open(os.path.join(GOLDEN, name)) as f:
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


def ksys_sorted_form(R, g=2):
    """Bring rounds to the reference's result() form: the players of every group
    ascending, groups ordered by their first player, rounds ordered by their second
    entry."""
    out = []
    for row in R:
        groups = sorted(tuple(sorted(int(row[i + j]) for j in range(g))) for i in range(0, len(row), g))
        out.append([x for grp in groups for x in grp])
    out.sort(key=lambda r: r[1])
    return np.array(out, np.uint8)


def ksys_relabel_random(R, rng, g=2):
    """Random relabeling of a complete/partial k-system that maps a random round onto
    round 0 = (0 1 ..)(g ..)..., then the sorted form."""
    nr, n = R.shape
    d = int(rng.integers(nr))
    groups = [[int(R[d][i + j]) for j in range(g)] for i in range(0, n, g)]
    order = rng.permutation(len(groups))
    lab = np.zeros(n, np.int64)
    for new_g, gi in enumerate(order):
        members = [groups[gi][k] for k in rng.permutation(g)]
        for k, a in enumerate(members):
            lab[a] = g * new_g + k
    return ksys_sorted_form(lab[R], g)


def ksys_relabel_keep_round0(R, rng, g=2):
    """Random relabeling that maps round 0 onto itself (groups and the players inside
    them permuted), then the sorted form: an isomorphic copy, mostly not canonical."""
    nr, n = R.shape
    lab = np.zeros(n, np.int64)
    for new_g, gi in enumerate(rng.permutation(n // g)):
        for k, pos in enumerate(rng.permutation(g)):
            lab[gi * g + pos] = g * new_g + k
    return ksys_sorted_form(lab[R], g)


def ksys_random_partial(np_, g, nr, rng, attempts=50, tries=200):
    """A random partial k-system in sorted form: round 0 = 0 1 .. np-1, every further
    round a random partition into groups of g that repeats no pair (None if the
    bounded random search finds none)."""
    for _ in range(attempts):
        rows = [list(range(np_))]
        used = {(a, b) for k in range(0, np_, g) for a in range(k, k + g) for b in range(a + 1, k + g)}
        ok = True
        for _r in range(1, nr):
            for _t in range(tries):
                perm = [int(x) for x in rng.permutation(np_)]
                groups = [sorted(perm[i:i + g]) for i in range(0, np_, g)]
                pairs = {(a, b) for grp in groups for i, a in enumerate(grp) for b in grp[i + 1:]}
                if not pairs & used:
                    break
            else:
                ok = False
                break
            used |= pairs
            rows.append([x for grp in sorted(groups) for x in grp])
        if ok:
            return ksys_sorted_form(np.array(rows, np.uint8), g)
    return None


def load_result_tables():
    import json
    with open(os.path.join(GOLDEN, "bibd_result_tables.json")) as f:
        return json.load(f)


def simple_design(M):
    """No replicated block: all columns distinct."""
    cols = {bytes(M[:, c]) for c in range(M.shape[1])}
    return len(cols) == M.shape[1]


def oracle_transitive(M):
    """Aut(D) transitive on the points, from the row automorphisms that the oracle's
    TestCanonicity stores (union of their cycles)."""
    o = oracle.bibd_test(M, oracle.SAVE_ROW_PERM | oracle.SAVE_AUT_ROWS, perm_cap=1 << 14)
    assert o["canonical"] and not o["perm_overflow"]
    v = M.shape[0]
    parent = list(range(v))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for p in o["perms"]:
        for i in range(v):
            a, b = find(i), find(int(p[i]))
            if a != b:
                parent[max(a, b)] = min(a, b)
    return len({find(i) for i in range(v)}) == 1


def table_rows(designs, simple, transitive):
    """[[|Aut|, Nd, Ns, Ndt, Nst], ...] by increasing |Aut|, as the reference counts them."""
    rows = {}
    for (_, aut), s, t in zip(designs, simple, transitive):
        r = rows.setdefault(aut, [aut, 0, 0, 0, 0])
        r[1] += 1
        r[2] += bool(s)
        r[3] += bool(t)
        r[4] += bool(s and t)
    return [rows[a] for a in sorted(rows)]


def oracle_sts_check(rows, b=35):
    """Oracle outputs of a complete STS check with |Aut| of rejected matrices from
    their canonical form (COMPLETE|RAW|AUT_CANON): (canonical, witness, aut)."""
    M = oracle.bibd_normalize(oracle.rows_to_matrix(rows, b))
    o = oracle.bibd_test(M, oracle.SAVE_ROW_PERM | oracle.SAVE_ROW_TO_CHANGE)
    aut = o["aut"]
    if not o["canonical"]:
        _, aut, _ = oracle.bibd_canonize(M)
    return o["canonical"], o["witness"], aut, o["row_to_change"]


def compare_sts_sample(rows, can, wit, aut, idx, v=15, b=35):
    """Every item of `idx` against the oracle (host threads)."""
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        for i, (oc, ow, oa, _) in zip(idx, ex.map(lambda i: oracle_sts_check(rows[i], b), idx)):
            assert bool(can[i]) == oc, i
            assert int(aut[i][0]) == oa and int(aut[i][1]) == 0, (i, aut[i], oa)
            if not oc:
                assert bytes(wit[i][:v]) == ow, i
