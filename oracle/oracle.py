"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle (canon_oracle.c) restates the reference canonicity checkers on the
CPU.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
it; it is the checker of the CUDA path, never part of the product.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libcanon_oracle.so")

SAVE_NOTHING = 0
SAVE_ROW_PERM = 1
SAVE_ROW_TO_CHANGE = 4
FULL_AUT = 0x100
SAVE_AUT_ROWS = 0x200


class Stats(ctypes.Structure):
    _fields_ = [("trials", ctypes.c_uint64), ("rows", ctypes.c_uint64),
                ("orbits", ctypes.c_uint64), ("auts", ctypes.c_uint64)]


class BibdResult(ctypes.Structure):
    _fields_ = [("canonical", ctypes.c_int), ("reject_row", ctypes.c_int),
                ("row_to_change", ctypes.c_int), ("witness", ctypes.c_uint8 * 64),
                ("aut_lo", ctypes.c_uint64), ("aut_hi", ctypes.c_uint64),
                ("n_perm", ctypes.c_int), ("len_perm", ctypes.c_int),
                ("perm_arena", ctypes.POINTER(ctypes.c_uint8)), ("perm_cap", ctypes.c_int),
                ("perm_overflow", ctypes.c_int), ("st", Stats)]


class KsysResult(ctypes.Structure):
    _fields_ = [("canonical", ctypes.c_int), ("player_index", ctypes.c_int),
                ("n_aut", ctypes.c_uint64), ("aut_arena", ctypes.POINTER(ctypes.c_uint8)),
                ("aut_cap", ctypes.c_int), ("aut_overflow", ctypes.c_int),
                ("candidates", ctypes.c_uint64)]


class OrGroup(ctypes.Structure):
    _fields_ = [("stab", ctypes.c_uint), ("stab_aut", ctypes.c_uint),
                ("order_lo", ctypes.c_uint64), ("order_hi", ctypes.c_uint64)]


DESIGN_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8), ctypes.c_int,
                             ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64)

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        L.or_bibd_test.argtypes = [u8p, ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.c_int,
                                   ctypes.POINTER(BibdResult)]
        L.or_bibd_canonize.argtypes = [u8p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(BibdResult)]
        L.or_bibd_normalize.argtypes = [u8p, ctypes.c_int, ctypes.c_int]
        L.or_bibd_is_normal.argtypes = [u8p, ctypes.c_int, ctypes.c_int]
        L.or_ksys_test.argtypes = [u8p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(KsysResult)]
        L.or_bibd_enumerate.argtypes = [ctypes.c_int] * 5 + [DESIGN_CB, ctypes.c_void_p,
                                                            ctypes.POINTER(ctypes.c_uint64)]
        L.or_bibd_enumerate.restype = ctypes.c_long
        L.or_ksys_enumerate.argtypes = [ctypes.c_int, DESIGN_CB, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_uint64)]
        L.or_ksys_enumerate.restype = ctypes.c_long
        L.or_sts_hillclimb.argtypes = [ctypes.c_int, ctypes.c_uint64, u8p]
        L.or_sts_random_rows.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64,
                                         ctypes.POINTER(ctypes.c_uint64)]
        L.or_set_group_impl.argtypes = [ctypes.c_void_p] * 3
        L.or_next_permutation.argtypes = [ctypes.POINTER(OrGroup), u8p, u8p, ctypes.c_uint8,
                                          ctypes.c_uint8, ctypes.c_uint8]
        L.or_next_permutation.restype = ctypes.c_uint8
        L.or_add_automorphism.argtypes = [ctypes.POINTER(OrGroup), ctypes.c_uint, u8p, u8p,
                                          ctypes.c_int, ctypes.c_int]
        L.or_update_group_order.argtypes = [ctypes.POINTER(OrGroup), ctypes.c_uint, u8p]
        _lib = L
    return _lib


def _u8p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def bibd_test(M, flags=SAVE_ROW_PERM | SAVE_ROW_TO_CHANGE, perm_cap=0, len_stab=0):
    """TestCanonicity on a normalised 0/1 matrix (rows x b).  Returns a dict."""
    M = np.ascontiguousarray(M, dtype=np.uint8)
    nr, b = M.shape
    res = BibdResult()
    arena = None
    if perm_cap:
        arena = np.zeros(perm_cap * 64, np.uint8)
        res.perm_arena = _u8p(arena)
        res.perm_cap = perm_cap
    rc = lib().or_bibd_test(_u8p(M), nr, b, flags, len_stab, ctypes.byref(res))
    if rc < 0:
        raise ValueError("oracle rejected input (rc=%d)" % rc)
    out = dict(canonical=bool(res.canonical), reject_row=res.reject_row,
               row_to_change=res.row_to_change, witness=bytes(res.witness[:nr]),
               aut=res.aut_lo | (res.aut_hi << 64), n_perm=res.n_perm, len_perm=res.len_perm,
               perm_overflow=bool(res.perm_overflow), trials=res.st.trials, rows=res.st.rows,
               orbits=res.st.orbits, auts=res.st.auts)
    if arena is not None:
        n = min(res.n_perm, perm_cap)
        out["perms"] = arena[: n * res.len_perm].reshape(n, res.len_perm).copy() if n else \
            np.zeros((0, res.len_perm), np.uint8)
    return out


def bibd_normalize(M):
    M = np.array(M, dtype=np.uint8, copy=True, order="C")
    lib().or_bibd_normalize(_u8p(M), M.shape[0], M.shape[1])
    return M


def bibd_is_normal(M):
    M = np.ascontiguousarray(M, dtype=np.uint8)
    return bool(lib().or_bibd_is_normal(_u8p(M), M.shape[0], M.shape[1]))


def bibd_canonize(M):
    M = np.array(M, dtype=np.uint8, copy=True, order="C")
    res = BibdResult()
    calls = lib().or_bibd_canonize(_u8p(M), M.shape[0], M.shape[1], ctypes.byref(res))
    if calls < 0:
        raise ValueError("oracle rejected input")
    return M, res.aut_lo | (res.aut_hi << 64), calls


def ksys_test(R, full_aut=False, aut_cap=0, g=2):
    """cnvCheckNew() of the rounds R (rows of np players in groups of g)."""
    R = np.ascontiguousarray(R, dtype=np.uint8)
    nr, np_ = R.shape
    res = KsysResult()
    arena = None
    if aut_cap:
        arena = np.zeros(aut_cap * np_, np.uint8)
        res.aut_arena = _u8p(arena)
        res.aut_cap = aut_cap
    rc = lib().or_ksys_test(_u8p(R), nr, np_, g, int(full_aut), ctypes.byref(res))
    if rc < 0:
        raise ValueError("oracle rejected input")
    out = dict(canonical=bool(res.canonical), player_index=res.player_index, n_aut=res.n_aut,
               candidates=res.candidates, aut_overflow=bool(res.aut_overflow))
    if arena is not None:
        n = min(res.n_aut, aut_cap)
        out["auts"] = arena[: n * np_].reshape(n, np_).copy()
    return out


def ksys_binary_canonize(R, np_, k=2, day_numb=0):
    """runCanonizer(): the canonical binary matrix (np x day_numb*np/k bytes) of the
    first day_numb rounds of a k-system (all rounds when day_numb <= 0)."""
    R = np.ascontiguousarray(R, dtype=np.uint8)
    days = (np_ - 1) // (k - 1) if day_numb <= 0 else day_numb
    out = np.zeros(np_ * days * (np_ // k), np.uint8)
    steps = ctypes.c_long()
    b = lib().or_ksys_binary_canonize(_u8p(R), np_, k, day_numb, _u8p(out), ctypes.byref(steps))
    if b < 0:
        raise ValueError("oracle rejected input (rc=%d)" % b)
    return out.reshape(np_, b), steps.value


def bibd_enumerate(v, b, r, k, lam):
    found = []

    def cb(user, M, v_, b_, lo, hi):
        arr = np.ctypeslib.as_array(M, shape=(v_ * b_,)).reshape(v_, b_).copy()
        found.append((arr, lo | (hi << 64)))

    c = DESIGN_CB(cb)
    nchk = ctypes.c_uint64()
    n = lib().or_bibd_enumerate(v, b, r, k, lam, c, None, ctypes.byref(nchk))
    assert n == len(found)
    return found, nchk.value


def ksys_enumerate(n):
    found = []

    def cb(user, M, rows, cols, lo, hi):
        arr = np.ctypeslib.as_array(M, shape=(rows * cols,)).reshape(rows, cols).copy()
        found.append((arr, lo))

    c = DESIGN_CB(cb)
    nchk = ctypes.c_uint64()
    cnt = lib().or_ksys_enumerate(n, c, None, ctypes.byref(nchk))
    assert cnt == len(found)
    return found, nchk.value


def sts_hillclimb(v, seed):
    b = v * (v - 1) // 6
    blocks = np.zeros(b * 3, np.uint8)
    lib().or_sts_hillclimb(v, seed, _u8p(blocks))
    return blocks.reshape(b, 3)


def sts_random_rows(v, seed, index):
    """Item `index` of a seeded STS(v) batch as packed rows (uint64, bit c = column c)."""
    rows = np.zeros(v, np.uint64)
    lib().or_sts_random_rows(v, seed, index, rows.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    return rows


def rows_to_matrix(rows, b):
    rows = np.asarray(rows, dtype=np.uint64)
    return ((rows[:, None] >> np.arange(b, dtype=np.uint64)) & np.uint64(1)).astype(np.uint8)


def use_reference_group_order(ref_lib_path):
    """Route the checker's permutation machinery through the reference's own
    CGroupOrder<T> (oracle/_ref/libref_grouporder.so); None restores the restatement."""
    L = lib()
    if ref_lib_path is None:
        L.or_set_group_impl(None, None, None)
        return None
    R = ctypes.CDLL(ref_lib_path)
    L.or_set_group_impl(ctypes.cast(R.ref_next_permutation, ctypes.c_void_p),
                        ctypes.cast(R.ref_add_automorphism, ctypes.c_void_p),
                        ctypes.cast(R.ref_update_group_order, ctypes.c_void_p))
    return R


def blocks_to_matrix(blocks, v):
    b = blocks.shape[0]
    M = np.zeros((v, b), np.uint8)
    for j, blk in enumerate(blocks):
        M[blk, j] = 1
    return M
