"""Host-side binding of the GB300 canonicity-check engine (libcanon_gb300.so).

The engine is C-ABI native code (include/canon_gb300.h); this module is a thin
ctypes layer for Python callers, tests and the benchmark.  It mirrors the
reference's checker surface:

  CanonicityChecker.TestCanonicity()   CCanonicityChecker::TestCanonicity(),
                                       Source/CanonicityChecker.h:58,255-586
  CanonicityChecker.CanonizeMatrix()   CMatrixCanonChecker::CanonizeMatrix(),
                                       Source/MatrixCanonChecker.cpp:420-564
  KSysChecker.cnvCheckNew()            alldata::cnvCheckNew(),
                                       k-Factorization/TripleSys/Source/cnv.cpp:211

There is no CPU fallback: if the native library is missing or no GPU is
present, construction raises.
"""
import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libcanon_gb300.so")

CANON_OK = 0
CANON_EINVAL = -1
CANON_ENOMEM = -2
CANON_ECUDA = -3
CANON_ETIMEOUT = -4
CANON_ENODEV = -5
CANON_ESIZE = -6
NOALLOC_MAX_ITEMS = 65536

ST_OK = 0
ST_BADINPUT = 1
ST_TIMEOUT = 2
ST_PERM_OVF = 4

COMPLETE = 0x1
RAW = 0x2
FULL_AUT = 0x4
SAVE_AUTS = 0x8
AUT_CANON = 0x10
REFERENCE_ORDER = 0x20
VERDICT_ONLY = 0x40

# t_canonOutInfo of the reference (Source/CanonicityChecker.h:27-32)
t_saveNothing = 0
t_saveRowPermutations = 1
t_saveColPermutations = 2
t_saveRowToChange = 4

HEADER_SYMBOLS = [
    "canon_create", "canon_destroy", "canon_last_error", "canon_submit_bibd", "canon_submit_ksys",
    "canon_submit_ksys_groups", "canon_sync", "canon_set_ordering", "canon_canonize_bibd", "canon_check_bibd_device",
    "canon_generate_sts_device", "canon_device_alloc", "canon_device_free", "canon_memcpy_d2h",
    "canon_memcpy_h2d", "canon_last_kernel_ms", "canon_kernel_launches", "canon_stream_sync",
    "canon_check_bibd_noalloc", "canon_enumerate_bibd", "canon_enumerate_ksys",
    "canon_enumerate_ksys_groups", "canon_mlp_features",
    "canon_label_first_rows", "canon_mlp_forward", "canon_mlp_grad", "canon_mlp_train",
    "canon_design_properties", "canon_report_bibd", "canon_ksys_cycles", "canon_report_ksys",
    "canon_tune_bibd", "canon_generate_partial_bibd", "canon_generate_partial_ksys", "canon_lexmax_nodes_bibd",
    "canon_measure_int_peak", "canon_canonize_ksys_binary", "canon_canonize_ksys_binary_groups",
    "canon_set_ksys_segment",
]
# the reference's plugin (k-Factorization/Utils/Include/CDTools.h:9-11)
PLUGIN_SYMBOLS = ["createCanonizer", "releaseCanonizer", "runCanonizer"]
MLP_PARAMS = 128 * 64 + 128 + 128 * 128 + 128 + 128 + 1


class CanonError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("canon error %d: %s" % (code, msg))
        self.code = code


class Cfg(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("max_items", ctypes.c_uint32),
                ("max_words", ctypes.c_uint32), ("aut_cap", ctypes.c_uint32),
                ("max_trials", ctypes.c_uint64), ("options", ctypes.c_uint32)]


OPT_AUT_PRUNE = 0x1
OPT_VERDICT_SYNC = 0x2    # canon_sync returns only canonical + status
KSYS_WHOLE = 0xFFFFFFFF   # canon_set_ksys_segment: one warp per matrix
OPT_NO_GRAPH = 0x4        # canon_enumerate_ksys level by level instead of its captured graph
OPT_MLP_WARP_MMA = 0x8    # the MLP forward on mma.sync instead of tcgen05


class BibdBatch(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("v", ctypes.c_uint32), ("b", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("rows", ctypes.POINTER(ctypes.c_uint64)),
                ("nrows", ctypes.POINTER(ctypes.c_uint8))]


class KsysBatch(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("np", ctypes.c_uint32), ("rounds", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("data", ctypes.POINTER(ctypes.c_uint8)),
                ("nrows", ctypes.POINTER(ctypes.c_uint8))]


class DeviceOutputs(ctypes.Structure):
    """canon_device_outputs: device pointers of canon_check_bibd_noalloc's outputs."""
    _fields_ = [("canonical", ctypes.c_void_p), ("status", ctypes.c_void_p),
                ("reject_row", ctypes.c_void_p), ("row_to_change", ctypes.c_void_p),
                ("player_index", ctypes.c_void_p), ("witness", ctypes.c_void_p),
                ("aut", ctypes.c_void_p), ("trials", ctypes.c_void_p), ("n_auts", ctypes.c_void_p),
                ("len_aut", ctypes.c_void_p), ("auts", ctypes.c_void_p), ("aut_cap", ctypes.c_uint32)]


class EnumStats(ctypes.Structure):
    _fields_ = [("checks", ctypes.c_uint64), ("designs", ctypes.c_uint64), ("levels", ctypes.c_uint32),
                ("batches", ctypes.c_uint32), ("seconds", ctypes.c_double), ("kernel_ms", ctypes.c_double),
                ("level_checks", ctypes.c_uint64 * 16), ("level_kernel_ms", ctypes.c_double * 16),
                ("gen_seconds", ctypes.c_double), ("trials", ctypes.c_uint64),
                ("level_gen_ms", ctypes.c_double * 16)]


DESIGN_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8), ctypes.c_uint32,
                             ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64)


class TuneResult(ctypes.Structure):
    _fields_ = [("variant", ctypes.c_int), ("ms", ctypes.c_float * 6)]


VARIANT_SINGLE, VARIANT_TWO_PASS, VARIANT_SPLIT, VARIANT_CONVERGED = 0, 1, 2, 3
VARIANT_CONVERGED_D2, VARIANT_CONVERGED_D8 = 4, 5
VARIANT_NAMES = ["one pass", "two passes", "split by first row", "two passes, converged lex-max pass",
                 "two passes, converged lex-max pass, loads staged 2 ahead",
                 "two passes, converged lex-max pass, loads staged 8 ahead"]


class MlpWeights(ctypes.Structure):
    _fields_ = [("in_dim", ctypes.c_uint32), ("hidden", ctypes.c_uint32),
                ("w1", ctypes.POINTER(ctypes.c_uint16)), ("w2", ctypes.POINTER(ctypes.c_uint16)),
                ("w3", ctypes.POINTER(ctypes.c_uint16)), ("b1", ctypes.POINTER(ctypes.c_float)),
                ("b2", ctypes.POINTER(ctypes.c_float)), ("b3", ctypes.POINTER(ctypes.c_float))]


class Results(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32),
                ("canonical", ctypes.POINTER(ctypes.c_uint8)),
                ("status", ctypes.POINTER(ctypes.c_uint8)),
                ("reject_row", ctypes.POINTER(ctypes.c_uint8)),
                ("row_to_change", ctypes.POINTER(ctypes.c_uint8)),
                ("player_index", ctypes.POINTER(ctypes.c_int32)),
                ("witness", ctypes.POINTER(ctypes.c_uint8)),
                ("aut", ctypes.POINTER(ctypes.c_uint64)),
                ("trials", ctypes.POINTER(ctypes.c_uint64)),
                ("n_auts", ctypes.POINTER(ctypes.c_uint16)),
                ("len_aut", ctypes.POINTER(ctypes.c_uint8)),
                ("auts", ctypes.POINTER(ctypes.c_uint8)),
                ("aut_cap", ctypes.c_uint32),
                ("kernel_ms", ctypes.c_float)]


_lib = None


def load_library(path=LIB_PATH):
    """Loads libcanon_gb300.so and declares the C ABI.  Raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise CanonError(CANON_ENODEV, "native library %s is not built (run build())" % path)
    L = ctypes.CDLL(path)
    vp, u32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64
    u64p = ctypes.POINTER(ctypes.c_uint64)
    L.canon_create.argtypes = [ctypes.POINTER(Cfg)]
    L.canon_create.restype = vp
    L.canon_destroy.argtypes = [vp]
    L.canon_last_error.argtypes = [vp]
    L.canon_last_error.restype = ctypes.c_char_p
    L.canon_submit_bibd.argtypes = [vp, ctypes.POINTER(BibdBatch)]
    L.canon_submit_ksys.argtypes = [vp, ctypes.POINTER(KsysBatch)]
    L.canon_submit_ksys_groups.argtypes = [vp, ctypes.POINTER(KsysBatch), u32]
    L.canon_sync.argtypes = [vp, ctypes.POINTER(Results)]
    L.canon_set_ordering.argtypes = [vp, vp]
    L.canon_canonize_bibd.argtypes = [vp, u32, u32, u32, u64p, u64p]
    L.canon_check_bibd_device.argtypes = [vp, u32, u32, u32, u32, vp, vp, vp, vp, vp, vp, vp]
    L.canon_generate_sts_device.argtypes = [vp, u32, u32, u64, ctypes.c_int, vp, vp]
    L.canon_device_alloc.argtypes = [vp, ctypes.c_size_t]
    L.canon_device_alloc.restype = vp
    L.canon_device_free.argtypes = [vp, vp]
    L.canon_memcpy_d2h.argtypes = [vp, vp, vp, ctypes.c_size_t]
    L.canon_memcpy_h2d.argtypes = [vp, vp, vp, ctypes.c_size_t]
    L.canon_last_kernel_ms.argtypes = [vp]
    L.canon_last_kernel_ms.restype = ctypes.c_float
    L.canon_kernel_launches.argtypes = [vp]
    L.canon_kernel_launches.restype = u64
    L.canon_stream_sync.argtypes = [vp]
    L.canon_check_bibd_noalloc.argtypes = [u32, u32, u32, u32, vp, vp, ctypes.POINTER(DeviceOutputs), u64, vp]
    L.canon_enumerate_bibd.argtypes = [vp, u32, u32, u32, u32, u32, DESIGN_CB, vp, ctypes.POINTER(EnumStats)]
    L.canon_enumerate_ksys.argtypes = [vp, u32, DESIGN_CB, vp, ctypes.POINTER(EnumStats)]
    L.canon_enumerate_ksys_groups.argtypes = [vp, u32, u32, DESIGN_CB, vp, ctypes.POINTER(EnumStats)]
    fp = ctypes.POINTER(ctypes.c_float)
    L.canon_mlp_features.argtypes = [vp, u32, u32, u32, vp, vp]
    L.canon_label_first_rows.argtypes = [vp, u32, u32, u32, u32, vp, vp, vp, vp]
    L.canon_mlp_forward.argtypes = [vp, u64, vp, fp, vp]
    L.canon_mlp_grad.argtypes = [vp, u64, vp, vp, fp, fp, fp]
    L.canon_mlp_train.argtypes = [vp, u64, vp, vp, u32, u32, ctypes.c_float, fp, fp]
    L.canon_set_ordering.argtypes = [vp, ctypes.POINTER(MlpWeights)]
    L.canon_set_ksys_segment.argtypes = [vp, u32]
    u8p, sz = ctypes.POINTER(ctypes.c_uint8), ctypes.c_size_t
    L.canon_tune_bibd.argtypes = [vp, u32, u32, u32, u32, vp, ctypes.POINTER(TuneResult)]
    L.canon_design_properties.argtypes = [vp, u32, u32, u32, u64p, u8p, u8p]
    L.canon_report_bibd.argtypes = [u32, u32, u32, u32, u32, u32, u64p, u8p, u8p, u64, ctypes.c_double,
                                    ctypes.c_char_p, sz]
    L.canon_report_bibd.restype = sz
    L.canon_ksys_cycles.argtypes = [u32, u32, u8p, ctypes.c_char_p, sz]
    L.canon_ksys_cycles.restype = sz
    L.canon_report_ksys.argtypes = [u32, u32, u32, u8p, u64p, ctypes.c_char_p, sz]
    L.canon_report_ksys.restype = sz
    L.canon_generate_partial_bibd.argtypes = [u32, u32, u32, u32, u32, u32, u64, u32, u32, u64p, u8p,
                                              ctypes.POINTER(ctypes.c_uint32)]
    L.canon_generate_partial_ksys.argtypes = [u32, u32, u64, u32, u32, u8p, u8p]
    L.canon_lexmax_nodes_bibd.argtypes = [vp, u32, u32, u32, u32, vp, vp, vp]
    L.canon_measure_int_peak.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
    L.canon_canonize_ksys_binary.argtypes = [vp, u32, u32, u32, u8p, u8p, u64p]
    L.canon_canonize_ksys_binary_groups.argtypes = [vp, u32, u32, u32, u32, u8p, u8p, u64p]
    L.createCanonizer.argtypes = [ctypes.c_int, ctypes.c_int]
    L.createCanonizer.restype = vp
    L.releaseCanonizer.argtypes = [vp]
    L.runCanonizer.argtypes = [vp, u8p, ctypes.c_int, ctypes.c_int]
    L.runCanonizer.restype = ctypes.POINTER(ctypes.c_uint8)
    _lib = L
    return L


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def to_bf16_bits(a):
    """FP32 -> BF16 bit patterns (round to nearest even)."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = u + 0x7FFF + ((u >> 16) & 1)
    return (u >> 16).astype(np.uint16)


def bf16_round(a):
    """FP32 values rounded to BF16 precision (as FP32)."""
    return (to_bf16_bits(a).astype(np.uint32) << 16).view(np.float32)


def init_mlp_params(seed):
    """He-initialised flat parameter vector of the 64-128-128-1 network."""
    rng = np.random.default_rng(seed)
    p = np.zeros(MLP_PARAMS, np.float32)
    p[:8192] = rng.normal(0, np.sqrt(2 / 64), 8192)
    p[8320:24704] = rng.normal(0, np.sqrt(2 / 128), 16384)
    p[24832:24960] = rng.normal(0, np.sqrt(1 / 128), 128)
    return p


def _text(call):
    """Runs a snprintf-convention writer twice: once for the length, once to fill."""
    n = call(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    call(buf, n + 1)
    return buf.value.decode()


def report_bibd(params, auts, simple=None, transitive=None, fully_constructed=0, seconds=0.0, lib=None):
    """The |Aut(D)| table of a BIBD run (canon_report_bibd), as text."""
    L = lib or load_library()
    v, b, r, k, lam = params
    n = len(auts)
    a = np.ascontiguousarray(auts, np.uint64)
    s_ = None if simple is None else np.ascontiguousarray(simple, np.uint8)
    t_ = None if transitive is None else np.ascontiguousarray(transitive, np.uint8)
    u8p = ctypes.POINTER(ctypes.c_uint8)
    return _text(lambda buf, cap: L.canon_report_bibd(
        v, b, r, k, lam, n, _ptr(a, ctypes.c_uint64), None if s_ is None else _ptr(s_, ctypes.c_uint8),
        None if t_ is None else _ptr(t_, ctypes.c_uint8), int(fully_constructed), float(seconds), buf, cap))


def ksys_cycles(M, lib=None):
    """Cycle descriptor of one k-system matrix (rounds x np, result() form)."""
    L = lib or load_library()
    M = np.ascontiguousarray(M, np.uint8)
    return _text(lambda buf, cap: L.canon_ksys_cycles(M.shape[1], M.shape[0], _ptr(M, ctypes.c_uint8), buf, cap))


def report_ksys(matrices, auts, lib=None):
    """The |Aut(M)| x cycles table of a k-system run (canon_report_ksys), as text."""
    L = lib or load_library()
    X = np.ascontiguousarray(np.stack(matrices), np.uint8)
    a = np.ascontiguousarray(auts, np.uint64)
    n, rounds, np_ = X.shape
    return _text(lambda buf, cap: L.canon_report_ksys(np_, rounds, n, _ptr(X, ctypes.c_uint8),
                                                      _ptr(a, ctypes.c_uint64), buf, cap))


def generate_partial_bibd(params, n, seed, min_rows, max_rows, lib=None):
    """n seeded partial BIBD(v,b,r,k,lambda) matrices by random backtracking of their
    rows (canon_generate_partial_bibd): (rows n x v uint64, nrows n uint8, number of
    items taken from a complete design)."""
    L = lib or load_library()
    v, b, r, k, lam = params
    rows = np.zeros((n, v), np.uint64)
    nrows = np.zeros(n, np.uint8)
    fc = ctypes.c_uint32(0)
    rc = L.canon_generate_partial_bibd(v, b, r, k, lam, n, seed, min_rows, max_rows, _ptr(rows, ctypes.c_uint64),
                                       _ptr(nrows, ctypes.c_uint8), ctypes.byref(fc))
    if rc != CANON_OK:
        raise CanonError(rc, "generate_partial_bibd")
    return rows, nrows, int(fc.value)


def generate_partial_ksys(np_, n, seed, min_rounds, max_rounds, lib=None):
    """n seeded partial 1-factorizations of K_np, round by round with random
    backtracking (canon_generate_partial_ksys): (data n x (np-1) x np uint8, nrows)."""
    L = lib or load_library()
    data = np.zeros((n, np_ - 1, np_), np.uint8)
    nrows = np.zeros(n, np.uint8)
    rc = L.canon_generate_partial_ksys(np_, n, seed, min_rounds, max_rounds, _ptr(data, ctypes.c_uint8),
                                       _ptr(nrows, ctypes.c_uint8))
    if rc != CANON_OK:
        raise CanonError(rc, "generate_partial_ksys")
    return data, nrows


def pack_rows(M):
    """0/1 matrix (rows x b, b <= 63) -> one uint64 per row, bit c = column c."""
    M = np.asarray(M, dtype=np.uint64)
    w = np.uint64(1) << np.arange(M.shape[-1], dtype=np.uint64)
    return (M * w).sum(axis=-1, dtype=np.uint64)


def unpack_rows(words, b):
    words = np.asarray(words, dtype=np.uint64)
    return ((words[..., None] >> np.arange(b, dtype=np.uint64)) & np.uint64(1)).astype(np.uint8)


class Context:
    """One engine context (one CUDA stream) on one GPU."""

    def __init__(self, device=0, max_items=1 << 16, max_words=0, aut_cap=64, max_trials=0, options=0):
        self.lib = load_library()
        cfg = Cfg(device, max_items, max_words, aut_cap, max_trials, options)
        self.h = self.lib.canon_create(ctypes.byref(cfg))
        if not self.h:
            raise CanonError(CANON_ENODEV, "canon_create failed (no GPU?)")
        self.aut_cap = aut_cap

    def close(self):
        if self.h:
            self.lib.canon_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != CANON_OK:
            raise CanonError(rc, self.lib.canon_last_error(self.h).decode())
        return rc

    def error(self):
        return self.lib.canon_last_error(self.h).decode()

    # ---- batched checks ----
    def submit_bibd(self, rows, v, b, flags=0, nrows=None):
        rows = np.ascontiguousarray(rows, dtype=np.uint64).reshape(-1)
        n = rows.size // v
        nr = None if nrows is None else np.ascontiguousarray(nrows, dtype=np.uint8)
        bt = BibdBatch(n, v, b, flags, _ptr(rows, ctypes.c_uint64),
                       _ptr(nr, ctypes.c_uint8) if nr is not None else None)
        self._check(self.lib.canon_submit_bibd(self.h, ctypes.byref(bt)))
        return n

    def submit_ksys(self, data, np_, rounds, flags=0, nrows=None):
        data = np.ascontiguousarray(data, dtype=np.uint8).reshape(-1)
        n = data.size // (np_ * rounds)
        nr = None if nrows is None else np.ascontiguousarray(nrows, dtype=np.uint8)
        bt = KsysBatch(n, np_, rounds, flags, _ptr(data, ctypes.c_uint8),
                       _ptr(nr, ctypes.c_uint8) if nr is not None else None)
        self._check(self.lib.canon_submit_ksys(self.h, ctypes.byref(bt)))
        return n

    def submit_ksys_groups(self, data, np_, rounds, group_size, flags=0, nrows=None):
        """canon_submit_ksys_groups: k-systems with groups of 2, 3 or 4 players."""
        data = np.ascontiguousarray(data, dtype=np.uint8).reshape(-1)
        n = data.size // (np_ * rounds)
        nr = None if nrows is None else np.ascontiguousarray(nrows, dtype=np.uint8)
        bt = KsysBatch(n, np_, rounds, flags, _ptr(data, ctypes.c_uint8),
                       _ptr(nr, ctypes.c_uint8) if nr is not None else None)
        self._check(self.lib.canon_submit_ksys_groups(self.h, ctypes.byref(bt), group_size))
        return n

    def sync(self, allow_timeout=False, raw=False, copy=True):
        """Runs canon_sync and copies the result arrays.  raw: |Aut| stays an (n, 2)
        uint64 array (low, high words) and the automorphism arena is not copied, so
        no per-item Python work is done.  copy=False (with raw): the arrays are views
        of the library's pinned result buffers, as the C API hands them out, valid
        until the next sync or close of this context."""
        r = Results()
        rc = self.lib.canon_sync(self.h, ctypes.byref(r))
        if rc != CANON_OK and not (allow_timeout and rc == CANON_ETIMEOUT):
            raise CanonError(rc, self.error())
        n = r.n
        out = {"n": n, "kernel_ms": r.kernel_ms}
        if n and raw:
            def view(p, count, dt):
                a = np.ctypeslib.as_array(p, shape=(count,)).view(dt)
                return a.copy() if copy else a
            out["canonical"] = view(r.canonical, n, np.uint8)
            out["status"] = view(r.status, n, np.uint8)
            out["witness"] = view(r.witness, n * 16, np.uint8).reshape(n, 16)
            out["aut"] = view(r.aut, 2 * n, np.uint64).reshape(n, 2)
            out["reject_row"] = view(r.reject_row, n, np.uint8)
            out["row_to_change"] = view(r.row_to_change, n, np.uint8)
            out["trials"] = view(r.trials, n, np.uint64)
            out["player_index"] = view(r.player_index, n, np.int32)
        elif n:
            def arr(p, count, dt):
                return np.ctypeslib.as_array(p, shape=(count,)).astype(dt, copy=True)
            out["canonical"] = arr(r.canonical, n, np.uint8).astype(bool)
            out["status"] = arr(r.status, n, np.uint8)
            out["reject_row"] = arr(r.reject_row, n, np.uint8)
            out["row_to_change"] = arr(r.row_to_change, n, np.uint8)
            out["player_index"] = arr(r.player_index, n, np.int32)
            out["witness"] = arr(r.witness, n * 16, np.uint8).reshape(n, 16)
            a = arr(r.aut, 2 * n, np.uint64).reshape(n, 2)
            out["aut"] = [int(lo) | (int(hi) << 64) for lo, hi in a]
            out["trials"] = arr(r.trials, n, np.uint64)
            out["n_auts"] = arr(r.n_auts, n, np.uint16)
            out["len_aut"] = arr(r.len_aut, n, np.uint8)
            out["auts_raw"] = np.ctypeslib.as_array(r.auts, shape=(n * r.aut_cap * 64,)).reshape(
                n, r.aut_cap, 64).copy()
        return out

    def canonize_bibd(self, rows, v, b):
        rows = np.array(rows, dtype=np.uint64, copy=True).reshape(-1)
        n = rows.size // v
        aut = np.zeros(2 * n, np.uint64)
        self._check(self.lib.canon_canonize_bibd(self.h, n, v, b, _ptr(rows, ctypes.c_uint64),
                                                 _ptr(aut, ctypes.c_uint64)))
        return rows.reshape(n, v), [int(aut[2 * i]) | (int(aut[2 * i + 1]) << 64) for i in range(n)]

    # ---- device-resident path ----
    def alloc(self, nbytes):
        p = self.lib.canon_device_alloc(self.h, nbytes)
        if not p:
            raise CanonError(CANON_ENOMEM, self.error())
        return p

    def free(self, p):
        self._check(self.lib.canon_device_free(self.h, p))

    def d2h(self, dst_array, src_ptr):
        self._check(self.lib.canon_memcpy_d2h(self.h, dst_array.ctypes.data, src_ptr, dst_array.nbytes))
        return dst_array

    def h2d(self, dst_ptr, src_array):
        src_array = np.ascontiguousarray(src_array)
        self._check(self.lib.canon_memcpy_h2d(self.h, dst_ptr, src_array.ctypes.data, src_array.nbytes))

    def generate_sts_device(self, n, v, seed, canon_odd, d_rows):
        self._check(self.lib.canon_generate_sts_device(self.h, n, v, seed, int(canon_odd), d_rows, None))

    def check_bibd_device(self, n, v, b, flags, d_rows, d_canonical, d_witness=None, d_aut=None,
                          d_status=None, d_trials=None, stream=None):
        self._check(self.lib.canon_check_bibd_device(self.h, n, v, b, flags, d_rows, d_canonical,
                                                     d_witness, d_aut, d_status, d_trials, stream))

    # ---- frontier-batched enumeration ----
    def enumerate_bibd(self, v, b, r, k, lam):
        """All BIBD(v,b,r,k,lambda) up to isomorphism: [(matrix v x b uint8, |Aut|)], stats."""
        found = []

        def cb(user, M, rows, cols, lo, hi):
            words = np.ctypeslib.as_array(ctypes.cast(M, ctypes.POINTER(ctypes.c_uint64)),
                                          shape=(rows,)).copy()
            found.append((unpack_rows(words, cols), int(lo) | (int(hi) << 64)))

        c = DESIGN_CB(cb)
        st = EnumStats()
        self._check(self.lib.canon_enumerate_bibd(self.h, v, b, r, k, lam, c, None, ctypes.byref(st)))
        return found, st

    def lexmax_nodes_bibd(self, n, v, b, flags, d_rows, d_nodes, d_orders=None):
        """Lex-max nodes per matrix of the resident check's first pass (device array);
        d_orders: first-row orders (device, nibble-packed) or the installed / plain order."""
        self._check(self.lib.canon_lexmax_nodes_bibd(self.h, n, v, b, flags, d_rows, d_nodes, d_orders))

    def measure_int_peak(self):
        """32-bit integer lane operations per second of this GPU (canon_measure_int_peak)."""
        x = ctypes.c_double(0)
        self._check(self.lib.canon_measure_int_peak(self.h, ctypes.byref(x)))
        return x.value

    def canonize_ksys_binary(self, data, np_, days, k=2):
        """Canonical binary matrices (n x np x days*np/k) of n k-systems' first `days`
        rounds (groups of k), and the labelings reaching each (canon_canonize_ksys_binary,
        canon_canonize_ksys_binary_groups for k > 2)."""
        X = np.ascontiguousarray(data, np.uint8).reshape(-1, days, np_)
        n = X.shape[0]
        b = days * np_ // k
        out = np.zeros((n, np_, b), np.uint8)
        aut = np.zeros(n, np.uint64)
        if k == 2:
            rc = self.lib.canon_canonize_ksys_binary(self.h, n, np_, days, _ptr(X, ctypes.c_uint8),
                                                     _ptr(out, ctypes.c_uint8), _ptr(aut, ctypes.c_uint64))
        else:
            rc = self.lib.canon_canonize_ksys_binary_groups(self.h, n, np_, k, days, _ptr(X, ctypes.c_uint8),
                                                            _ptr(out, ctypes.c_uint8), _ptr(aut, ctypes.c_uint64))
        self._check(rc)
        return out, aut

    def tune_bibd(self, n, v, b, flags, d_rows):
        """Autotunes the check variant for (v, b, flags) on n device-resident matrices;
        returns (variant kept, [ms per variant: -1 not applicable, -2 outputs differed])."""
        r = TuneResult()
        self._check(self.lib.canon_tune_bibd(self.h, n, v, b, flags, d_rows, ctypes.byref(r)))
        return r.variant, [float(x) for x in r.ms]

    def design_properties(self, designs):
        """(simple, transitive) flags of complete designs (v x b 0/1 matrices)."""
        designs = list(designs)
        if not designs:
            return np.zeros(0, np.uint8), np.zeros(0, np.uint8)
        v, b = designs[0].shape
        rows = np.ascontiguousarray(np.stack([pack_rows(M) for M in designs]), np.uint64)
        simple = np.zeros(len(designs), np.uint8)
        trans = np.zeros(len(designs), np.uint8)
        self._check(self.lib.canon_design_properties(self.h, len(designs), v, b, _ptr(rows, ctypes.c_uint64),
                                                     _ptr(simple, ctypes.c_uint8), _ptr(trans, ctypes.c_uint8)))
        return simple, trans

    def enumerate_ksys(self, np_):
        """All 1-factorizations of K_np up to isomorphism: [(rounds x np uint8, |Aut|)], stats."""
        found = []

        def cb(user, M, rows, cols, lo, hi):
            found.append((np.ctypeslib.as_array(M, shape=(rows * cols,)).reshape(rows, cols).copy(), int(lo)))

        c = DESIGN_CB(cb)
        st = EnumStats()
        self._check(self.lib.canon_enumerate_ksys(self.h, np_, c, None, ctypes.byref(st)))
        return found, st

    def enumerate_ksys_groups(self, np_, g):
        """All k-systems of np players in groups of g (2, 3 or 4) up to isomorphism:
        [(rounds x np uint8, |Aut|)], stats."""
        found = []

        def cb(user, M, rows, cols, lo, hi):
            found.append((np.ctypeslib.as_array(M, shape=(rows * cols,)).reshape(rows, cols).copy(),
                          int(lo) | (int(hi) << 64)))

        c = DESIGN_CB(cb)
        st = EnumStats()
        self._check(self.lib.canon_enumerate_ksys_groups(self.h, np_, g, c, None, ctypes.byref(st)))
        return found, st

    # ---- learned search order ----
    def mlp_features(self, n, v, b, d_rows, d_feat):
        self._check(self.lib.canon_mlp_features(self.h, n, v, b, d_rows, d_feat))

    def label_first_rows(self, n, v, b, flags, d_rows, d_first_rows, d_nodes=None, d_orders=None):
        self._check(self.lib.canon_label_first_rows(self.h, n, v, b, flags, d_rows, d_first_rows, d_nodes,
                                                    d_orders))

    def mlp_forward(self, n, d_x, params, d_logits):
        params = np.ascontiguousarray(params, np.float32)
        self._check(self.lib.canon_mlp_forward(self.h, n, d_x, _ptr(params, ctypes.c_float), d_logits))

    def mlp_grad(self, n, d_x, d_labels, params):
        params = np.ascontiguousarray(params, np.float32)
        grad = np.zeros(MLP_PARAMS, np.float32)
        loss = ctypes.c_float()
        self._check(self.lib.canon_mlp_grad(self.h, n, d_x, d_labels, _ptr(params, ctypes.c_float),
                                            _ptr(grad, ctypes.c_float), ctypes.byref(loss)))
        return grad, loss.value

    def mlp_train(self, n, d_x, d_labels, params, epochs, batch, lr):
        params = np.array(params, np.float32, copy=True)
        losses = np.zeros(epochs, np.float32)
        self._check(self.lib.canon_mlp_train(self.h, n, d_x, d_labels, epochs, batch, lr,
                                             _ptr(params, ctypes.c_float), _ptr(losses, ctypes.c_float)))
        return params, losses

    def set_ksys_segment(self, cands):
        """Candidates per warp task of the k-system check: 0 = chosen per launch,
        KSYS_WHOLE = one warp per matrix (canon_set_ksys_segment)."""
        self._check(self.lib.canon_set_ksys_segment(self.h, cands))

    def set_ordering(self, params):
        """Install (or with None remove) the learned first-row order from flat FP32 params."""
        if params is None:
            self._check(self.lib.canon_set_ordering(self.h, None))
            return
        p = np.asarray(params, np.float32)
        bf = lambda a: (to_bf16_bits(a))
        w1, b1 = bf(p[:8192]), p[8192:8320].copy()
        w2, b2 = bf(p[8320:24704]), p[24704:24832].copy()
        w3, b3 = bf(p[24832:24960]), p[24960:24961].copy()
        self._keep = (w1, b1, w2, b2, w3, b3)
        w = MlpWeights(64, 128, _ptr(w1, ctypes.c_uint16), _ptr(w2, ctypes.c_uint16), _ptr(w3, ctypes.c_uint16),
                       _ptr(b1, ctypes.c_float), _ptr(b2, ctypes.c_float), _ptr(b3, ctypes.c_float))
        self._check(self.lib.canon_set_ordering(self.h, ctypes.byref(w)))

    def stream_sync(self):
        self._check(self.lib.canon_stream_sync(self.h))

    def last_kernel_ms(self):
        return float(self.lib.canon_last_kernel_ms(self.h))

    def kernel_launches(self):
        return int(self.lib.canon_kernel_launches(self.h))


class Canonizer:
    """The reference's plugin (createCanonizer / runCanonizer / releaseCanonizer,
    k-Factorization/Utils/Include/CDTools.h:9-11) through the C ABI."""

    def __init__(self, v, k=2):
        self.lib = load_library()
        self.v, self.k = v, k
        self.h = self.lib.createCanonizer(v, k)
        if not self.h:
            raise CanonError(CANON_EINVAL, "createCanonizer(%d, %d) failed" % (v, k))

    def run(self, matrix, iDay=0):
        """runCanonizer(): the canonical binary matrix (v x days*v/k) or None on error."""
        M = np.ascontiguousarray(matrix, np.uint8)
        p = self.lib.runCanonizer(self.h, _ptr(M, ctypes.c_uint8), self.k, iDay)
        if not p:
            return None
        days = (self.v - 1) // (self.k - 1) if iDay <= 0 else iDay
        b = days * self.v // self.k
        return np.ctypeslib.as_array(p, shape=(self.v * b,)).reshape(self.v, b).copy()

    def close(self):
        if self.h:
            self.lib.releaseCanonizer(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CanonicityChecker:
    """Mirror of CCanonicityChecker<uchar,uchar> for rank-2 incidence matrices.

    TestCanonicity(nRowMax, matrix, outInfo) follows
    Source/CanonicityChecker.h:255: it returns True for a canonical (partial)
    matrix; afterwards permRow() is the first rejecting row permutation,
    rowToChange() the backjump row (t_saveRowToChange), groupOrder() |Aut| and
    permStorage() the automorphisms found (column-orbit permutations for partial
    matrices, CPermutStorage layout with slot 0 the identity).
    """

    def __init__(self, nRow, nCol, ctx=None, save_automorphisms=False):
        if nRow > 16 or nCol > 63:
            raise CanonError(CANON_EINVAL, "this engine handles v <= 16 rows and b <= 63 columns")
        self.nRow, self.nCol = nRow, nCol
        self.ctx = ctx or Context(max_items=1024)
        self.save = save_automorphisms
        self._last = None

    def TestCanonicity(self, nRowMax, matrix, outInfo=t_saveNothing, raw=False):
        M = np.asarray(matrix, dtype=np.uint8)[:nRowMax, :self.nCol]
        rows = pack_rows(M)
        flags = (COMPLETE if outInfo & t_saveRowPermutations else 0) | (RAW if raw else 0)
        flags |= SAVE_AUTS if self.save else 0
        self.ctx.submit_bibd(rows, nRowMax, self.nCol, flags)
        r = self.ctx.sync()
        if r["status"][0] & ST_BADINPUT:
            raise CanonError(CANON_EINVAL, "matrix is not in column-orbit normal form")
        self._last = (nRowMax, r)
        return bool(r["canonical"][0])

    def permRow(self):
        n, r = self._last
        return r["witness"][0][:n].copy()

    def rowToChange(self):
        return int(self._last[1]["row_to_change"][0])

    def groupOrder(self):
        return self._last[1]["aut"][0]

    def permStorage(self):
        n, r = self._last
        k, ln = int(r["n_auts"][0]), int(r["len_aut"][0])
        return r["auts_raw"][0][:k, :ln].copy()

    def CanonizeMatrix(self, matrix):
        M = np.asarray(matrix, dtype=np.uint8)
        rows, aut = self.ctx.canonize_bibd(pack_rows(M), M.shape[0], M.shape[1])
        return unpack_rows(rows[0], M.shape[1]), aut[0]


class KSysChecker:
    """Mirror of alldata::cnvCheckNew(0, nrows) for group size 2 (k-Factorization)."""

    def __init__(self, numPlayers, ctx=None, save_automorphisms=False):
        self.np = numPlayers
        self.ctx = ctx or Context(max_items=1024)
        self.save = save_automorphisms
        self._last = None

    def cnvCheckNew(self, iMode, nrows, result):
        R = np.asarray(result, dtype=np.uint8)[:nrows]
        self.ctx.submit_ksys(R, self.np, nrows, SAVE_AUTS if self.save else 0)
        r = self.ctx.sync()
        if r["status"][0] & ST_BADINPUT:
            raise CanonError(CANON_EINVAL, "rounds are not in the sorted result() form")
        self._last = r
        return bool(r["canonical"][0])

    def playerIndex(self):
        return int(self._last["player_index"][0])

    def orderOfGroup(self):
        return self._last["aut"][0]

    def groupInfo(self):
        r = self._last
        k = int(r["n_auts"][0])
        return r["auts_raw"][0][:k, :self.np].copy()
