"""The C-ABI library builds, loads and exports every symbol include/canon_gb300.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import conftest

HEADER = os.path.join(conftest.REPO, "include", "canon_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(canon_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_header_symbols():
    conftest.build_native()
    import ise_gb300
    lib = ctypes.CDLL(ise_gb300.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(ise_gb300.HEADER_SYMBOLS) == names


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        return
    import ise_gb300
    lib = ise_gb300.load_library()
    cfg = ise_gb300.Cfg(0, 16, 0, 4, 0)
    assert not lib.canon_create(ctypes.byref(cfg))
