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


def test_library_exports_the_reference_plugin():
    """createCanonizer / runCanonizer / releaseCanonizer, the reference's exported
    plugin (k-Factorization/Utils/Include/CDTools.h:9-11), are declared and exported
    under their own names."""
    conftest.build_native()
    import ise_gb300
    lib = ctypes.CDLL(ise_gb300.LIB_PATH)
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    for name in ise_gb300.PLUGIN_SYMBOLS:
        assert re.search(r"\b%s\s*\(" % name, src), name
        assert hasattr(lib, name), name
    # arguments the plugin refuses without touching a GPU
    lib = ise_gb300.load_library()
    assert not lib.createCanonizer(10, 3)          # group size 2 only
    assert not lib.createCanonizer(7, 2)           # v must be even
    assert not lib.runCanonizer(None, None, 2, 0)


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        return
    import ise_gb300
    lib = ise_gb300.load_library()
    cfg = ise_gb300.Cfg(0, 16, 0, 4, 0, 0)
    assert not lib.canon_create(ctypes.byref(cfg))


C_PROGRAM = r"""
#include <stdio.h>
#include "canon_gb300.h"
int main(void) {
    uint64_t aut[1] = {168};
    char buf[4096];
    size_t n = canon_report_bibd(7, 7, 3, 3, 1, 1, aut, NULL, NULL, 1, 0.0, buf, sizeof buf);
    if (n == 0 || n >= sizeof buf)
        return 1;
    fputs(buf, stdout);
    return 0;
}
"""

CPP_PROGRAM = r"""
#include <cstdio>
#include "canon_gb300.hpp"
int main() {
    const unsigned char fano[7 * 7] = {1,1,1,0,0,0,0, 1,0,0,1,1,0,0, 1,0,0,0,0,1,1, 0,1,0,1,0,1,0,
                                       0,1,0,0,1,0,1, 0,0,1,1,0,0,1, 0,0,1,0,1,1,0};
    auto rows = canon_gb300::packRows(fano, 7, 7);
    if (rows.size() != 7 || rows[0] != 7u)
        return 2;
    try {
        canon_gb300::Context ctx(0, 16);
        std::puts("device");
    } catch (const canon_gb300::Error &e) {
        std::puts("no device");          // a machine without a GPU: the adapter reports it
    }
    return 0;
}
"""


def test_headers_compile_and_link_from_c_and_cpp(tmp_path):
    """include/canon_gb300.h is plain C99 and include/canon_gb300.hpp plain C++17: a
    caller outside this repository builds against them and the library alone."""
    import subprocess
    conftest.build_native()
    import ise_gb300
    libdir = os.path.dirname(ise_gb300.LIB_PATH)
    inc = os.path.join(conftest.REPO, "include")
    (tmp_path / "use.c").write_text(C_PROGRAM)
    (tmp_path / "use.cpp").write_text(CPP_PROGRAM)
    link = ["-L", libdir, "-lcanon_gb300", "-Wl,-rpath," + libdir]
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", inc, str(tmp_path / "use.c"), "-o",
                    str(tmp_path / "use_c")] + link, check=True)
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", inc, str(tmp_path / "use.cpp"), "-o",
                    str(tmp_path / "use_cpp")] + link, check=True)
    out_c = subprocess.run([str(tmp_path / "use_c")], capture_output=True, text=True, check=True).stdout
    assert out_c.startswith("BIBD(  7,   7,  3,  3,  1)") and "168" in out_c
    out_cpp = subprocess.run([str(tmp_path / "use_cpp")], capture_output=True, text=True, check=True).stdout
    assert out_cpp.strip() in ("device", "no device")
