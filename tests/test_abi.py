"""The C-ABI library loads and exports every entry point include/qed3.h declares."""
import os
import re
import subprocess

import qed3_gb300 as Q

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "qed3.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qed3_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    L = Q.lib()
    names = declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", Q.LIB_PATH], capture_output=True, text=True).stdout
    for n in names:
        assert re.search(r"\bT " + n + r"\b", out), n


def test_python_binding_covers_the_header():
    bound = {s[0] for s in Q.SIGNATURES}
    assert set(declared()) <= bound


def test_error_string_and_version():
    L = Q.lib()
    assert L.qed3_version() >= 100
    import ctypes
    h = ctypes.c_void_p()
    assert L.qed3_lattice_create(-3, ctypes.byref(h)) == Q.ERR_ARG
    assert b"n_refine" in L.qed3_last_error_string()
    assert L.qed3_lattice_destroy(None) == Q.OK
