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


def _compile_and_run(tmp_path, compiler, std):
    exe = str(tmp_path / f"host_calls_{compiler}")
    src = os.path.join(ROOT, "tests", "c_abi", "host_calls.c")
    lang = ["-x", "c++"] if compiler == "g++" else []
    libdir = os.path.dirname(Q.LIB_PATH)
    cmd = [compiler, *lang, f"-std={std}", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I",
           os.path.join(ROOT, "include"), src, "-o", exe, "-L", libdir, "-lqed3", f"-Wl,-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")


def test_header_is_plain_c_and_c_plus_plus(tmp_path):
    """include/qed3.h compiles as strict C99 and as C++17, a C program links
    the library and its host-side calls agree with the Python binding."""
    import numpy as np
    Q.lib()
    for compiler, std in (("gcc", "c99"), ("g++", "c++17")):
        out = _compile_and_run(tmp_path, compiler, std)
        f = out[0].split()
        lat = Q.S2Trivalent(4)
        assert [int(v) for v in f[:4]] == [lat.n_sites, lat.n_links, lat.n_faces, lat.face_total]
        assert float(f[4]) == lat.tables()["ell"][0]
        assert int(f[5]) == Q.ERR_ARG
        z = Q.zolotarev(0.01, 21)
        assert int(f[6]) == z["size"] and float(f[7]) == z["C"]
        from oracle import oracle as O

        class Sizes:
            n_links, n_sites = 3, 1
        assert float(f[8]) == O.Rng(Sizes(), 7).gaussian_links(1.0)[0]
        assert out[1] == "message"
