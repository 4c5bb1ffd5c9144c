"""The C-ABI library loads and exports every entry point include/qed3.h declares."""
import os
import re
import subprocess

import pytest

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
        assert int(f[9]) == Q.ERR_ARG and int(f[10]) == Q.ERR_ARG  # batch argument checks
        assert out[1] == "message"


def test_rng_checkpoint_is_the_references(tmp_path):
    """A random-stream checkpoint written by the library after the same draws
    is byte-identical to the reference's ParallelRngExt::ckpoint file
    (tests/golden/rng_ckpoint_ref.txt), and loading the reference's file
    continues with the reference's draws."""
    import ctypes
    import json

    import numpy as np
    L = Q.lib()
    gold = json.load(open(os.path.join(ROOT, "tests", "golden", "rng_ckpoint_ref.json")))
    nl, ns, seed = gold["n_links"], gold["n_sites"], gold["seed"]
    cont = np.array([float.fromhex(s) for s in gold["continuation"]])

    def new(seed_):
        h = ctypes.c_void_p()
        assert L.qed3_rng_create(nl, ns, seed_, ctypes.byref(h)) == Q.OK
        return h

    def draws(h, nu, z2):
        links = np.zeros(nl)
        L.qed3_rng_gaussian_links(h, 1.0, links.ctypes.data_as(ctypes.c_void_p))
        sp = np.zeros(4 * ns)
        L.qed3_rng_gaussian_spinor(h, sp.ctypes.data_as(ctypes.c_void_p))
        out = [links, sp * np.sqrt(2.0)]
        u = ctypes.c_double()
        us = []
        for _ in range(nu):
            L.qed3_rng_uniform(h, ctypes.byref(u))
            us.append(u.value)
        out.append(np.array(us))
        if z2:
            zz = np.zeros(4 * ns)
            L.qed3_rng_z2_spinor(h, zz.ctypes.data_as(ctypes.c_void_p))
            out.append(np.rint(zz * np.sqrt(2.0 * ns)))
        return np.concatenate(out)

    h = new(seed)
    draws(h, 3, False)
    path = str(tmp_path / "ckpoint_rng")
    assert L.qed3_rng_save(h, path.encode()) == Q.OK
    assert open(path, "rb").read() == open(os.path.join(ROOT, "tests", "golden", "rng_ckpoint_ref.txt"), "rb").read()
    mine = draws(h, 2, True)
    h2 = new(seed + 1)
    assert L.qed3_rng_load(h2, os.path.join(ROOT, "tests", "golden", "rng_ckpoint_ref.txt").encode()) == Q.OK
    loaded = draws(h2, 2, True)
    k = nl + 4 * ns
    # the spinor draws are compared after undoing the 1/sqrt(2) scaling
    assert np.array_equal(mine[:nl], cont[:nl]) and np.array_equal(loaded[:nl], cont[:nl])
    assert np.allclose(mine[nl:k], cont[nl:k], rtol=0, atol=4e-16) and np.allclose(loaded[nl:k], cont[nl:k],
                                                                                 rtol=0, atol=4e-16)
    assert np.array_equal(mine[k:], cont[k:]) and np.array_equal(loaded[k:], cont[k:])
    for hh in (h, h2):
        L.qed3_rng_destroy(hh)
    bad = str(tmp_path / "short")
    open(bad, "w").write("1 2 3\n")
    h3 = new(1)
    assert L.qed3_rng_load(h3, bad.encode()) == Q.ERR_ARG
    L.qed3_rng_destroy(h3)


def test_gauge_checkpoint_layout(tmp_path):
    """GaugeExt::ckpoint layout at Nt = 1: n_links spatial doubles, then
    n_sites temporal doubles; load returns the spatial angles."""
    import numpy as np
    lat = Q.S2Trivalent(3)
    A = np.random.default_rng(4).uniform(-np.pi, np.pi, lat.n_links)
    p = str(tmp_path / "ckpoint_lat")
    Q.save_links(lat, A, p)
    raw = np.fromfile(p, dtype=np.float64)
    assert raw.size == lat.n_links + lat.n_sites
    assert np.array_equal(raw[:lat.n_links], A) and not raw[lat.n_links:].any()
    assert np.array_equal(Q.load_links(lat, p), A)
    with pytest.raises(Q.Qed3Error):
        Q.load_links(Q.S2Trivalent(2), p)
