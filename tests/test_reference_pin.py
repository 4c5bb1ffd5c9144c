"""The oracle's operator and CG against the reference's own code built in place.

tests/golden/dirac_ref.npz holds what the reference's operator pipeline
computes when compiled from its headers (oracle/ref_dirac.cu, made by
`make -C oracle ref`, fixture written by tests/golden/make_golden.py): the
lattice read from .dat tables by S2Simp / S2Trivalent
(src/both_3d/s2n_simp.h:43-402, src/both_3d/s2n_dual.h:49-166), the spin
structure and kappa of DiracS2Dual (src/both_3d/dirac_dual.h:15-215), the
coefficients of DiracExt::coo_format (src/both_3d/dirac_ext.h:122-213), the
CSR of DWDevice (src/both_3d/sparse_dirac.h:52-151), products by the host
SpMV `matmul` (src/both_3d/sparse_matrix.h:257-270), and MatPoly::solve's CG
iteration (src/both_3d/matpoly.h:204-267) over that SpMV.  These tests run
without a GPU; tests/test_reference_pin_gpu.py holds the GPU operator to the
same fixture.
"""
import ctypes
import os
import tempfile

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
FIX = os.path.join(HERE, "golden", "dirac_ref.npz")
CASES = ["n2_t1", "n4_t1", "n8_t1", "n2_t2", "n4_t4"]


def _case(f, key):
    n, Nt = int(key[1]), int(key.split("_t")[1])
    r, M5, at = f[key + "/params"]
    return n, Nt, float(r), float(M5), float(at)


@pytest.fixture(scope="module")
def fix():
    return np.load(FIX)


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("key", ["n2_t1", "n4_t1", "n8_t1"])
def test_oracle_operator_matches_reference_build(fix, key):
    n, Nt, r, M5, at = _case(fix, key)
    g = O.geometry(n)
    D = O.Dirac(g, r, M5)
    D.update(np.ascontiguousarray(fix[key + "/A"][:g.n_links]))
    v = fix[key + "/v"]
    for op, name in ((0, "Dv"), (1, "DHv"), (2, "DHDv")):
        if key + "/" + name in fix:
            assert _rel(D.apply(v, op), fix[key + "/" + name]) < 1e-14, (key, name)
    assert np.array_equal(D.kappa(), fix[key + "/kappa"])


def test_oracle_csr_is_the_references(fix):
    """DWDevice's CSR of D at n=2: identical row pointers and columns, values to rounding."""
    g = O.geometry(2)
    D = O.Dirac(g, 1.0, 0.1)
    D.update(np.ascontiguousarray(fix["n2_t1/A"][:g.n_links]))
    L = O.lib()
    nnz = L.orc_dirac_nnz(D.h)
    rows = np.zeros(2 * g.n_sites + 1, np.int32)
    cols = np.zeros(nnz, np.int32)
    val = np.zeros(nnz, np.complex128)
    c_int_p = ctypes.POINTER(ctypes.c_int)
    L.orc_dirac_get_csr(D.h, rows.ctypes.data_as(c_int_p), cols.ctypes.data_as(c_int_p),
                        val.ctypes.data_as(ctypes.c_void_p))
    assert nnz == fix["n2_t1/csr_cols"].size
    assert np.array_equal(rows, fix["n2_t1/csr_rows"])
    assert np.array_equal(cols, fix["n2_t1/csr_cols"])
    assert np.abs(val - fix["n2_t1/csr_val"]).max() < 1e-15 * np.abs(val).max()


@pytest.mark.parametrize("key", ["n2_t1", "n4_t1", "n8_t1"])
def test_oracle_cg_follows_reference_iterates(fix, key):
    n, Nt, r, M5, at = _case(fix, key)
    g = O.geometry(n)
    D = O.Dirac(g, r, M5)
    D.update(np.ascontiguousarray(fix[key + "/A"][:g.n_links]))
    v = fix[key + "/v"]
    x, it, _ = D.cg(v, tol=1e-10)
    assert it == int(fix[key + "/cg_iters"][0])
    assert np.linalg.norm(x - fix[key + "/x_final"]) / np.linalg.norm(x) < 1e-11
    if key + "/iters_at" in fix:
        for k, xk in zip(fix[key + "/iters_at"], fix[key + "/x_at"]):
            x, _, _ = D.cg(v, tol=1e-30, maxiter=int(k))
            assert np.linalg.norm(x - xk) / np.linalg.norm(xk) < 1e-13, (key, k)


@pytest.mark.parametrize("key", ["n2_t2", "n4_t4"])
def test_oracle_ext_operator_matches_reference_build(fix, key):
    n, Nt, r, M5, at = _case(fix, key)
    g = O.geometry(n)
    A, v = fix[key + "/A"], fix[key + "/v"]
    for op, name in ((0, "Dv"), (1, "DHv"), (2, "DHDv")):
        if key + "/" + name in fix:
            assert _rel(O.dirac_ext_apply(g, r, M5, Nt, at, A, v, op), fix[key + "/" + name]) < 1e-14, (key, name)


def _ref_lib(n, Nt):
    p = os.path.join(ROOT, "oracle", "_ref", f"libdirac_ref_n{n}_t{Nt}.so")
    return ctypes.CDLL(p) if os.path.exists(p) else None


@pytest.mark.parametrize("key", ["n2_t1", "n4_t4"])
def test_reference_build_reproduces_fixture(fix, key):
    """Where the reference tree was built (oracle/_ref), rerun it: the fixture
    is what the reference computes on this project's lattice tables."""
    n, Nt, r, M5, at = _case(fix, key)
    L = _ref_lib(n, Nt)
    if L is None:
        pytest.skip("reference build absent (oracle/_ref is made only where the reference tree is present)")
    import qed3_gb300 as Q
    from qed3_gb300 import dats
    lat = Q.S2Trivalent(n)
    N = 2 * lat.n_sites * Nt
    A, v = fix[key + "/A"], fix[key + "/v"]
    Dv, DHv, DHDv, xf = (np.zeros(N, np.complex128) for _ in range(4))
    its = np.zeros(1, np.int32)
    xa = np.zeros((1, N), np.complex128)
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    with tempfile.TemporaryDirectory() as d:
        dats.write(lat, d)
        k = L.ref_dirac_run(d.encode(), ctypes.c_double(r), ctypes.c_double(M5), ctypes.c_double(at),
                            A.ctypes.data_as(dp), v.ctypes.data_as(dp), Dv.ctypes.data_as(dp), DHv.ctypes.data_as(dp),
                            DHDv.ctypes.data_as(dp), None, None, None, None, ctypes.c_double(1e-10), 100000, 0,
                            its.ctypes.data_as(ip), xa.ctypes.data_as(dp), xf.ctypes.data_as(dp))
    assert k == int(fix[key + "/cg_iters"][0])
    assert np.array_equal(DHDv, fix[key + "/DHDv"])
    assert np.array_equal(xf, fix[key + "/x_final"])
