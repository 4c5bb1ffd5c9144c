"""The benchmark's reference-GPU-algorithm baseline (oracle/ref_gpu_cg.cu)
against the reference's own CG iteration built in place.

The restated kernels (CSR SpMV one thread per row, axpy, cuBLAS dots) run the
reference's MatPoly::solve step for step; on the n=8 case of
tests/golden/dirac_ref.npz they must take the reference build's iteration
count and reach its solution, so the baseline the benchmark times is the
reference's algorithm."""
import ctypes
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_ref_gpu_cg_is_the_reference_iteration(cuda):
    f = np.load(os.path.join(HERE, "golden", "dirac_ref.npz"))
    key = "n8_t1/"
    r, M5, _ = f[key + "params"]
    g = O.geometry(8)
    D = O.Dirac(g, float(r), float(M5))
    D.update(np.ascontiguousarray(f[key + "A"][:g.n_links]))
    rows, cols, val = D.csr()
    rowsT, colsT, valH = D.csr(dagger=True)
    b = np.ascontiguousarray(f[key + "v"])
    x = np.zeros_like(b)
    ms = np.zeros(2)
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "librefgpu.so"))
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    it = L.refgpu_cg(ctypes.c_int(D.N), ctypes.c_int(cols.size), p(rows), p(cols), p(val), p(rowsT), p(colsT),
                     p(valH), p(b), p(x), ctypes.c_double(1e-10), ctypes.c_int(100000), ctypes.c_int(0),
                     ctypes.c_int(2), p(ms))
    assert it == int(f[key + "cg_iters"][0])
    xr = f[key + "x_final"]
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-9
    assert np.all(ms > 0)
