"""The GPU operator and FP64 CG against the reference's own code built in place.

The fixture tests/golden/dirac_ref.npz is what the reference computes --
S2Simp / S2Trivalent reading this project's lattice from .dat tables,
DiracS2Dual / DiracExt::coo_format (src/both_3d/dirac_dual.h:63-215,
src/both_3d/dirac_ext.h:122-213), DWDevice's CSR (src/both_3d/sparse_dirac.h)
and the host SpMV `matmul` (src/both_3d/sparse_matrix.h:257-270), plus
MatPoly::solve's CG iteration (src/both_3d/matpoly.h:204-267) over that SpMV
(see tests/golden/make_golden.py).  Here the same inputs go through the C ABI:
qed3_dirac_apply (D, D^dag, D^dag D) within 1e-13 of the reference's
products, qed3_cg_solve in FP64 reaching the reference's iterates after 1, 2,
5 and 20 iterations and its converged solution, and the S^2 x S^1 operator
(qed3_dirac_ext_apply, Nt = 2 and 4) within 1e-13.
"""
import os

import numpy as np
import pytest

import qed3_gb300 as Q
from tests.gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "dirac_ref.npz")


@pytest.fixture(scope="module")
def fix():
    return np.load(FIX)


def _case(f, key):
    n, Nt = int(key[1]), int(key.split("_t")[1])
    r, M5, at = f[key + "/params"]
    return n, Nt, float(r), float(M5), float(at)


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _operator(fix, key):
    n, Nt, r, M5, at = _case(fix, key)
    lat = Q.S2Trivalent(n)
    D = Q.DiracS2Dual(lat, r, M5)
    D.update(np.ascontiguousarray(fix[key + "/A"][:lat.n_links]))
    return D


@pytest.mark.parametrize("key", ["n2_t1", "n4_t1", "n8_t1"])
def test_apply_matches_reference_build(cuda, fix, key):
    import torch
    D = _operator(fix, key)
    v = to_dev(fix[key + "/v"], cuda)
    out = torch.empty_like(v)
    for op, name in ((Q.OP_D, "Dv"), (Q.OP_DDAG, "DHv"), (Q.OP_DDAGD, "DHDv")):
        if key + "/" + name not in fix:
            continue
        D.apply(out, v, op)
        torch.cuda.synchronize()
        assert _rel(from_dev(out), fix[key + "/" + name]) < 1e-13, (key, name)


@pytest.mark.parametrize("flags", [0, Q.SOLVE_STREAMING])
@pytest.mark.parametrize("key", ["n2_t1", "n4_t1"])
def test_cg_follows_reference_iterates(cuda, fix, key, flags):
    """FP64 CG stopped after k iterations is the reference iteration's x_k."""
    D = _operator(fix, key)
    b = to_dev(fix[key + "/v"], cuda)
    x = b.clone() * 0
    for k, xk in zip(fix[key + "/iters_at"], fix[key + "/x_at"]):
        rep = D.solve(x, b, tol=1e-30, maxiter=int(k), precision=Q.PREC_F64, flags=flags)
        assert rep.status == Q.ERR_NOCONV and rep.iters == int(k)
        err = np.linalg.norm(from_dev(x) - xk) / np.linalg.norm(xk)
        assert err < 1e-11, (key, int(k), err)


@pytest.mark.parametrize("flags", [0, Q.SOLVE_STREAMING])
@pytest.mark.parametrize("key", ["n2_t1", "n4_t1", "n8_t1"])
def test_cg_converges_to_reference_solution(cuda, fix, key, flags):
    D = _operator(fix, key)
    b = to_dev(fix[key + "/v"], cuda)
    x = b.clone() * 0
    rep = D.solve(x, b, tol=1e-10, precision=Q.PREC_F64, flags=flags)
    it_ref = int(fix[key + "/cg_iters"][0])
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    assert abs(rep.iters - it_ref) <= max(5, it_ref // 20), (rep.iters, it_ref)
    xr = fix[key + "/x_final"]
    assert np.linalg.norm(from_dev(x) - xr) / np.linalg.norm(xr) < 1e-7


@pytest.mark.parametrize("key", ["n2_t2", "n4_t4"])
def test_ext_apply_matches_reference_build(cuda, fix, key):
    import torch
    n, Nt, r, M5, at = _case(fix, key)
    lat = Q.S2Trivalent(n)
    De = Q.DiracExt(lat, r, M5, Nt, at)
    De.update(to_dev(fix[key + "/A"], cuda))
    v = to_dev(fix[key + "/v"], cuda)
    out = torch.empty_like(v)
    for op, name in ((Q.OP_D, "Dv"), (Q.OP_DDAG, "DHv"), (Q.OP_DDAGD, "DHDv")):
        if key + "/" + name not in fix:
            continue
        De.apply(out, v, op)
        torch.cuda.synchronize()
        assert _rel(from_dev(out), fix[key + "/" + name]) < 1e-13, (key, name)
    x = torch.zeros_like(v)
    rep = De.solve(x, v, tol=1e-10)
    xr = fix[key + "/x_final"]
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    assert np.linalg.norm(from_dev(x) - xr) / np.linalg.norm(xr) < 1e-7
