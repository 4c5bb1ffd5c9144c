"""The allocation-free CG entry point, qed3_cg_solve_noalloc.

It serves callers that cannot allocate device memory at solve time (memory
owned by another allocator or pool, multi-stream drivers that must not trigger
cudaFree's device-wide synchronisation).  Its scratch is a static
device array of the library shared by every call, so this test calls it twice
in a row through the C ABI -- the second call must not be disturbed by what
the first left in the array -- and compares each result with the regular
qed3_cg_solve on the same inputs, to the solver tolerance the other GPU tests
use.  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

import qed3_gb300 as Q

pytestmark = pytest.mark.gpu


def _solve(fn_name, d, x, b, prec):
    L = Q.lib()
    p = Q.SolveParams(1e-10, 100000, prec, 0.1, 0.0, 0)
    r = Q.SolveReport()
    rc = getattr(L, fn_name)(d.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(b.data_ptr()),
                             ctypes.byref(p), ctypes.byref(r), None)
    return rc, r


@pytest.mark.parametrize("prec", [Q.PREC_F64, Q.PREC_F32])
def test_noalloc_matches_regular_solve_twice(cuda, prec):
    import torch
    rng = np.random.default_rng(77)
    n = 32  # the largest lattice the static scratch holds
    lat = Q.S2Trivalent(n)
    D = Q.DiracS2Dual(lat, 1.0, 0.05)
    D.update(rng.uniform(-np.pi, np.pi, lat.n_links))
    for call in range(2):
        b = torch.from_numpy(rng.normal(size=2 * lat.n_sites) + 1j * rng.normal(size=2 * lat.n_sites)).to(cuda)
        x_ref = torch.zeros_like(b)
        x_na = torch.full_like(b, 7.0)  # garbage in the output must not matter
        rc1, r1 = _solve("qed3_cg_solve", D, x_ref, b, prec)
        rc2, r2 = _solve("qed3_cg_solve_noalloc", D, x_na, b, prec)
        torch.cuda.synchronize()
        assert rc1 == Q.OK and rc2 == Q.OK, (call, rc1, rc2, Q.lib().qed3_last_error_string())
        assert r2.status == Q.OK and r2.true_rel_res <= 1e-10
        assert abs(r2.iters - r1.iters) <= max(5, r1.iters // 10)
        xr, xn = x_ref.cpu().numpy(), x_na.cpu().numpy()
        assert np.linalg.norm(xn - xr) / np.linalg.norm(xr) < 1e-7, call
        # independent residual check through the apply entry point
        q = torch.empty_like(b)
        D.apply(q, x_na, Q.OP_DDAGD)
        assert float((b - q).norm() / b.norm()) <= 1.05e-10


def test_noalloc_rejects_oversized_lattice(cuda):
    import torch
    lat = Q.S2Trivalent(33)  # 21,780 sites > QED3_NOALLOC_MAX_SITES
    D = Q.DiracS2Dual(lat, 1.0, 0.1)
    D.update(np.zeros(lat.n_links))
    b = torch.ones(2 * lat.n_sites, dtype=torch.complex128, device=cuda)
    x = torch.zeros_like(b)
    rc, _ = _solve("qed3_cg_solve_noalloc", D, x, b, Q.PREC_F32)
    assert rc == Q.ERR_ARG
    assert b"at most 20480" in Q.lib().qed3_last_error_string()


def test_noalloc_allocates_no_device_memory(cuda):
    """A fresh operator handle that has never run the regular solve: after one
    warm-up call (which looks up the scratch array's address), a second call
    leaves the device's free memory unchanged."""
    import torch
    rng = np.random.default_rng(78)
    lat = Q.S2Trivalent(16)
    D = Q.DiracS2Dual(lat, 1.0, 0.1)
    D.update(rng.uniform(-np.pi, np.pi, lat.n_links))
    b = torch.from_numpy(rng.normal(size=2 * lat.n_sites) + 1j * rng.normal(size=2 * lat.n_sites)).to(cuda)
    x = torch.zeros_like(b)
    rc, r = _solve("qed3_cg_solve_noalloc", D, x, b, Q.PREC_F32)
    assert rc == Q.OK and r.status == Q.OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc, r = _solve("qed3_cg_solve_noalloc", D, x, b, Q.PREC_F32)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert rc == Q.OK and r.status == Q.OK and r.true_rel_res <= 1e-10
    assert free1 == free0, (free0, free1)
