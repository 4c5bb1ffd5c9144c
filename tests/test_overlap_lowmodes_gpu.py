"""Overlap with low-mode projection and the options of the outer solve.

At M5 = -1 and beta = 1.4 the Wilson operator has near-zero modes, so the
Zolotarev range [lambda_min, lambda_max] of |H_W| starts very low (k ~ 2e-4
at n=32): 20 poles then approximate sign(H) only to ~1e-8 and the smallest
pole systems have condition ~3e7.  The projection treats the nev lowest
eigenmodes of H = gamma5 D_W exactly.  Checked here against the dense FP64
eigendecomposition of H at n=8 (the configuration carries topological charge
Q = 2, so the overlap has two exact zero modes), and the outer
D_ov^dag D_ov solve against a dense least-squares solution.  The massless
D_ov^dag D_ov is singular there (exact zero modes) and, at strong coupling,
has near-zero modes that make the outer CG ill-conditioned; the massive
overlap D(m) = (1 - m/2) D_ov + m is checked against dense D(m) at n=8 and
its outer solve certified at 1e-10 at n=32 (the benchmark's overlap
configuration).
"""
import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O
from tests.gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu


def _dense_overlap(n, seed):
    g = O.geometry(n)
    A, _ = O.thermalized_links(g, 1.4, seed, 50, init="uniform")
    Do = O.Dirac(g, 1.0, -1.0)
    Do.update(A)
    M = Do.dense()
    N = M.shape[0]
    g5 = np.tile([1.0, -1.0], N // 2)
    w, V = np.linalg.eigh(g5[:, None] * M)
    eps = (V * np.sign(w)) @ V.conj().T
    return g, A, np.eye(N) + g5[:, None] * eps, w


@pytest.fixture(scope="module")
def n8():
    return _dense_overlap(8, 2)


def _charge(g, A):
    th = O.plaquettes(g, A)
    return ((th + np.pi) % (2 * np.pi) - np.pi).sum() / (2 * np.pi)


def test_projected_sign_function_matches_dense(cuda, n8):
    g, A, Dex, w = n8
    assert abs(_charge(g, A) - 2.0) < 1e-9
    lat = Q.S2Trivalent(8)
    D = Q.DiracS2Dual(lat, 1.0, -1.0)
    D.update(A)
    ov = Q.Overlap(D, order=41)
    ov.update_lanczos()
    k0 = ov.info()["k"]
    info = ov.project_low_modes(16)
    assert info["nev"] == 16 and info["max_residual"] < 1e-9
    # the projected modes are the 16 eigenvalues of H = gamma5 D / lambda_max nearest zero
    lmax = info["lambda_max"]
    ref = np.sort(w[np.argsort(np.abs(w))[:16]]) / lmax
    assert np.abs(np.sort(info["mu"]) - ref).max() < 1e-10
    assert info["k"] > 5 * k0  # the Zolotarev range now starts above them
    rng = np.random.default_rng(3)
    xi = rng.normal(size=Dex.shape[0]) + 1j * rng.normal(size=Dex.shape[0])
    xt = to_dev(xi, cuda)
    import torch
    yt = torch.empty_like(xt)
    for op, M in ((Q.OP_D, Dex), (Q.OP_DDAG, Dex.conj().T), (Q.OP_DDAGD, Dex + Dex.conj().T)):
        ov.apply(yt, xt, op, tol_inner=1e-12)
        ref = M @ xi
        assert np.abs(from_dev(yt) - ref).max() / np.abs(ref).max() < 1e-9, op
    # switched off: back to the unprojected range
    assert ov.project_low_modes(0)["k"] == pytest.approx(k0, rel=1e-12)


@pytest.mark.parametrize("flags", [0, Q.OVSOLVE_CHIRAL])
def test_projected_outer_solve_matches_dense(cuda, n8, flags):
    g, A, Dex, _ = n8
    lat = Q.S2Trivalent(8)
    D = Q.DiracS2Dual(lat, 1.0, -1.0)
    D.update(A)
    ov = Q.Overlap(D, order=41)
    ov.update_lanczos()
    ov.project_low_modes(16)
    rng = np.random.default_rng(5)
    xi = rng.normal(size=Dex.shape[0]) + 1j * rng.normal(size=Dex.shape[0])
    b = Dex.conj().T @ xi  # the propagator's right-hand side: in the range despite the two zero modes
    bt = to_dev(b, cuda)
    x = bt.clone() * 0
    rep = ov.solve(x, bt, tol=1e-10, tol_inner=1e-12, maxiter=5000, flags=flags)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    A_ = Dex + Dex.conj().T
    xd = np.linalg.lstsq(A_, b, rcond=None)[0]  # the minimum-norm solution (no zero-mode part)
    assert np.linalg.norm(from_dev(x) - xd) / np.linalg.norm(xd) < 1e-6
    assert np.linalg.norm(A_ @ from_dev(x) - b) / np.linalg.norm(b) < 1e-9


@pytest.mark.parametrize("flags", [0, Q.OVSOLVE_CHIRAL])
def test_massive_outer_solve_matches_dense(cuda, n8, flags):
    """D(m) = (1 - m/2) D_ov + m: the outer solve of D(m)^dag D(m) x = D(m)^dag xi
    gives x = D(m)^{-1} xi (nonsingular for m > 0, zero modes or not)."""
    g, A, Dex, _ = n8
    m = 0.05
    lat = Q.S2Trivalent(8)
    D = Q.DiracS2Dual(lat, 1.0, -1.0)
    D.update(A)
    ov = Q.Overlap(D, order=41)
    ov.update_lanczos()
    ov.project_low_modes(16)
    ov.set_mass(m)
    Dm = (1 - m / 2) * Dex + m * np.eye(Dex.shape[0])
    rng = np.random.default_rng(6)
    xi = rng.normal(size=Dex.shape[0]) + 1j * rng.normal(size=Dex.shape[0])
    import torch
    xt = to_dev(xi, cuda)
    y = torch.empty_like(xt)
    for op, M in ((Q.OP_D, Dm), (Q.OP_DDAG, Dm.conj().T), (Q.OP_DDAGD, Dm.conj().T @ Dm)):
        ov.apply(y, xt, op, tol_inner=1e-12)
        ref = M @ xi
        assert np.abs(from_dev(y) - ref).max() / np.abs(ref).max() < 1e-9, op
    b = torch.empty_like(xt)
    ov.apply(b, xt, Q.OP_DDAG, tol_inner=1e-12)
    x = torch.zeros_like(b)
    rep = ov.solve(x, b, tol=1e-10, tol_inner=1e-12, maxiter=5000, flags=flags)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    xd = np.linalg.solve(Dm, xi)
    assert np.linalg.norm(from_dev(x) - xd) / np.linalg.norm(xd) < 1e-8


def test_force_refuses_projection(cuda, n8):
    g, A, _, _ = n8
    lat = Q.S2Trivalent(8)
    D = Q.DiracS2Dual(lat, 1.0, -1.0)
    D.update(A)
    ov = Q.Overlap(D, order=21)
    ov.update_lanczos()
    ov.project_low_modes(4)
    import torch
    eta = torch.ones(2 * lat.n_sites, dtype=torch.complex128, device=cuda)
    F = torch.zeros(lat.n_links, dtype=torch.float64, device=cuda)
    with pytest.raises(Q.Qed3Error):
        ov.force(F, eta)
    ov.project_low_modes(0)
    ov.force(F, eta)


def test_overlap_n32_outer_solve_certified(cuda):
    """The benchmark's overlap configuration: n=32, beta=1.4 (topological
    charge 17), M5=-1, 20 poles with the 48 lowest modes of gamma5 D_W
    projected, outer solve of the massive overlap (m = 0.05) per chirality
    sector, certified at 1e-10."""
    import torch
    lat = Q.S2Trivalent(32)
    A, _ = Q.thermalized_links(lat, 1.4, seed=2, ntraj=50, init="uniform", device=cuda)
    D = Q.DiracS2Dual(lat, 1.0, -1.0)
    D.update(A)
    ov = Q.Overlap(D, order=41)
    ov.update_lanczos()
    k0 = ov.info()["k"]
    info = ov.project_low_modes(48)
    assert info["k"] > 10 * k0 and info["max_residual"] < 1e-9
    ov.set_mass(0.05)
    xi = torch.from_numpy(Q.ParallelRng(lat, 5).gaussian_spinor()).to(cuda)
    b = torch.empty_like(xi)
    ov.apply(b, xi, Q.OP_DDAG, tol_inner=1e-12)
    x = torch.zeros_like(b)
    rep = ov.solve(x, b, tol=1e-10, tol_inner=1e-12, maxiter=6000, flags=Q.OVSOLVE_CHIRAL)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    q = torch.empty_like(b)
    ov.apply(q, x, Q.OP_DDAGD, tol_inner=1e-12)
    assert float((b - q).norm() / b.norm()) <= 1.05e-10
