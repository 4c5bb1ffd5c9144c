"""Overlap operator (Overlap, src/both_3d/overlap.h:137-390) on the GPU.

* against the oracle's restatement (CG per pole) with the same spectral bounds;
* the device estimate of (lambda_min, lambda_max) against the oracle's
  restatement of compute_lambda_max (same algorithm);
* the sign function at n=8 against an FP64 dense eigendecomposition: D_ov - 1
  = X (X^dag X)^{-1/2} up to the Zolotarev error Delta and the pole tolerance;
* the Ginsparg-Wilson relation g5 D + D g5 = D g5 D to the same accuracy.
"""
import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O
from tests.gpu_util import from_dev, rand_spinor, rel, to_dev

pytestmark = pytest.mark.gpu


def _setup(n, M5, seed):
    rng = np.random.default_rng(seed)
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = rng.normal(size=g.n_links) * 0.4
    Do = O.Dirac(g, 1.0, M5)
    Do.update(A)
    Dq = Q.DiracS2Dual(lat, 1.0, M5)
    Dq.update(A)
    return rng, g, lat, Do, Dq


@pytest.mark.parametrize("n,order", [(2, 21), (4, 31)])
def test_overlap_matches_oracle(cuda, n, order):
    rng, g, lat, Do, Dq = _setup(n, -1.0, 60 + n)
    lmin, lmax = Do.lambda_bounds()
    ov = Q.Overlap(Dq, order, Q.PREC_F32)
    info = ov.update(lmin, lmax)
    assert info["npoles"] == order // 2
    v = rand_spinor(rng, g.n_sites)
    vt = to_dev(v, cuda)
    for op, oop in ((Q.OP_D, 0), (Q.OP_DDAG, 1), (Q.OP_DDAGD, 2)):
        out = vt.clone() * 0
        rep = ov.apply(out, vt, op, tol_inner=1e-11)
        assert rep.status == Q.OK and rep.true_rel_res <= 1e-11
        ref = Do.overlap(v, lmin, lmax, order, oop, tol_inner=1e-12)
        assert rel(from_dev(out), ref) < 1e-8, (op, rel(from_dev(out), ref))


def test_lambda_estimate_matches_oracle(cuda):
    rng, g, lat, Do, Dq = _setup(2, -1.0, 70)
    lmin, lmax = Do.lambda_bounds(tol_outer=1e-10)
    ov = Q.Overlap(Dq, 21, Q.PREC_F32)
    info = ov.update(tol_outer=1e-10)
    assert abs(info["lambda_max"] / lmax - 1) < 1e-6
    assert abs(info["lambda_min"] / lmin - 1) < 1e-5
    assert abs(info["k"] - lmin / lmax) < 1e-5


def test_sign_function_against_dense_eigh_n8(cuda):
    # benchmark spec: sign-function error checked against FP64 dense eigh at n=8
    rng, g, lat, Do, Dq = _setup(8, -1.0, 71)
    M = Do.dense()
    ev = np.linalg.eigvalsh(M.conj().T @ M)
    lmin, lmax = np.sqrt(ev.min()) * 0.999, np.sqrt(ev.max()) * 1.001
    order = 41
    ov = Q.Overlap(Dq, order, Q.PREC_F32)
    info = ov.update(lmin, lmax)
    X = M / lmax
    w, U = np.linalg.eigh(X.conj().T @ X)
    V = X @ (U @ np.diag(w ** -0.5) @ U.conj().T)  # exact X (X^dag X)^{-1/2}
    g5 = np.tile([1.0, -1.0], g.n_sites)
    for _ in range(2):
        v = rand_spinor(rng, g.n_sites)
        vt = to_dev(v, cuda)
        out = vt.clone() * 0
        rep = ov.apply(out, vt, Q.OP_D, tol_inner=1e-12)
        assert rep.status == Q.OK
        Vv = from_dev(out) - v
        err = np.linalg.norm(Vv - V @ v) / np.linalg.norm(v)
        assert err < 10 * max(info["delta"], 1e-11), (err, info["delta"])
        # sign(H_W) = g5 V for H_W = g5 X: g5 V is hermitian and squares to 1
        sv = g5 * Vv
        assert abs(np.linalg.norm(sv) / np.linalg.norm(v) - 1) < 1e-8


def test_ginsparg_wilson_relation(cuda):
    rng, g, lat, Do, Dq = _setup(4, -1.0, 72)
    lmin, lmax = Do.lambda_bounds()
    ov = Q.Overlap(Dq, 41, Q.PREC_F32)
    info = ov.update(lmin, lmax)
    v = rand_spinor(rng, g.n_sites)
    g5 = np.tile([1.0, -1.0], g.n_sites)

    def D(x):
        xt = to_dev(x, cuda)
        out = xt.clone() * 0
        ov.apply(out, xt, Q.OP_D, tol_inner=1e-12)
        return from_dev(out)

    lhs = g5 * D(v) + D(g5 * v)
    rhs = D(g5 * D(v))
    assert np.linalg.norm(lhs - rhs) / np.linalg.norm(v) < 1e-8 + 10 * info["delta"]


@pytest.mark.parametrize("n,order", [(2, 21), (4, 21)])
def test_overlap_force_matches_oracle(cuda, n, order):
    """All-links overlap force against the oracle's per-link restatement of
    Overlap::grad_deviceAsyncLaunch (src/both_3d/overlap.h:418-470)."""
    import torch
    rng = np.random.default_rng(80 + n)
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = rng.normal(size=g.n_links) * 0.4
    Do = O.Dirac(g, 1.0, -1.0)
    Do.update(A)
    Dq = Q.DiracS2Dual(lat, 1.0, -1.0)
    Dq.update(A)
    lmin, lmax = Do.lambda_bounds()
    eta = rand_spinor(rng, g.n_sites)
    F_ref = Do.overlap_force(A, eta, lmin, lmax, order, tol_inner=1e-13)
    ov = Q.Overlap(Dq, order, Q.PREC_F32)
    ov.update(lmin, lmax)
    F = torch.zeros(g.n_links, dtype=torch.float64, device=cuda)
    rep = ov.force(F, to_dev(eta, cuda), tol_inner=1e-12)
    assert rep.status == Q.OK
    assert rel(from_dev(F), F_ref) < 1e-8


def test_overlap_outer_solve_n8(cuda):
    """Outer CG on D_ov^dag D_ov to 1e-10 with b = D_ov^dag xi (in the range of the
    operator, as the reference's propagator driver builds it); the solution's
    residual is re-checked with the oracle's overlap restatement."""
    rng, g, lat, Do, Dq = _setup(8, -1.0, 90)
    lmin, lmax = Do.lambda_bounds()
    ov = Q.Overlap(Dq, 41, Q.PREC_F32)  # 20 poles
    ov.update(lmin, lmax)
    xi = to_dev(rand_spinor(rng, g.n_sites), cuda)
    b = xi.clone()
    ov.apply(b, xi, Q.OP_DDAG, tol_inner=1e-12)
    x = b.clone() * 0
    rep = ov.solve(x, b, tol=1e-10, tol_inner=1e-12)
    assert rep.status == Q.OK
    assert rep.true_rel_res <= 1.5e-10
    xh, bh = from_dev(x), from_dev(b)
    r = bh - Do.overlap(xh, lmin, lmax, 41, op=2, tol_inner=1e-13)
    assert np.linalg.norm(r) / np.linalg.norm(bh) < 1e-9


def test_ill_conditioned_poles_run_in_fp64(cuda):
    """A small lambda_min/lambda_max puts the leading (smallest-shift) poles
    beyond what mixed-precision inner iterations resolve; they move to a second,
    FP64, batched launch and the operator still matches the oracle (to
    kappa x tol_inner: the leading poles' condition is ~1e7 here)."""
    rng, g, lat, Do, Dq = _setup(8, -1.0, 93)
    lmin, lmax = Do.lambda_bounds()
    lmin = lmax * 2e-4  # shifts down to ~1e-8 lmax^2: kappa of the first poles > 2e5
    ov = Q.Overlap(Dq, 41, Q.PREC_F32)
    info = ov.update(lmin, lmax)
    assert 0 < info["npoles_fp64"] < info["npoles"]
    xi = rand_spinor(rng, g.n_sites)
    out = to_dev(np.zeros_like(xi), cuda)
    rep = ov.apply(out, to_dev(xi, cuda), Q.OP_D, tol_inner=1e-12)
    assert rep.status == Q.OK
    ref = Do.overlap(xi, lmin, lmax, 41, op=0, tol_inner=1e-13)
    assert rel(from_dev(out), ref) < 1e-8
    # FP64 overlap: one launch, nothing split off
    ov64 = Q.Overlap(Dq, 41, Q.PREC_F64)
    assert ov64.update(lmin, lmax)["npoles_fp64"] == 0


@pytest.mark.parametrize("integrator", [Q.INTEGRATOR_LEAPFROG_ML, Q.INTEGRATOR_LEAPFROG])
def test_overlap_hmc_matches_oracle(cuda, integrator):
    """Overlap-fermion HMC (HMC2::run with Overlap fermions, fixed spectral
    bounds) against the oracle's composition of its overlap pieces from the
    same RNG streams: same Metropolis decisions, dH and links."""
    n = 2
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    ro, rq = O.Rng(g, 21), Q.ParallelRng(lat, 21)
    A0 = ro.gaussian_links(0.2)
    assert np.array_equal(A0, rq.gaussian_links(0.2))
    Do = O.Dirac(g, 1.0, -1.0)
    Do.update(A0)
    lmin, lmax = Do.lambda_bounds()
    Dq = Q.DiracS2Dual(lat, 1.0, -1.0)
    Dq.update(to_dev(A0, cuda))
    ov = Q.Overlap(Dq, 21, Q.PREC_F64)
    ov.update(lmin, lmax)
    Ao = np.ascontiguousarray(A0.copy())
    At = to_dev(A0, cuda)
    for it in range(2):
        acc_o, dh_o, its_o = O.hmc_overlap(g, Do, ro, Ao, 1.4, tmax=0.5, nsteps=4, nsteps_inner=4, lmin=lmin,
                                           lmax=lmax, order=21, tol=1e-11, tol_inner=1e-13, integrator=integrator)
        acc_q, dh_q, its_q = Q.hmc_overlap(lat, ov, rq, At, 1.4, tmax=0.5, nsteps=4, nsteps_inner=4,
                                           lambda_min=lmin, lambda_max=lmax, tol=1e-11, tol_inner=1e-13,
                                           integrator=integrator)
        assert acc_o == acc_q and its_q > 0
        assert abs(dh_o - dh_q) < 1e-7, (dh_o, dh_q)
        assert np.abs(from_dev(At) - Ao).max() < 1e-9


def test_overlap_hmc_dH_scales_as_tau_squared(cuda):
    """dH ~ tau^2 for the overlap trajectory (fixed bounds; RMS over four draws)."""
    n = 2
    lat = Q.S2Trivalent(n)
    A0 = Q.ParallelRng(lat, 22).gaussian_links(0.2)
    Dq = Q.DiracS2Dual(lat, 1.0, -1.0)
    Dq.update(to_dev(A0, cuda))
    ov = Q.Overlap(Dq, 21, Q.PREC_F32)
    info = ov.update()
    rms = []
    for ns in (16, 32):
        v = []
        for seed in range(23, 27):
            At = to_dev(A0, cuda)
            _, d, _ = Q.hmc_overlap(lat, ov, Q.ParallelRng(lat, seed), At, 1.4, tmax=0.5, nsteps=ns, nsteps_inner=2,
                                    lambda_min=info["lambda_min"], lambda_max=info["lambda_max"], tol=1e-11,
                                    tol_inner=1e-12, no_reject=True)
            v.append(d)
        rms.append(np.sqrt(np.mean(np.square(v))))
    assert 2.8 < rms[0] / rms[1] < 5.5, rms


def test_overlap_hmc_recomputed_bounds(cuda):
    """lambda_min = lambda_max = 0: every operator update re-estimates the
    bounds (Overlap::update); after the trajectory the overlap holds the
    bounds of the final links."""
    n = 2
    lat = Q.S2Trivalent(n)
    A0 = Q.ParallelRng(lat, 24).gaussian_links(0.2)
    At = to_dev(A0, cuda)
    Dq = Q.DiracS2Dual(lat, 1.0, -1.0)
    Dq.update(At)
    ov = Q.Overlap(Dq, 21, Q.PREC_F32)
    ov.update()
    acc, d, its = Q.hmc_overlap(lat, ov, Q.ParallelRng(lat, 25), At, 1.4, tmax=0.25, nsteps=4, nsteps_inner=2,
                                tol=1e-10, tol_inner=1e-12, no_reject=True)
    assert acc and np.isfinite(d) and abs(d) < 0.5 and its > 0
    before = ov.info()
    Dq.update(At)
    after = ov.update(tol_outer=1e-12)
    assert abs(before["lambda_max"] / after["lambda_max"] - 1) < 1e-6
    assert abs(before["lambda_min"] / after["lambda_min"] - 1) < 1e-4


@pytest.mark.parametrize("M5", [0.1, -1.0])
def test_lanczos_spectral_bounds_against_dense(cuda, M5):
    """Device Lanczos on D^dag D (no solves): the extremal eigenvalues of a
    dense FP64 eigendecomposition at n=4 to 1e-9, approached from inside, and
    bounds that enclose the power-iteration estimate's range."""
    rng, g, lat, Do, Dq = _setup(4, M5, 80)
    w = np.linalg.eigvalsh((lambda M: M.conj().T @ M)(Do.dense()))
    lo, hi, steps, ok = Dq.spectral_bounds(tol=1e-12)
    assert ok and steps < 5000
    assert lo >= w[0] * (1 - 1e-12) and hi <= w[-1] * (1 + 1e-12)
    assert abs(lo / w[0] - 1) < 1e-9 and abs(hi / w[-1] - 1) < 1e-9
    ov = Q.Overlap(Dq, 21, Q.PREC_F32)
    info = ov.update_lanczos(tol=1e-12)
    assert info["lambda_min"] <= np.sqrt(w[0]) and info["lambda_max"] >= np.sqrt(w[-1])
