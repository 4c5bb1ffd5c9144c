"""GPU CG solves (plain FP64 and mixed precision with FP64 reliable updates)
against the oracle's restatement of MatPoly::solve.

Every solve must be certified by the FP64 true residual
||b - D^dag D x|| / ||b|| <= tol (recomputed independently here through the
apply entry point); solutions agree with the oracle's within tol * cond."""
import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O
from tests.gpu_util import from_dev, rand_spinor, to_dev

pytestmark = pytest.mark.gpu


def _setup(n, M5, seed, cuda):
    rng = np.random.default_rng(seed)
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = rng.uniform(-np.pi, np.pi, g.n_links)
    Do = O.Dirac(g, 1.0, M5)
    Do.update(A)
    Dq = Q.DiracS2Dual(lat, 1.0, M5)
    Dq.update(A)
    b = rand_spinor(rng, g.n_sites)
    return g, lat, Do, Dq, b


def _true_res(Dq, x_t, b_t, shift=0.0):
    q = b_t.clone()
    Dq.apply(q, x_t, Q.OP_DDAGD)
    q = q + shift * x_t
    return float((b_t - q).norm() / b_t.norm())


@pytest.mark.parametrize("flags", [0, Q.SOLVE_STREAMING])
@pytest.mark.parametrize("prec", [Q.PREC_F64, Q.PREC_F32, Q.PREC_BF16])
def test_cg_matches_oracle_n8(cuda, prec, flags):
    g, lat, Do, Dq, b = _setup(8, 0.1, 21, cuda)
    x_ref, it_ref, _ = Do.cg(b, tol=1e-10)
    bt = to_dev(b, cuda)
    xt = bt.clone() * 0
    rep = Dq.solve(xt, bt, tol=1e-10, precision=prec, flags=flags)
    assert rep.status == Q.OK
    assert rep.true_rel_res <= 1e-10
    assert _true_res(Dq, xt, bt) <= 1.05e-10
    x = from_dev(xt)
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-7
    if prec == Q.PREC_F64:
        assert abs(rep.iters - it_ref) <= max(5, it_ref // 20)
    else:
        assert rep.reliable_updates >= 2


@pytest.mark.parametrize("flags", [0, Q.SOLVE_STREAMING])
@pytest.mark.parametrize("prec", [Q.PREC_F64, Q.PREC_F32, Q.PREC_BF16])
def test_cg_n64_certified(cuda, prec, flags):
    g, lat, Do, Dq, b = _setup(64, 0.05, 22, cuda)
    bt = to_dev(b, cuda)
    xt = bt.clone() * 0
    rep = Dq.solve(xt, bt, tol=1e-10, precision=prec, flags=flags)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    assert _true_res(Dq, xt, bt) <= 1.05e-10
    # the oracle's residual of the GPU solution (FP64 CSR operator)
    x = from_dev(xt)
    r = b - Do.apply(x, 2)
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.05e-10


@pytest.mark.parametrize("flags", [0, Q.SOLVE_STREAMING])
def test_cg_shifted(cuda, flags):
    g, lat, Do, Dq, b = _setup(8, 0.0, 23, cuda)
    bt = to_dev(b, cuda)
    xt = bt.clone() * 0
    rep = Dq.solve(xt, bt, tol=1e-11, precision=Q.PREC_F32, shift=0.37, flags=flags)
    assert rep.status == Q.OK
    x_ref, _, _ = Do.cg(b, tol=1e-12, shift=0.37)
    assert np.linalg.norm(from_dev(xt) - x_ref) / np.linalg.norm(x_ref) < 1e-9
    assert _true_res(Dq, xt, bt, 0.37) <= 1.1e-11


@pytest.mark.parametrize("flags", [0, Q.SOLVE_STREAMING])
def test_cg_zero_rhs_and_noconv(cuda, flags):
    g, lat, Do, Dq, b = _setup(4, 0.1, 24, cuda)
    import torch
    z = torch.zeros(2 * g.n_sites, dtype=torch.complex128, device=cuda)
    x = torch.ones_like(z)
    rep = Dq.solve(x, z, flags=flags)
    assert rep.status == Q.OK and rep.iters == 0 and float(x.abs().max()) == 0.0
    bt = to_dev(b, cuda)
    rep = Dq.solve(x, bt, tol=1e-14, maxiter=3, flags=flags)
    assert rep.status == Q.ERR_NOCONV and rep.iters == 3


@pytest.mark.parametrize("n", [4, 8])
def test_multishift_matches_oracle(cuda, n):
    """FP64 multi-shift CG (one Krylov space) against the oracle's CG per shift;
    every shift certified by its own FP64 true residual."""
    import torch
    g, lat, Do, Dq, b = _setup(n, 0.1, 40 + n, cuda)
    shifts = [0.0, 1e-3, 0.05, 0.7, 3.0]
    bt = to_dev(b, cuda)
    x = torch.zeros(len(shifts), bt.numel(), dtype=torch.complex128, device=cuda)
    reps, ms = Q.multishift_solve(Dq, x, bt, shifts, tol=1e-10)
    X = from_dev(x)
    for m, sg in enumerate(shifts):
        assert reps[m].status == Q.OK and reps[m].true_rel_res <= 1.05e-10
        x_ref, _, _ = Do.cg(b, tol=1e-12, shift=sg)
        assert np.linalg.norm(X[m] - x_ref) / np.linalg.norm(x_ref) < 1e-8
    # larger shifts converge (and stop) no later than the base shift
    its = [r.iters for r in reps]
    assert its == sorted(its, reverse=True)


@pytest.mark.parametrize("prec", [Q.PREC_F64, Q.PREC_F32, Q.PREC_BF16])
@pytest.mark.parametrize("streaming", [False, True])
def test_solve_scale_invariance(cuda, prec, streaming):
    """Right-hand sides scaled by 1e-30 and 1e30: the solvers iterate on b / |b|
    (reduced-precision vectors stay near unit scale) and return |b| x, so the
    iterations and the scaled solution match the unit-scale solve."""
    import torch
    g, lat, Do, Dq, b = _setup(8, 0.1, 91, cuda)
    bt = to_dev(b, cuda)
    flags = Q.SOLVE_STREAMING if streaming else 0
    x1 = torch.zeros_like(bt)
    r1 = Dq.solve(x1, bt, tol=1e-10, precision=prec, flags=flags)
    assert r1.status == Q.OK
    for scale in (1e-30, 1e30):
        xs = torch.zeros_like(bt)
        rs = Dq.solve(xs, bt * scale, tol=1e-10, precision=prec, flags=flags)
        assert rs.status == Q.OK and rs.true_rel_res <= 1e-10, (scale, rs)
        assert abs(rs.iters - r1.iters) <= 2
        assert float((xs / scale - x1).norm() / x1.norm()) < 1e-8


@pytest.mark.parametrize("op", [Q.OP_D, Q.OP_DDAG, Q.OP_DDAGD])
@pytest.mark.parametrize("n", [4, 8])
def test_bicgstab_matches_oracle(cuda, op, n):
    """BiCGStab (MatPoly::bicgstab restated) on the non-hermitian D, on D^dag and
    on D^dag D.  The iterates follow the oracle's step for step (compared after
    a fixed number of iterations, before rounding differences in the inner
    products grow: on the non-normal D, BiCGStab's erratic residual amplifies
    them and the absolute eps = 1e-8 stop can then fall some iterations apart);
    the full solves both meet the reference's stopping rule."""
    import torch
    g, lat, Do, Dq, b = _setup(n, 0.1, 95 + n, cuda)
    bt = to_dev(b, cuda)
    for k in (1, 3, 8):
        x_ref, it_ref, ok = Do.bicgstab(b, op, tol=1e-10, maxiter=k)
        xt = torch.zeros_like(bt)
        rep = Dq.bicgstab(xt, bt, op=op, tol=1e-10, maxiter=k)
        assert rep.iters == it_ref and (rep.status == Q.OK) == ok
        x = from_dev(xt)
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-10, k
    x_ref, it_ref, ok = Do.bicgstab(b, op, tol=1e-10)
    xt = torch.zeros_like(bt)
    rep = Dq.bicgstab(xt, bt, op=op, tol=1e-10)
    assert ok and rep.status == Q.OK
    if op == Q.OP_DDAGD:
        assert abs(rep.iters - it_ref) <= 2, (rep.iters, it_ref)
    x = from_dev(xt)
    res = np.linalg.norm(b - Do.apply(x, op)) / np.linalg.norm(b)
    res_ref = np.linalg.norm(b - Do.apply(x_ref, op)) / np.linalg.norm(b)
    assert abs(rep.true_rel_res - res) <= 1e-3 * res + 1e-14
    assert res < 10 * max(res_ref, 1e-6)


def test_bicgstab_to_tolerance_and_shift(cuda):
    """eps = 0 on D^dag D + shift: the relative stop alone ends the solve; the
    result agrees with the oracle and with CG."""
    import torch
    g, lat, Do, Dq, b = _setup(8, 0.1, 99, cuda)
    bt = to_dev(b, cuda)
    for shift in (0.0, 0.3):
        # tol 1e-9 relative to |r0|, above the FP64 floor where BiCGStab's
        # stagnating residual makes the count depend on rounding
        x_ref, it_ref, ok = Do.bicgstab(b, Q.OP_DDAGD, tol=1e-9, shift=shift, eps=0.0)
        xt = torch.zeros_like(bt)
        rep = Dq.bicgstab(xt, bt, op=Q.OP_DDAGD, tol=1e-9, shift=shift, eps=0.0)
        # the count itself is not reproducible to the iteration (the oracle's
        # OpenMP inner products alone move it by ~10 %); the solutions agree
        assert ok and rep.status == Q.OK and abs(rep.iters - it_ref) <= max(5, it_ref // 4), (rep.iters, it_ref)
        x = from_dev(xt)
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-7
        x_cg, _, _ = Do.cg(b, tol=1e-12, shift=shift)
        assert np.linalg.norm(x - x_cg) / np.linalg.norm(x_cg) < 1e-6
    # x0 = b is already the solution of the identity-like zero source: b = 0
    xt = torch.ones_like(bt)
    rep = Dq.bicgstab(xt, torch.zeros_like(bt), op=Q.OP_D)
    assert rep.status == Q.OK and float(xt.abs().max()) == 0.0


def test_cpu_runnable_configuration_n8_on_the_gpu(cuda):
    """The plain method's CPU-runnable configuration (n=8; links from the
    reference's pure-gauge HMC recipe at beta = 1.4, seed 1, 200 trajectories;
    r = 1, m = 0.1; Gaussian source seed 7): the device FP64 CG takes the
    oracle's iterations and solution; the mixed solvers reach the same
    certified 1e-10."""
    import torch
    from tests.configs import reference_thermalised_links
    g = O.geometry(8)
    lat = Q.S2Trivalent(8)
    A, _ = reference_thermalised_links(g, 1.4, 1, 200)
    Do = O.Dirac(g, 1.0, 0.1)
    Do.update(A)
    Dq = Q.DiracS2Dual(lat, 1.0, 0.1)
    Dq.update(A)
    b = O.Rng(g, 7).gaussian_spinor()
    xo, it_o, _ = Do.cg(b, tol=1e-10)
    bt = to_dev(b, cuda)
    for prec in (Q.PREC_F64, Q.PREC_F32, Q.PREC_BF16):
        xt = torch.zeros_like(bt)
        rep = Dq.solve(xt, bt, tol=1e-10, precision=prec)
        assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
        x = from_dev(xt)
        assert np.linalg.norm(x - xo) / np.linalg.norm(xo) < 1e-8
        if prec == Q.PREC_F64:
            assert abs(rep.iters - it_o) <= 1, (rep.iters, it_o)


def test_bounded_waits_run_out_and_the_context_survives(cuda):
    """Failure detection without a GPU fault: a grid barrier whose partner
    block never arrives gives up after its poll limit, raises the abort flag
    and returns an error status; a solve right after works normally."""
    import torch
    rc, resident, streaming = Q.selftest_wait_timeout(20000)
    assert rc == Q.ERR_TIMEOUT and resident and streaming
    g, lat, Do, Dq, b = _setup(4, 0.1, 123, cuda)
    bt = to_dev(b, cuda)
    x = torch.zeros_like(bt)
    rep = Dq.solve(x, bt, tol=1e-10, precision=Q.PREC_F32)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
