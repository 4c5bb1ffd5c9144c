"""The S^2 x S^1 operator (DiracExt, src/both_3d/dirac_ext.h:6-334) on the
GPU against the oracle's restatement: apply for D, D^dag, D^dag D at several
Nt and temporal spacings (Nt = 1 is the dual-lattice operator), and the FP64
CG on D^dag D certified by the true residual."""
import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O
from tests.gpu_util import from_dev, rel, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [2, 4])
@pytest.mark.parametrize("Nt,at", [(1, 1.0), (2, 0.7), (4, 0.3), (5, 1.3)])
def test_ext_apply_matches_oracle(cuda, n, Nt, at):
    import torch
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    rng = np.random.default_rng(100 * n + Nt)
    A = rng.uniform(-np.pi, np.pi, Nt * (g.n_links + g.n_sites))
    v = rng.normal(size=2 * g.n_sites * Nt) + 1j * rng.normal(size=2 * g.n_sites * Nt)
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, at)
    De.update(to_dev(A, cuda))
    vt = to_dev(v, cuda)
    for op in (Q.OP_D, Q.OP_DDAG, Q.OP_DDAGD):
        out = torch.zeros_like(vt)
        De.apply(out, vt, op)
        ref = O.dirac_ext_apply(g, 1.0, 0.1, Nt, at, A, v, op)
        assert rel(from_dev(out), ref) < 1e-13, (op, rel(from_dev(out), ref))
    # in place for D
    w = vt.clone()
    De.apply(w, w, Q.OP_D)
    assert rel(from_dev(w), O.dirac_ext_apply(g, 1.0, 0.1, Nt, at, A, v, 0)) < 1e-13


def test_ext_nt1_is_the_dual_lattice_operator(cuda):
    import torch
    lat = Q.S2Trivalent(4)
    rng = np.random.default_rng(5)
    A = rng.uniform(-np.pi, np.pi, lat.n_links + lat.n_sites)
    De = Q.DiracExt(lat, 1.0, 0.05, 1, 1.0)
    De.update(to_dev(A, cuda))
    D = Q.DiracS2Dual(lat, 1.0, 0.05)
    D.update(A[:lat.n_links])
    vt = to_dev(rng.normal(size=2 * lat.n_sites) * (1 + 0.5j), cuda)
    o1, o2 = torch.zeros_like(vt), torch.zeros_like(vt)
    De.apply(o1, vt, Q.OP_DDAGD)
    D.apply(o2, vt, Q.OP_DDAGD)
    assert float((o1 - o2).abs().max() / o2.abs().max()) < 1e-14


@pytest.mark.parametrize("shift", [0.0, 0.2])
def test_ext_cg_solve(cuda, shift):
    import torch
    n, Nt, at = 4, 4, 0.5
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    rng = np.random.default_rng(7)
    A = rng.uniform(-0.5, 0.5, Nt * (g.n_links + g.n_sites))
    b = rng.normal(size=2 * g.n_sites * Nt) + 1j * rng.normal(size=2 * g.n_sites * Nt)
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, at)
    De.update(to_dev(A, cuda))
    bt = to_dev(b, cuda)
    xt = torch.zeros_like(bt)
    rep = De.solve(xt, bt, tol=1e-10, shift=shift)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    x = from_dev(xt)
    r = b - O.dirac_ext_apply(g, 1.0, 0.1, Nt, at, A, x, 2) - shift * x
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1.05e-10


@pytest.mark.parametrize("n,Nt", [(2, 3), (4, 4)])
def test_ext_gauge_side_matches_oracle(cuda, n, Nt):
    """Anisotropic action, force (the reference's update order) and Polyakov
    loop; plaquette angles bit for bit."""
    import torch
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    at, gsq = 0.6, 0.4
    A = np.random.default_rng(n + Nt).normal(size=Nt * (g.n_links + g.n_sites)) * 0.5
    ths_o, tht_o, S_o, F_o = O.ext_gauge(g, Nt, at, gsq, A)
    At = to_dev(A, cuda)
    ths = torch.zeros(Nt * lat.n_faces, dtype=torch.float64, device=cuda)
    tht = torch.zeros(Nt * lat.n_links, dtype=torch.float64, device=cuda)
    Q.ext_plaquettes(lat, Nt, At, ths, tht)
    assert np.array_equal(from_dev(ths), ths_o.ravel()) and np.array_equal(from_dev(tht), tht_o.ravel())
    S = Q.ext_gauge_action(lat, Nt, at, gsq, At)
    assert abs(S - S_o) < 1e-13 * abs(S_o)
    F = torch.zeros_like(At)
    Q.ext_gauge_force(lat, Nt, at, gsq, At, F)
    # same update order as the reference; the device contracts a*b+c into FMAs
    assert np.abs(from_dev(F) - F_o).max() < 1e-13 * np.abs(F_o).max()
    P = torch.zeros(lat.n_sites, dtype=torch.complex128, device=cuda)
    avg = Q.ext_polyakov(lat, Nt, At, P)
    Po = O.ext_polyakov(g, Nt, A)
    assert np.abs(from_dev(P) - Po).max() < 1e-15 and abs(avg - Po.mean()) < 1e-14


@pytest.mark.parametrize("Nt", [1, 2, 3])
def test_ext_fermion_force_is_the_derivative(cuda, Nt):
    """F = -2 Re <D eta, dD/dA eta> = -d/dA <eta, D^dag D eta> (eta fixed), for
    spatial and temporal links, against finite differences of the oracle's
    restatement of the operator."""
    import torch
    n, at = 2, 0.8
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    rng = np.random.default_rng(40 + Nt)
    A = rng.uniform(-np.pi, np.pi, Nt * (g.n_links + g.n_sites))
    eta = rng.normal(size=2 * g.n_sites * Nt) + 1j * rng.normal(size=2 * g.n_sites * Nt)
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, at)
    De.update(to_dev(A, cuda))
    F = torch.zeros(A.size, dtype=torch.float64, device=cuda)
    De.fermion_force(to_dev(eta, cuda), F)
    F = from_dev(F)
    f = lambda B: np.vdot(eta, O.dirac_ext_apply(g, 1.0, 0.1, Nt, at, B, eta, 2)).real
    h = 1e-6
    nsp = Nt * g.n_links
    picks = list(rng.choice(nsp, 6, replace=False))
    picks += list(nsp + rng.choice(Nt * g.n_sites, 6, replace=False)) if Nt > 1 else [nsp]
    for k in picks:
        Ap, Am = A.copy(), A.copy()
        Ap[k] += h
        Am[k] -= h
        fd = -(f(Ap) - f(Am)) / (2 * h)
        assert abs(fd - F[k]) < 1e-6 * max(1.0, abs(fd)), (k, fd, F[k])


@pytest.mark.parametrize("Nt,npf,integrator", [(2, 1, 0), (3, 2, 0), (2, 2, 1), (4, 1, 1)])
def test_hmc_ext_matches_oracle(cuda, Nt, npf, integrator):
    """S^2 x S^1 HMC trajectories (HMC2::run, U1WilsonExt + DiracExt
    pseudofermions) on the GPU against the oracle from the same seeded
    ParallelRngExt streams: same Metropolis decisions, dH to 1e-8, links to
    1e-9 after three trajectories, CG iterations within 10%."""
    import torch
    n, at, gsq, r, M5 = 2, 0.8, 1.0, 1.0, 0.1
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = np.random.default_rng(50 + Nt).uniform(-0.3, 0.3, Nt * (g.n_links + g.n_sites))
    De = Q.DiracExt(lat, r, M5, Nt, at)
    seed = 90 + 7 * Nt + npf
    rd, ro = Q.ParallelRng(lat, seed, n_slices=Nt), O.Rng(g, seed, Nt)
    Ad = to_dev(A, cuda)
    Ao = A.copy()
    for t in range(3):
        acc_d, dH_d, it_d = Q.hmc_ext(De, rd, Ad, gsq, tmax=0.5, nsteps=4, nsteps_inner=2, npf=npf,
                                      integrator=integrator, tol=1e-12)
        acc_o, dH_o, it_o = O.hmc_ext(g, ro, Ao, r, M5, Nt, at, gsq, tmax=0.5, nsteps=4, nsteps_inner=2, npf=npf,
                                      integrator=integrator, tol=1e-12)
        assert acc_d == acc_o, (t, dH_d, dH_o)
        assert abs(dH_d - dH_o) < 1e-8 * (1 + abs(dH_o)), (t, dH_d, dH_o)
        assert abs(it_d - it_o) <= 0.1 * it_o + 2, (it_d, it_o)
        torch.cuda.synchronize()
        assert np.abs(from_dev(Ad) - Ao).max() < 1e-9
    # the streams stayed in step: the next draws agree
    assert np.array_equal(rd.gaussian_links(), ro.gaussian_links())


def test_hmc_ext_rejects_bad_rng(cuda):
    """The RNG must hold Nt times the lattice's engines (ParallelRngExt)."""
    lat = Q.S2Trivalent(2)
    De = Q.DiracExt(lat, 1.0, 0.1, 2, 0.8)
    A = torch_zeros(2 * (lat.n_links + lat.n_sites), cuda)
    with pytest.raises(Q.Qed3Error):
        Q.hmc_ext(De, Q.ParallelRng(lat, 1), A, 1.0)


def torch_zeros(n, device):
    import torch
    return torch.zeros(n, dtype=torch.float64, device=device)


@pytest.mark.parametrize("Nt,at", [(1, 1.0), (4, 0.5)])
def test_ext_propagator_matches_oracle(cuda, Nt, at):
    """prop.cu's point-source propagator: sink = (D^dag D)^{-1} D^dag delta on
    the GPU = the oracle's dense D^{-1} delta, for a random and the free field;
    the written profiles carry the sink's values."""
    import torch
    from qed3_gb300 import correlators as C
    n = 2
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    De = Q.DiracExt(lat, 1.0, 0.0, Nt, at)
    for A in (np.random.default_rng(60 + Nt).uniform(-np.pi, np.pi, Nt * (g.n_links + g.n_sites)),
              np.zeros(Nt * (g.n_links + g.n_sites))):
        De.update(to_dev(A, cuda))
        M = O.dirac_ext_matrix(g, 1.0, 0.0, Nt, at, A)
        for s, ix, a, dag in ((0, 0, 0, False), (Nt - 1, 7, 1, False), (0, 3, 1, True)):
            sink = torch.zeros(2 * g.n_sites * Nt, dtype=torch.complex128, device=cuda)
            rep = De.propagator(sink, s, ix, a, tol=1e-12, dagger=dag)
            assert rep.status == Q.OK and rep.true_rel_res <= 1e-12
            delta = np.zeros(2 * g.n_sites * Nt, np.complex128)
            delta[(s * g.n_sites + ix) * 2 + a] = 1.0
            ref = np.linalg.solve(M.conj().T if dag else M, delta)
            got = from_dev(sink)
            assert rel(got, ref) < 1e-8, dag
            if not dag:
                sink_d, got_d = sink, got
        sink, got = sink_d, got_d
        sp, tp = C.prop_profiles(lat, sink, Nt, at)
        fac = (at if Nt > 1 else 1.0) * lat.tables()["means"][0]
        assert np.allclose(tp[0::2, 1], got.reshape(Nt, -1, 2)[:, 0, 0].real / fac)
    with pytest.raises(Q.Qed3Error):
        De.propagator(sink, Nt, 0, 0)


@pytest.mark.parametrize("shift", [0.0, 0.05])
def test_ext_cg_mixed_precision(cuda, shift):
    """FP32 iterations with FP64 reliable updates on the S^2 x S^1 operator:
    the FP64 certificate holds at 1e-10, the solution is the FP64 solve's,
    iterations stay within 1.5x of FP64, and b scaled by 1e+-30 gives the
    same iteration count (the FP32 iteration runs on r / |r|)."""
    import torch
    n, Nt, at = 4, 4, 0.6
    lat = Q.S2Trivalent(n)
    rng = np.random.default_rng(80)
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, at)
    De.update(to_dev(rng.uniform(-np.pi, np.pi, Nt * (lat.n_links + lat.n_sites)), cuda))
    b = rng.normal(size=2 * lat.n_sites * Nt) + 1j * rng.normal(size=2 * lat.n_sites * Nt)
    x64 = torch.zeros(b.size, dtype=torch.complex128, device=cuda)
    r64 = De.solve(x64, to_dev(b, cuda), tol=1e-10, shift=shift)
    assert r64.status == Q.OK
    its = []
    for scale in (1.0, 1e-30, 1e30):
        x = torch.zeros_like(x64)
        r = De.solve(x, to_dev(b * scale, cuda), tol=1e-10, shift=shift, precision=Q.PREC_F32)
        assert r.status == Q.OK and r.true_rel_res <= 1e-10 and r.reliable_updates >= 1, (scale, r)
        assert rel(from_dev(x) / scale, from_dev(x64)) < 1e-8
        its.append(r.iters)
    assert its[0] <= 1.5 * r64.iters + 10, (its, r64.iters)
    assert max(its) - min(its) <= 2, its


def test_ext_propagator_mixed_precision(cuda):
    import torch
    n, Nt, at = 2, 4, 0.5
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    De = Q.DiracExt(lat, 1.0, 0.0, Nt, at)
    A = np.random.default_rng(81).uniform(-np.pi, np.pi, Nt * (g.n_links + g.n_sites))
    De.update(to_dev(A, cuda))
    M = O.dirac_ext_matrix(g, 1.0, 0.0, Nt, at, A)
    for dag in (False, True):
        sink = torch.zeros(2 * g.n_sites * Nt, dtype=torch.complex128, device=cuda)
        rep = De.propagator(sink, 1, 5, 0, tol=1e-11, dagger=dag, precision=Q.PREC_F32)
        assert rep.status == Q.OK and rep.true_rel_res <= 1e-11
        delta = np.zeros(2 * g.n_sites * Nt, np.complex128)
        delta[(1 * g.n_sites + 5) * 2] = 1.0
        assert rel(from_dev(sink), np.linalg.solve(M.conj().T if dag else M, delta)) < 1e-8


def test_ext_cg_large_field_iteration_counts(cuda):
    """n=32, Nt=8 (327,680 complex unknowns: the reduction partials fill their
    whole scratch): FP64 and mixed solves report consistent iteration counts
    and meet the certificate."""
    import torch
    n, Nt, at = 32, 8, 0.5
    lat = Q.S2Trivalent(n)
    rng = np.random.default_rng(82)
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, at)
    De.update(to_dev(0.3 * rng.uniform(-np.pi, np.pi, Nt * (lat.n_links + lat.n_sites)), cuda))
    b = to_dev(rng.normal(size=2 * lat.n_sites * Nt) + 1j * rng.normal(size=2 * lat.n_sites * Nt), cuda)
    x = torch.zeros_like(b)
    r64 = De.solve(x, b, tol=1e-10)
    r32 = De.solve(x, b, tol=1e-10, precision=Q.PREC_F32)
    assert r64.status == Q.OK and r32.status == Q.OK and r32.true_rel_res <= 1e-10
    assert 0.8 * r64.iters <= r32.iters <= 1.5 * r64.iters + 10, (r64.iters, r32.iters)


def test_hmc_ext_mixed_precision_matches_fp64(cuda):
    """The S^2 x S^1 trajectory with FP32 + reliable-update solves to 1e-12
    follows the FP64 one: same decisions, dH to 1e-7, links to 1e-8."""
    import torch
    n, Nt, at = 2, 3, 0.8
    lat = Q.S2Trivalent(n)
    A = torch.from_numpy(np.random.default_rng(83).uniform(-0.3, 0.3, Nt * (lat.n_links + lat.n_sites))).to(cuda)
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, at)
    A64, A32 = A.clone(), A.clone()
    r64, r32 = Q.ParallelRng(lat, 7, n_slices=Nt), Q.ParallelRng(lat, 7, n_slices=Nt)
    for t in range(2):
        a64 = Q.hmc_ext(De, r64, A64, 1.0, tmax=0.5, nsteps=4, nsteps_inner=2, npf=2, tol=1e-12)
        a32 = Q.hmc_ext(De, r32, A32, 1.0, tmax=0.5, nsteps=4, nsteps_inner=2, npf=2, tol=1e-12,
                        precision=Q.PREC_F32)
        assert a64[0] == a32[0] and abs(a64[1] - a32[1]) < 1e-7 * (1 + abs(a64[1])), (a64, a32)
        assert float((A64 - A32).abs().max()) < 1e-8


def test_overlap_ext_matches_oracle(cuda):
    """Overlap<DiracExt> (the reference's IS_OVERLAP operator on S^2 x S^1):
    D_ov, D_ov^dag and D_ov + D_ov^dag from one multi-shift CG per product =
    the oracle's dense restatement to 1e-9 at given bounds; Lanczos bounds =
    the dense spectrum's within the margin; the outer solve and the
    propagator (D_ov^dag D_ov)^{-1} D_ov^dag b are certified and match the
    dense solves; the Ginsparg-Wilson defect D_ov + D_ov^dag - D_ov^dag D_ov
    is at the Zolotarev error."""
    import torch
    n, Nt, at, r, M5, order = 2, 2, 0.7, 1.0, -1.0, 21
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = np.random.default_rng(90).uniform(-0.5, 0.5, Nt * (g.n_links + g.n_sites))
    De = Q.DiracExt(lat, r, M5, Nt, at)
    De.update(to_dev(A, cuda))
    M = O.dirac_ext_matrix(g, r, M5, Nt, at, A)
    sv = np.sqrt(np.linalg.eigvalsh(M.conj().T @ M))
    lmin, lmax = sv[0] * 0.99, sv[-1] * 1.01
    ov = Q.OverlapExt(De, order)
    ov.update(lmin, lmax)
    Dov = O.overlap_ext_matrix(g, r, M5, Nt, at, A, lmin, lmax, order)
    v = np.random.default_rng(91).normal(size=Dov.shape[0]) + 1j * np.random.default_rng(92).normal(size=Dov.shape[0])
    vd = to_dev(v, cuda)
    for op, ref in ((Q.OP_D, Dov @ v), (Q.OP_DDAG, Dov.conj().T @ v), (Q.OP_DDAGD, (Dov + Dov.conj().T) @ v)):
        out = torch.zeros_like(vd)
        its = ov.apply(out, vd, op, tol_inner=1e-13)
        assert its > 0 and rel(from_dev(out), ref) < 1e-9, op
    gw = Dov + Dov.conj().T - Dov.conj().T @ Dov
    assert np.abs(gw).max() < 10 * ov.info()["delta"] + 1e-9
    x = torch.zeros_like(vd)
    rep = ov.solve(x, vd, tol=1e-10, tol_inner=1e-13)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-9
    H = Dov + Dov.conj().T
    assert rel(from_dev(x), np.linalg.solve(H, v)) < 1e-7
    rep = ov.solve(x, vd, tol=1e-10, tol_inner=1e-13, propagator=True)
    assert rep.status == Q.OK
    assert rel(from_dev(x), np.linalg.solve(H, Dov.conj().T @ v)) < 1e-7
    ov2 = Q.OverlapExt(De, order)
    ov2.update(tol=1e-12, margin=1e-6)
    inf = ov2.info()
    assert abs(inf["lambda_min"] / sv[0] - 1) < 1e-4 and abs(inf["lambda_max"] / sv[-1] - 1) < 1e-4, (inf, sv[0], sv[-1])


def _ext_overlap_case(cuda):
    n, Nt, at, r, M5, order = 2, 2, 0.7, 1.0, -1.0, 21
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = np.random.default_rng(90).uniform(-0.5, 0.5, Nt * (g.n_links + g.n_sites))
    M = O.dirac_ext_matrix(g, r, M5, Nt, at, A)
    sv = np.sqrt(np.linalg.eigvalsh(M.conj().T @ M))
    return g, lat, A, (n, Nt, at, r, M5, order), sv[0] * 0.99, sv[-1] * 1.01


def test_overlap_ext_force_matches_oracle(cuda):
    """F = -2 d/dA Re<eta, D_ov eta> for Overlap<DiracExt> on the GPU (one pass
    of the link kernels per bilinear) = the oracle's chain-rule restatement on
    dense matrices (itself checked against finite differences)."""
    import torch
    g, lat, A, (n, Nt, at, r, M5, order), lmin, lmax = _ext_overlap_case(cuda)
    De = Q.DiracExt(lat, r, M5, Nt, at)
    De.update(to_dev(A, cuda))
    ov = Q.OverlapExt(De, order)
    ov.update(lmin, lmax)
    rng = np.random.default_rng(93)
    eta = rng.normal(size=2 * g.n_sites * Nt) + 1j * rng.normal(size=2 * g.n_sites * Nt)
    F = torch.zeros(A.size, dtype=torch.float64, device=cuda)
    ov.force(to_dev(eta, cuda), F, tol_inner=1e-13)
    ref = O.overlap_ext_force(g, r, M5, Nt, at, A, eta, lmin, lmax, order)
    assert rel(from_dev(F), ref) < 1e-9


def test_hmc_ext_overlap_matches_oracle(cuda):
    """S^2 x S^1 HMC with overlap pseudofermions (the reference's IS_OVERLAP
    hmc.cu) at fixed bounds against the oracle's dense restatement from the
    same ParallelRngExt streams: same decisions, dH to 1e-7, links to 1e-8."""
    import torch
    g, lat, A, (n, Nt, at, r, M5, order), lmin, lmax = _ext_overlap_case(cuda)
    De = Q.DiracExt(lat, r, M5, Nt, at)
    ov = Q.OverlapExt(De, order)
    rd, ro = Q.ParallelRng(lat, 5, n_slices=Nt), O.Rng(g, 5, Nt)
    Ad, Ao = to_dev(A, cuda), A.copy()
    for t in range(2):
        acc_d, dH_d, its = Q.hmc_ext_overlap(ov, rd, Ad, 1.0, tmax=0.3, nsteps=3, nsteps_inner=2, tol=1e-11,
                                             tol_inner=1e-13, lambda_min=lmin, lambda_max=lmax)
        acc_o, dH_o = O.hmc_ext_overlap(g, ro, Ao, r, M5, Nt, at, 1.0, lmin, lmax, order, tmax=0.3, nsteps=3,
                                        nsteps_inner=2)
        assert acc_d == acc_o and its > 0, (t, dH_d, dH_o)
        assert abs(dH_d - dH_o) < 1e-7 * (1 + abs(dH_o)), (t, dH_d, dH_o)
        torch.cuda.synchronize()
        assert np.abs(from_dev(Ad) - Ao).max() < 1e-8


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_ext_cg_edge_cases(cuda, prec):
    """maxiter reached: status NOCONV with exactly maxiter iterations (the
    device counter, graph chunks or not); b = 0: x = 0 at once."""
    import torch
    lat = Q.S2Trivalent(4)
    Nt = 3
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, 0.6)
    rng = np.random.default_rng(84)
    De.update(to_dev(rng.uniform(-np.pi, np.pi, Nt * (lat.n_links + lat.n_sites)), cuda))
    p = Q.PREC_F64 if prec == "f64" else Q.PREC_F32
    b = to_dev(rng.normal(size=2 * lat.n_sites * Nt) + 1j * rng.normal(size=2 * lat.n_sites * Nt), cuda)
    x = torch.zeros_like(b)
    for maxiter in (5, 21):
        r = De.solve(x, b, tol=1e-14, maxiter=maxiter, precision=p)
        assert r.status == Q.ERR_NOCONV and r.iters == maxiter, (maxiter, r)
        assert 0 < r.true_rel_res < 1
    z = torch.zeros_like(b)
    r = De.solve(x, z, tol=1e-10, precision=p)
    assert r.status == Q.OK and r.iters == 0 and float(x.abs().max()) == 0.0
