"""GPU gauge side, fermion force and pure-gauge HMC against the oracle."""
import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O
from tests.gpu_util import from_dev, rand_spinor, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [2, 8, 32])
def test_plaquette_action_force(cuda, n):
    import torch
    rng = np.random.default_rng(30 + n)
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = rng.uniform(-np.pi, np.pi, g.n_links)
    At = to_dev(A, cuda)
    th = torch.zeros(g.n_faces, dtype=torch.float64, device=cuda)
    avg = Q.plaquette(lat, At, th)
    th_ref = O.plaquettes(g, A)
    assert np.abs(from_dev(th) - th_ref).max() < 1e-13
    assert abs(avg - np.mean(np.cos(th_ref))) < 1e-13
    for compact in (True, False):
        S = Q.gauge_action(lat, At, 1.4, compact)
        S_ref = O.gauge_action(g, A, 1.4, compact)
        assert abs(S - S_ref) <= 1e-12 * max(1.0, abs(S_ref))
        for exact in (True, False):
            F = torch.zeros(g.n_links, dtype=torch.float64, device=cuda)
            Q.gauge_force(lat, At, F, 1.4, compact, exact)
            F_ref = O.gauge_force(g, A, 1.4, compact, exact)
            assert np.abs(from_dev(F) - F_ref).max() < 1e-12


@pytest.mark.parametrize("n", [2, 8, 16])
def test_fermion_force_matches_oracle(cuda, n):
    import torch
    rng = np.random.default_rng(40 + n)
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = rng.uniform(-np.pi, np.pi, g.n_links)
    Do = O.Dirac(g, 1.0, 0.1)
    Do.update(A)
    Dq = Q.DiracS2Dual(lat, 1.0, 0.1)
    Dq.update(A)
    eta = rand_spinor(rng, g.n_sites)
    F = torch.zeros(g.n_links, dtype=torch.float64, device=cuda)
    Q.fermion_force(Dq, to_dev(eta, cuda), F)
    F_ref = Do.fermion_force(A, eta)
    assert np.abs(from_dev(F) - F_ref).max() <= 1e-12 * np.abs(F_ref).max()


def test_rng_streams_match_oracle():
    g = O.geometry(4)
    lat = Q.S2Trivalent(4)
    r1, r2 = O.Rng(g, 9), Q.ParallelRng(lat, 9)
    assert np.array_equal(r1.gaussian_links(0.7), r2.gaussian_links(0.7))
    assert np.array_equal(r1.gaussian_spinor(), r2.gaussian_spinor())


@pytest.mark.parametrize("compact", [True, False])
def test_hmc_trajectory_matches_oracle(cuda, compact):
    # same seed, same libstdc++ streams: the trajectory and the Metropolis
    # decision agree; dH agrees to the oracle's own cancellation error
    n = 4
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    ro, rq = O.Rng(g, 3), Q.ParallelRng(lat, 3)
    A0 = ro.gaussian_links(0.2)
    assert np.array_equal(A0, rq.gaussian_links(0.2))
    Ao = np.ascontiguousarray(A0.copy())
    At = to_dev(A0, cuda)
    for it in range(5):
        acc_o, dh_o = O.hmc_pure_gauge(g, ro, Ao, 1.4, compact, True, 1.0, 10)
        acc_q, dh_q = Q.hmc_pure_gauge(lat, rq, At, 1.4, compact, True, 1.0, 10)
        assert acc_o == acc_q
        assert abs(dh_o - dh_q) < 1e-11
        assert np.abs(from_dev(At) - Ao).max() < 1e-11


@pytest.mark.parametrize("integrator", [Q.INTEGRATOR_LEAPFROG_ML, Q.INTEGRATOR_LEAPFROG])
def test_fermion_hmc_matches_oracle(cuda, integrator):
    """Wilson-fermion HMC trajectories (HMC::run + ExplicitLeapfrogML, one
    pseudofermion) against the oracle's restatement from the same RNG streams:
    same Metropolis decisions, dH and links to the pseudofermion-solve tolerance."""
    n = 4
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    ro, rq = O.Rng(g, 7), Q.ParallelRng(lat, 7)
    A0 = ro.gaussian_links(0.2)
    assert np.array_equal(A0, rq.gaussian_links(0.2))
    Ao = np.ascontiguousarray(A0.copy())
    At = to_dev(A0, cuda)
    Do = O.Dirac(g, 1.0, 0.1)
    Dq = Q.DiracS2Dual(lat, 1.0, 0.1)
    for it in range(3):
        acc_o, dh_o, _ = O.hmc_fermion(g, Do, ro, Ao, 1.4, tmax=0.5, nsteps=5, nsteps_inner=4, tol=1e-13,
                                       integrator=integrator)
        acc_q, dh_q, its = Q.hmc_fermion(lat, Dq, rq, At, 1.4, tmax=0.5, nsteps=5, nsteps_inner=4, tol=1e-13,
                                         precision=Q.PREC_F64, integrator=integrator)
        assert acc_o == acc_q and its > 0
        assert abs(dh_o - dh_q) < 1e-8 * max(1.0, abs(dh_o))
        assert np.abs(from_dev(At) - Ao).max() < 1e-9


def test_fermion_hmc_dH_scales_as_tau_squared(cuda):
    """Second-order integrator: halving the outer step divides dH by ~4 (the
    reference's dH ~ tau^2 check; RMS over four draws), in mixed precision with
    FP64 certificates."""
    n = 4
    lat = Q.S2Trivalent(n)
    A0 = Q.ParallelRng(lat, 11).gaussian_links(0.3)
    D = Q.DiracS2Dual(lat, 1.0, 0.1)
    rms = []
    for ns in (16, 32):
        v = []
        for seed in range(12, 16):
            At = to_dev(A0, cuda)
            _, d, _ = Q.hmc_fermion(lat, D, Q.ParallelRng(lat, seed), At, 1.4, tmax=1.0, nsteps=ns, nsteps_inner=4,
                                    tol=1e-12, precision=Q.PREC_F32, no_reject=True)
            v.append(d)
        rms.append(np.sqrt(np.mean(np.square(v))))
    assert 2.8 < rms[0] / rms[1] < 5.5, rms


def test_fermion_hmc_rejection_restores_links(cuda):
    lat = Q.S2Trivalent(2)
    A0 = Q.ParallelRng(lat, 13).gaussian_links(0.3)
    At = to_dev(A0, cuda)
    D = Q.DiracS2Dual(lat, 1.0, 0.1)
    # a huge step makes dH large: the trajectory is rejected and A restored
    acc, d, _ = Q.hmc_fermion(lat, D, Q.ParallelRng(lat, 14), At, 1.4, tmax=4.0, nsteps=1, nsteps_inner=1,
                              tol=1e-10, precision=Q.PREC_F64)
    if not acc:
        assert np.array_equal(from_dev(At), A0)
    assert np.isfinite(d)


def test_fermion_hmc_two_pseudofermions_matches_oracle(cuda):
    """HMC2::run: two pseudofermions drawn one after the other from the same
    streams, their forces kicking the momenta in turn; GPU = oracle."""
    n = 2
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    ro, rq = O.Rng(g, 17), Q.ParallelRng(lat, 17)
    A0 = ro.gaussian_links(0.2)
    assert np.array_equal(A0, rq.gaussian_links(0.2))
    Ao = np.ascontiguousarray(A0.copy())
    At = to_dev(A0, cuda)
    Do = O.Dirac(g, 1.0, 0.1)
    Dq = Q.DiracS2Dual(lat, 1.0, 0.1)
    for it in range(3):
        acc_o, dh_o, its_o = O.hmc_fermion(g, Do, ro, Ao, 1.4, tmax=0.5, nsteps=5, nsteps_inner=4, tol=1e-13, npf=2)
        acc_q, dh_q, its = Q.hmc_fermion(lat, Dq, rq, At, 1.4, tmax=0.5, nsteps=5, nsteps_inner=4, tol=1e-13,
                                         precision=Q.PREC_F64, npf=2)
        assert acc_o == acc_q and its > 0
        assert abs(dh_o - dh_q) < 1e-8 * max(1.0, abs(dh_o))
        assert np.abs(from_dev(At) - Ao).max() < 1e-9


def test_product_rng_matches_reference_build(cuda):
    """The library's host ParallelRng streams against the reference's own
    src/both/rng.h (golden fixture made by compiling it in place)."""
    import json
    import os
    data = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "rng_ref.json")))
    h = lambda v: np.array([float.fromhex(s) for s in v])
    for c in data["cases"]:
        nref = {30: 1, 120: 2, 480: 4}[c["n_links"]]
        lat = Q.S2Trivalent(nref)
        assert lat.n_links == c["n_links"] and lat.n_sites == c["n_sites"]
        rng = Q.ParallelRng(lat, c["seed"])
        links2 = np.concatenate([rng.gaussian_links(1.0), rng.gaussian_links(1.0)])
        assert np.array_equal(links2, h(c["links2"]))
        xi = rng.gaussian_spinor()
        s4 = h(c["sites4"])
        assert np.array_equal(xi.real, s4[0::2] / np.sqrt(2.0))
        assert np.array_equal(xi.imag, s4[1::2] / np.sqrt(2.0))
        z = rng.z2_spinor()
        z2 = np.array(c["z2"], dtype=np.float64)
        nrm = np.sqrt(2.0 * c["n_sites"])
        assert np.array_equal(z.real, z2[0::2] / nrm) and np.array_equal(z.imag, z2[1::2] / nrm)


def test_product_gauge_side_matches_reference_build(cuda):
    """The library's plaquettes, action, force and pure-gauge HMC against the
    reference's own gauge code compiled in place (golden fixture): angles bit
    for bit, forces to rounding, the same Metropolis decisions, dH within 1e-12
    and the links to rounding after three trajectories."""
    import json
    import os
    import torch
    data = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "gauge_ref.json")))
    h = lambda v: np.array([float.fromhex(s) for s in v])
    for c in data["cases"]:
        lat = Q.S2Trivalent(c["n"])
        A = h(c["A"])
        At = to_dev(A, cuda)
        th = torch.zeros(lat.n_faces, dtype=torch.float64, device=cuda)
        avg = Q.plaquette(lat, At, th)
        assert np.array_equal(from_dev(th), h(c["theta"]))
        assert abs(avg - float.fromhex(c["avg_plaquette"])) < 1e-14
        S_ref = float.fromhex(c["action"])
        assert abs(Q.gauge_action(lat, At, c["beta"], c["compact"]) - S_ref) < 1e-13 * abs(S_ref)
        F = torch.zeros_like(At)
        Q.gauge_force(lat, At, F, c["beta"], c["compact"], exact=False)
        Fr = h(c["force"])
        assert np.abs(from_dev(F) - Fr).max() < 1e-13 * np.abs(Fr).max()
        hm = c["hmc"]
        rng = Q.ParallelRng(lat, hm["seed"])
        for t in range(len(hm["dH"])):
            acc, dH = Q.hmc_pure_gauge(lat, rng, At, c["beta"], c["compact"], False, hm["tmax"], hm["nsteps"])
            assert acc == bool(hm["accepted"][t])
            assert abs(dH - float.fromhex(hm["dH"][t])) < 1e-12  # measured <= 1.7e-13
        assert np.abs(from_dev(At) - h(hm["A_final"])).max() < 1e-13
