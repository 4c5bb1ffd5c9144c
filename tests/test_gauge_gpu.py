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
