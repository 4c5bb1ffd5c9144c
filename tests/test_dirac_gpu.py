"""GPU parity of the Wilson-Dirac apply against the oracle's CSR operator.

Tolerance (stated by the target): FP64 apply within 1e-13 relative of the
reference FP64 apply; FP32 within 2e-6 and BF16-stored spinors within 2e-2
relative (storage rounding), both against the FP64 result.
"""
import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O
from tests.gpu_util import from_dev, rand_spinor, rel, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 8, 16, 64])
def test_apply_matches_oracle(cuda, n):
    rng = np.random.default_rng(100 + n)
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = rng.uniform(-np.pi, np.pi, g.n_links)
    M5 = 0.1
    Do = O.Dirac(g, 1.0, M5)
    Do.update(A)
    Dq = Q.DiracS2Dual(lat, 1.0, M5)
    Dq.update(A)
    v = rand_spinor(rng, g.n_sites)
    vt = to_dev(v, cuda)
    for op in (Q.OP_D, Q.OP_DDAG, Q.OP_DDAGD):
        ref = Do.apply(v, op)
        out = vt.clone() * 0
        Dq.apply(out, vt, op)
        assert rel(from_dev(out), ref) < 1e-13, (n, op)
    # D D^dagger
    out = vt.clone() * 0
    Dq.apply(out, vt, Q.OP_DDDAG)
    assert rel(from_dev(out), Do.apply(Do.apply(v, 1), 0)) < 1e-13


def test_apply_in_place_and_device_links(cuda):
    import torch
    rng = np.random.default_rng(5)
    n = 4
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = rng.normal(size=g.n_links)
    Do = O.Dirac(g, 1.0, -0.4)
    Do.update(A)
    Dq = Q.DiracS2Dual(lat, 1.0, -0.4)
    Dq.update(torch.from_numpy(A).to(cuda))  # device-resident links
    v = rand_spinor(rng, g.n_sites)
    vt = to_dev(v, cuda)
    Dq.apply(vt, vt, Q.OP_D)  # in place
    torch.cuda.synchronize()
    assert rel(from_dev(vt), Do.apply(v, 0)) < 1e-13


@pytest.mark.parametrize("prec,tol", [(Q.PREC_F64, 0.0), (Q.PREC_F32, 2e-6), (Q.PREC_BF16, 2e-2)])
def test_field_roundtrip_and_low_precision_apply(cuda, prec, tol):
    import torch
    rng = np.random.default_rng(7)
    n = 16
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = rng.uniform(-np.pi, np.pi, g.n_links)
    Do = O.Dirac(g, 1.0, 0.05)
    Do.update(A)
    Dq = Q.DiracS2Dual(lat, 1.0, 0.05)
    Dq.update(A)
    nrhs = 3
    v = rand_spinor(rng, g.n_sites, nrhs)
    vt = to_dev(v, cuda)
    f_in = torch.empty(Dq.field_bytes(prec, nrhs), dtype=torch.uint8, device=cuda)
    f_out = torch.empty_like(f_in)
    Dq.field_import(f_in, vt, prec, nrhs)
    back = torch.empty_like(vt)
    Dq.field_export(back, f_in, prec, nrhs)
    torch.cuda.synchronize()
    if prec == Q.PREC_F64:
        assert np.array_equal(from_dev(back), v)
    for op in (Q.OP_D, Q.OP_DDAG):
        Dq.apply_field(f_out, f_in, op, prec, nrhs)
        out = torch.empty_like(vt)
        Dq.field_export(out, f_out, prec, nrhs)
        torch.cuda.synchronize()
        o = from_dev(out)
        for r in range(nrhs):
            ref = Do.apply(v[r], op)
            assert rel(o[r], ref) < max(tol, 1e-13), (prec, op, r)


def test_set_coefficients_generic_builder(cuda):
    # any builder with the same sparsity (e.g. Dirac1fonS2) feeds the same kernel
    rng = np.random.default_rng(11)
    n = 2
    lat = Q.S2Trivalent(n)
    t = lat.tables()
    Ns = lat.n_sites
    hop = rng.normal(size=(Ns, 3, 4)) + 1j * rng.normal(size=(Ns, 3, 4))
    diag = rng.normal(size=Ns)
    M = np.zeros((2 * Ns, 2 * Ns), complex)
    for x in range(Ns):
        M[2 * x:2 * x + 2, 2 * x:2 * x + 2] += diag[x] * np.eye(2)
        for k in range(3):
            y = t["nns"][x, k]
            M[2 * x:2 * x + 2, 2 * y:2 * y + 2] += hop[x, k].reshape(2, 2)
    Dq = Q.DiracS2Dual(lat, 1.0, 0.0)
    Dq.set_coefficients(hop, diag)
    v = rand_spinor(rng, Ns)
    vt = to_dev(v, cuda)
    for op, Mo in ((Q.OP_D, M), (Q.OP_DDAG, M.conj().T), (Q.OP_DDAGD, M.conj().T @ M)):
        out = vt.clone()
        Dq.apply(out, vt, op)
        assert rel(from_dev(out), Mo @ v) < 1e-13


def test_apply_before_links_is_a_state_error(cuda):
    lat = Q.S2Trivalent(1)
    Dq = Q.DiracS2Dual(lat, 1.0, 0.0)
    import torch
    v = torch.zeros(2 * lat.n_sites, dtype=torch.complex128, device=cuda)
    with pytest.raises(Q.Qed3Error) as e:
        Dq.apply(v.clone(), v, Q.OP_D)
    assert e.value.status == Q.ERR_STATE


def test_operator_on_a_callers_mesh(cuda):
    """The same sphere in a caller's numbering (vertices and triangles
    relabelled, windings reversed, links in a shuffled order): the plaquettes of
    the correspondingly mapped link field agree face by face and D^dag D has the
    same spectrum (the spin structures differ at most by a sign per site)."""
    import torch
    from tests.test_lattice import _relabelled_mesh
    lat, v2, t2, pv, pt = _relabelled_mesh(2, 3)
    links_default = Q.S2Trivalent.from_mesh(v2, t2).tables()["links"]
    lat2 = Q.S2Trivalent.from_mesh(v2, t2, links=links_default[np.random.default_rng(4).permutation(lat.n_links)])
    a, b = lat.tables(), lat2.tables()
    A = np.random.default_rng(5).uniform(-np.pi, np.pi, lat.n_links)
    old = {tuple(l): i for i, l in enumerate(a["links"])}
    A2 = np.empty_like(A)
    for i, (x, y) in enumerate(b["links"]):
        ox, oy = pt[x], pt[y]
        A2[i] = (1.0 if ox < oy else -1.0) * A[old[(min(ox, oy), max(ox, oy))]]
    th = torch.zeros(lat.n_faces, dtype=torch.float64, device=cuda)
    th2 = torch.zeros_like(th)
    Q.plaquette(lat, to_dev(A, cuda), th)
    Q.plaquette(lat2, to_dev(A2, cuda), th2)
    assert np.abs(from_dev(th2) - from_dev(th)[pv]).max() < 1e-13

    def dense(L, Ah):
        D = Q.DiracS2Dual(L, 1.0, 0.1)
        D.update(Ah)
        N = 2 * L.n_sites
        M = np.zeros((N, N), np.complex128)
        e = torch.zeros(N, dtype=torch.complex128, device=cuda)
        out = torch.zeros_like(e)
        for j in range(N):
            e.zero_()
            e[j] = 1.0
            D.apply(out, e, Q.OP_DDAGD)
            M[:, j] = from_dev(out)
        return M
    w1 = np.linalg.eigvalsh(dense(lat, A))
    w2 = np.linalg.eigvalsh(dense(lat2, A2))
    assert np.abs(w1 - w2).max() < 1e-12 * w1.max()


def test_caller_spin_structure_enters_the_operator(cuda):
    """omega(l) + 2 pi flips the sign of both hop blocks of link l (the half-angle
    Omega), which is the same operator as A_l + pi: the caller's table is used."""
    import torch
    n, l = 4, 17
    A = np.random.default_rng(6).uniform(-np.pi, np.pi, 30 * n * n)
    lat1 = Q.S2Trivalent(n)
    om = lat1.tables()["omega"].copy()
    om[l] += 2 * np.pi
    lat1.set_spin_structure(om)
    D1 = Q.DiracS2Dual(lat1, 1.0, 0.1)
    D1.update(A)
    lat2 = Q.S2Trivalent(n)
    D2 = Q.DiracS2Dual(lat2, 1.0, 0.1)
    A2 = A.copy()
    A2[l] += np.pi
    D2.update(A2)
    v = to_dev(np.random.default_rng(7).normal(size=2 * lat1.n_sites) * (1 + 1j), cuda)
    o1, o2 = torch.zeros_like(v), torch.zeros_like(v)
    D1.apply(o1, v, Q.OP_D)
    D2.apply(o2, v, Q.OP_D)
    assert float((o1 - o2).abs().max()) < 1e-13 * float(o2.abs().max())


def test_oriented_links_give_the_same_operator(cuda):
    """Reversing the stored orientation of some links and negating their
    angles is the same gauge field: identical D apply, plaquettes and fermion
    force up to the links' signs."""
    import torch
    lat = Q.S2Trivalent(4)
    v, t = lat.mesh()
    a = lat.tables()
    flip = np.zeros(lat.n_links, bool)
    flip[1::4] = True
    links = a["links"].copy()
    links[flip] = links[flip][:, ::-1]
    lat2 = Q.S2Trivalent.from_mesh(v, t, links=links)
    A = np.random.default_rng(8).uniform(-np.pi, np.pi, lat.n_links)
    A2 = np.where(flip, -A, A)
    D1, D2 = Q.DiracS2Dual(lat, 1.0, 0.1), Q.DiracS2Dual(lat2, 1.0, 0.1)
    D1.update(A)
    D2.update(A2)
    vt = to_dev(np.random.default_rng(9).normal(size=2 * lat.n_sites) * (1 - 1j), cuda)
    o1, o2 = torch.zeros_like(vt), torch.zeros_like(vt)
    D1.apply(o1, vt, Q.OP_D)
    D2.apply(o2, vt, Q.OP_D)
    assert float((o1 - o2).abs().max()) < 1e-14 * float(o1.abs().max())
    th1 = torch.zeros(lat.n_faces, dtype=torch.float64, device=cuda)
    th2 = torch.zeros_like(th1)
    Q.plaquette(lat, to_dev(A, cuda), th1)
    Q.plaquette(lat2, to_dev(A2, cuda), th2)
    assert float((th1 - th2).abs().max()) < 1e-14
    F1, F2 = torch.zeros_like(th1[:0]).new_zeros(lat.n_links), torch.zeros(lat.n_links, dtype=torch.float64, device=cuda)
    eta = vt.clone()
    Q.fermion_force(D1, eta, F1)
    Q.fermion_force(D2, eta, F2)
    sgn = torch.from_numpy(np.where(flip, -1.0, 1.0)).to(cuda)
    assert float((F1 - sgn * F2).abs().max()) < 1e-13 * float(F1.abs().max())


@pytest.mark.parametrize("n", [2, 4])
def test_dirac1f_matches_oracle(cuda, n):
    """Dirac1fonS2's coefficients (u, v tables computed from the lattice) in the
    3-hop kernels: D, D^dag, D^dag D = the oracle's dense matrix_form(U) to
    1e-12; the FP32 solver on it is certified in FP64."""
    import torch
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    rng = np.random.default_rng(70 + n)
    A = rng.uniform(-np.pi, np.pi, g.n_links)
    r, m, M5 = 1.0, 0.3, 0.1
    D = Q.DiracS2Dual(lat, r, M5, one_flavor_mass=m)
    D.update(to_dev(A, cuda))
    M = O.dirac1f_matrix(g, r, m, M5, A)
    v = rand_spinor(rng, g.n_sites)
    for op, ref in ((Q.OP_D, M @ v), (Q.OP_DDAG, M.conj().T @ v), (Q.OP_DDAGD, M.conj().T @ (M @ v))):
        out = torch.zeros(v.size, dtype=torch.complex128, device=cuda)
        D.apply(out, to_dev(v, cuda), op)
        assert rel(from_dev(out), ref) < 1e-12, op
    x = torch.zeros(v.size, dtype=torch.complex128, device=cuda)
    rep = D.solve(x, to_dev(v, cuda), tol=1e-10, precision=Q.PREC_F32)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    assert rel(from_dev(x), np.linalg.solve(M.conj().T @ M, v)) < 1e-7
