"""Learned preconditioner and preconditioned CG on the GPU.

The network is checked against a plain torch restatement on the CPU
(complex64): hop blocks taken from the oracle's CSR matrix of D in reference
order, masked to the solver's site blocks through the lattice permutation.
Gradients are checked against torch autograd of the same loss; the collapsed
word form against the layer form; hermiticity and positivity of N directly;
preconditioned CG against the oracle's CG and the FP64 true residual."""
import ctypes

import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O
from tests.gpu_util import from_dev, rand_spinor, to_dev

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _setup(n, M5=0.05, seed=3):
    rng = np.random.default_rng(seed)
    g = O.geometry(n)
    lat = Q.S2Trivalent(n)
    A = rng.uniform(-np.pi, np.pi, g.n_links)
    Do = O.Dirac(g, 1.0, M5)
    Do.update(A)
    Dq = Q.DiracS2Dual(lat, 1.0, M5)
    Dq.update(A)
    return rng, g, lat, A, Do, Dq


def _csr(Do):
    import scipy.sparse as sp
    L = O.lib()
    nnz = L.orc_dirac_nnz(Do.h)
    rows = np.zeros(Do.N + 1, np.int32)
    cols = np.zeros(nnz, np.int32)
    val = np.zeros(nnz, np.complex128)
    ip = ctypes.POINTER(ctypes.c_int)
    L.orc_dirac_get_csr(Do.h, rows.ctypes.data_as(ip), cols.ctypes.data_as(ip), val.ctypes.data_as(ctypes.c_void_p))
    return sp.csr_matrix((val, cols, rows), shape=(Do.N, Do.N))


class TorchNet:
    """N(r) = a^2 r + G^dag G r restated in torch (CPU, complex64)."""

    def __init__(self, g, Do, perm, per, C, LG, w):
        Ds = _csr(Do)
        Ns = g.n_sites
        nns = np.asarray(g.nns).reshape(Ns, 3)
        iperm = np.argsort(perm)
        blk = iperm // per
        Hb = np.zeros((Ns, 3, 2, 2), complex)
        for x in range(Ns):
            for k in range(3):
                y = nns[x, k]
                Hb[x, k] = Ds[2 * x:2 * x + 2, 2 * y:2 * y + 2].toarray()
        mask = (blk[nns] == blk[:, None]).astype(float)
        Hd = np.zeros_like(Hb)
        Ho = np.zeros_like(Hb)
        Hd[:, :, 0, 0] = Hb[:, :, 0, 0]
        Hd[:, :, 1, 1] = Hb[:, :, 1, 1]
        Ho[:, :, 0, 1] = Hb[:, :, 0, 1]
        Ho[:, :, 1, 0] = Hb[:, :, 1, 0]
        Hd *= mask[:, :, None, None]
        Ho *= mask[:, :, None, None]
        self.Hd = torch.tensor(Hd, dtype=torch.complex64)
        self.Ho = torch.tensor(Ho, dtype=torch.complex64)
        self.nns = torch.tensor(nns, dtype=torch.long)
        A = (Ds.conj().T @ Ds).tocsr()
        self.A = torch.sparse_csr_tensor(torch.tensor(A.indptr, dtype=torch.int64),
                                         torch.tensor(A.indices, dtype=torch.int64),
                                         torch.tensor(A.data, dtype=torch.complex64), size=A.shape)
        self.Ns, self.C, self.LG = Ns, C, LG
        chans = [1] + [C] * LG
        self.Ws = []
        off = 0
        for l in range(LG):
            k = 3 * chans[l + 1] * chans[l]
            W = torch.tensor(w[off:off + k].reshape(3, chans[l + 1], chans[l]), dtype=torch.complex64)
            self.Ws.append(W.requires_grad_(True))
            off += k
        self.a = torch.tensor(float(w[off].real), dtype=torch.float32, requires_grad=True)

    def hops(self, h):
        hn = h[:, self.nns]
        return (torch.einsum("xkab,nxkcb->nxca", self.Hd, hn), torch.einsum("xkab,nxkcb->nxca", self.Ho, hn))

    def layer(self, W, h, adj):
        fa, fb = self.hops(h)
        if adj:
            Wc = W.conj().transpose(1, 2)
            return (torch.einsum("oc,nxca->nxoa", Wc[0], h) + torch.einsum("oc,nxca->nxoa", Wc[1], fa)
                    - torch.einsum("oc,nxca->nxoa", Wc[2], fb))
        return (torch.einsum("oc,nxca->nxoa", W[0], h) + torch.einsum("oc,nxca->nxoa", W[1], fa)
                + torch.einsum("oc,nxca->nxoa", W[2], fb))

    def __call__(self, r):  # r: [B, Ns, 2]
        h = r[:, :, None, :]
        for W in self.Ws:
            h = self.layer(W, h, False)
        for W in reversed(self.Ws):
            h = self.layer(W, h, True)
        return self.a * self.a * r + h[:, :, 0, :]

    def loss(self, R, E):
        Z = self(R)
        B = R.shape[0]
        Zf, Rf, Ef = Z.reshape(B, -1), R.reshape(B, -1), E.reshape(B, -1)
        AZ = (self.A @ Zf.T).T
        zr = (Zf.conj() * Rf).sum(1)
        zAz = (Zf.conj() * AZ).sum(1).real
        er = (Ef.conj() * Rf).sum(1).real
        return (1 - zr.abs() ** 2 / (zAz * er)).mean()


def _net(n, C, LG, seed=5):
    rng, g, lat, A, Do, Dq = _setup(n)
    pc = Q.LearnedPreconditioner(Dq, channels=C, layers=LG, seed=seed)
    info = pc.info()
    w = pc.get_weights()
    assert w.shape == (info["nparams"],)
    tn = TorchNet(g, Do, lat.permutation(), info["block_sites"], C, LG, w)
    return rng, g, lat, Do, Dq, pc, tn


def _crel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("C,LG", [(8, 1), (8, 2), (16, 2), (16, 3)])
def test_lpc_forward_matches_torch(cuda, C, LG):
    """Layer by layer (form 0) and in the solver's collapsed form (form 1,
    up to two layers; the 3-layer 16-channel network of the learned-
    preconditioner configuration runs layer by layer)."""
    rng, g, lat, Do, Dq, pc, tn = _net(8, C, LG)
    if C == 16:
        pc.set_tensor_cores(False)  # FP32 CUDA-core mixing; the tensor-core path is checked below
    Ns = g.n_sites
    B = 3
    r = rand_spinor(rng, Ns, B)
    rt = to_dev(r.reshape(-1), cuda)
    z0 = torch.zeros_like(rt)
    pc.apply(z0, rt, nrhs=B, form=0)
    with torch.no_grad():
        zr = tn(torch.tensor(r.reshape(B, Ns, 2), dtype=torch.complex64)).numpy().reshape(-1)
    assert _crel(from_dev(z0), zr) < 2e-5
    z1 = torch.zeros_like(rt)
    if LG > 2:
        with pytest.raises(Q.Qed3Error):
            pc.apply(z1, rt, nrhs=B, form=1)
        return
    pc.apply(z1, rt, nrhs=B, form=1)
    assert _crel(from_dev(z1), zr) < 2e-5


def test_lpc_hermitian_positive(cuda):
    rng, g, lat, Do, Dq, pc, tn = _net(8, 8, 2)
    Ns = g.n_sites
    u = rand_spinor(rng, Ns)
    v = rand_spinor(rng, Ns)
    ut, vt = to_dev(u, cuda), to_dev(v, cuda)
    Nu, Nv = torch.zeros_like(ut), torch.zeros_like(vt)
    pc.apply(Nu, ut)
    pc.apply(Nv, vt)
    Nu, Nv = from_dev(Nu), from_dev(Nv)
    lhs, rhs = np.vdot(u, Nv), np.vdot(Nu, v)
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
    # <u, N u> >= a^2 |u|^2 > 0
    a2 = pc.get_weights()[-1].real ** 2
    assert np.vdot(u, Nu).real >= a2 * np.vdot(u, u).real * (1 - 1e-5)


@pytest.mark.parametrize("C,LG", [(8, 1), (8, 2), (16, 1), (16, 2), (16, 3)])
def test_lpc_gradient_matches_autograd(cuda, C, LG):
    rng, g, lat, Do, Dq, pc, tn = _net(8, C, LG)
    if LG == 1:
        with pytest.raises(Q.Qed3Error):
            pc.set_tensor_cores(True)  # no 16 -> 16 layer
    else:
        pc.set_tensor_cores(False)  # FP32 kernels against autograd
    Ns = g.n_sites
    B = 4
    R = rand_spinor(rng, Ns, B)
    E = rand_spinor(rng, Ns, B) + 0.5 * R  # <e, r> > 0
    loss_gpu, grad = pc.loss_grad(to_dev(R.reshape(-1), cuda), to_dev(E.reshape(-1), cuda), nrhs=B)
    Rt = torch.tensor(R.reshape(B, Ns, 2), dtype=torch.complex64)
    Et = torch.tensor(E.reshape(B, Ns, 2), dtype=torch.complex64)
    L = tn.loss(Rt, Et)
    L.backward()
    assert abs(loss_gpu - float(L)) < 1e-5 * max(1.0, abs(float(L)))
    gt = np.concatenate([W.grad.numpy().reshape(-1) for W in tn.Ws] + [np.array([float(tn.a.grad)])])
    scale = np.abs(gt).max()
    assert np.abs(grad - gt).max() / scale < 2e-3


def test_lpc_training_lowers_loss_and_pcg_converges(cuda):
    rng, g, lat, A, Do, Dq = _setup(16, M5=0.05, seed=11)
    pc = Q.LearnedPreconditioner(Dq, channels=8, layers=2, seed=1)
    pc.collect(Dq, nsrc=4, seed=7, snapshots=(0, 5, 20, 40))
    assert pc.info()["npairs"] == 16
    hist = pc.train(300, batch=8, lr=3e-3, seed=2)
    assert np.all(np.isfinite(hist))
    assert hist[-30:].mean() < hist[:30].mean() - 0.02
    b = rand_spinor(rng, g.n_sites)
    bt = to_dev(b, cuda)
    x_ref, it_ref, _ = Do.cg(b, tol=1e-10)
    iters = {}
    for prec, flexible in ((Q.PREC_F32, False), (Q.PREC_BF16, False), (Q.PREC_F32, True)):
        xt = torch.zeros_like(bt)
        rep = pc.solve(Dq, xt, bt, tol=1e-10, precision=prec, flexible=flexible)
        assert rep.status == Q.OK
        assert rep.true_rel_res <= 1e-10
        q = torch.zeros_like(bt)
        Dq.apply(q, xt, Q.OP_DDAGD)
        assert float((bt - q).norm() / bt.norm()) <= 1.05e-10
        assert np.linalg.norm(from_dev(xt) - x_ref) / np.linalg.norm(x_ref) < 1e-7
        assert rep.iters < it_ref
        iters[(prec, flexible)] = rep.iters
    # Polak-Ribiere and Fletcher-Reeves beta agree in exact arithmetic
    assert abs(iters[(Q.PREC_F32, True)] - iters[(Q.PREC_F32, False)]) <= max(3, iters[(Q.PREC_F32, False)] // 10)


def test_pcg_untrained_and_shifted(cuda):
    rng, g, lat, A, Do, Dq = _setup(8, M5=0.1, seed=12)
    pc = Q.LearnedPreconditioner(Dq, channels=4, layers=1, seed=3)
    b = rand_spinor(rng, g.n_sites)
    bt = to_dev(b, cuda)
    for shift in (0.0, 0.3):
        x_ref, _, _ = Do.cg(b, tol=1e-11, shift=shift)
        xt = torch.zeros_like(bt)
        rep = pc.solve(Dq, xt, bt, tol=1e-10, precision=Q.PREC_F32, shift=shift)
        assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
        assert np.linalg.norm(from_dev(xt) - x_ref) / np.linalg.norm(x_ref) < 1e-7
    # a zero source returns x = 0 with no iterations
    xt = torch.ones_like(bt)
    rep = pc.solve(Dq, xt, torch.zeros_like(bt), precision=Q.PREC_F32)
    assert rep.status == Q.OK and rep.iters == 0
    assert float(xt.abs().max()) == 0.0


def test_pcg_rejects_fp64_and_other_lattice(cuda):
    rng, g, lat, A, Do, Dq = _setup(8)
    pc = Q.LearnedPreconditioner(Dq, channels=4, layers=1)
    bt = to_dev(rand_spinor(rng, g.n_sites), cuda)
    with pytest.raises(Q.Qed3Error):
        pc.solve(Dq, torch.zeros_like(bt), bt, precision=Q.PREC_F64)
    lat2 = Q.S2Trivalent(4)
    D2 = Q.DiracS2Dual(lat2, 1.0, 0.1)
    D2.update(np.zeros(O.geometry(4).n_links))
    b2 = torch.zeros(2 * lat2.n_sites, dtype=torch.complex128, device=cuda)
    with pytest.raises(Q.Qed3Error):
        pc.solve(D2, torch.zeros_like(b2), b2)


@pytest.mark.parametrize("n,B", [(8, 2), (6, 3)])
def test_lpc_tensor_cores_match_fp32(cuda, n, B):
    """tcgen05 BF16 channel mixing (forward, adjoint, weight gradients) against
    the FP32 CUDA-core kernels, including a partial last 128-row tile (n=6, B=3)."""
    rng, g, lat, Do, Dq, pc, tn = _net(n, 16, 2)
    Ns = g.n_sites
    R = rand_spinor(rng, Ns, B)
    E = rand_spinor(rng, Ns, B) + 0.5 * R
    Rt, Et = to_dev(R.reshape(-1), cuda), to_dev(E.reshape(-1), cuda)
    out = {}
    for tc in (False, True):
        pc.set_tensor_cores(tc)
        z = torch.zeros_like(Rt)
        pc.apply(z, Rt, nrhs=B)
        loss, grad = pc.loss_grad(Rt, Et, nrhs=B)
        out[tc] = (from_dev(z), loss, grad)
    z32, l32, g32 = out[False]
    ztc, ltc, gtc = out[True]
    assert _crel(ztc, z32) < 2e-2
    assert abs(ltc - l32) < 2e-2 * max(1e-3, abs(l32))
    # the 16 -> 16 layer's weights (the tensor-core GEMM's output) and the rest
    assert np.abs(gtc - g32).max() / np.abs(g32).max() < 5e-2
    # layer-2 block (3 x 16 x 16) compared on its own scale
    s2 = slice(3 * 16, 3 * 16 + 3 * 256)
    assert np.abs(gtc[s2] - g32[s2]).max() / np.abs(g32[s2]).max() < 5e-2


def test_lpc_tensor_core_training_n16(cuda):
    rng, g, lat, A, Do, Dq = _setup(16, M5=0.05, seed=11)
    pc = Q.LearnedPreconditioner(Dq, channels=16, layers=2, seed=1)  # tensor cores on by default
    pc.collect(Dq, nsrc=4, seed=7, snapshots=(0, 5, 20, 40))
    hist = pc.train(300, batch=8, lr=3e-3, seed=2)
    assert np.all(np.isfinite(hist))
    assert hist[-30:].mean() < hist[:30].mean() - 0.02
    b = rand_spinor(rng, g.n_sites)
    bt = to_dev(b, cuda)
    _, it_ref, _ = Do.cg(b, tol=1e-10)
    xt = torch.zeros_like(bt)
    rep = pc.solve(Dq, xt, bt, tol=1e-10, precision=Q.PREC_F32)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    assert rep.iters < it_ref


@pytest.mark.parametrize("prec", [Q.PREC_F32])
def test_pipelined_pcg_matches_two_barrier(cuda, prec):
    """The one-barrier pipelined recurrence against the two-barrier PCG: same
    certificate, same solution to the tolerance, iteration counts within a few."""
    rng, g, lat, A, Do, Dq = _setup(16, M5=0.05, seed=13)
    pc = Q.LearnedPreconditioner(Dq, channels=8, layers=2, seed=4)
    pc.collect(Dq, nsrc=2, seed=9, snapshots=(0, 10, 30))
    pc.train(200, batch=6, lr=3e-3, seed=1)
    b = rand_spinor(rng, g.n_sites)
    bt = to_dev(b, cuda)
    x_ref, it_ref, _ = Do.cg(b, tol=1e-10)
    reps = {}
    for pipelined in (False, True):
        for shift in (0.0, 0.2):
            xt = torch.zeros_like(bt)
            rep = pc.solve(Dq, xt, bt, tol=1e-10, precision=prec, shift=shift, pipelined=pipelined)
            assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
            q = torch.zeros_like(bt)
            Dq.apply(q, xt, Q.OP_DDAGD)
            q = q + shift * xt
            assert float((bt - q).norm() / bt.norm()) <= 1.05e-10
            if shift == 0.0:
                assert np.linalg.norm(from_dev(xt) - x_ref) / np.linalg.norm(x_ref) < 1e-7
            reps[(pipelined, shift)] = rep.iters
    for shift in (0.0, 0.2):
        a, c = reps[(False, shift)], reps[(True, shift)]
        assert abs(a - c) <= max(4, a // 20)


@pytest.mark.parametrize("flexible", [False, True])
def test_pcg_scale_invariance(cuda, flexible):
    """b far from unit scale: the preconditioned solve iterates on b / |b| and
    rescales the solution, so FP32/BF16 vectors neither underflow nor overflow."""
    rng, g, lat, A, Do, Dq = _setup(8, M5=0.1, seed=13)
    pc = Q.LearnedPreconditioner(Dq, channels=4, layers=1, seed=4)
    bt = to_dev(rand_spinor(rng, g.n_sites), cuda)
    x1 = torch.zeros_like(bt)
    r1 = pc.solve(Dq, x1, bt, tol=1e-10, precision=Q.PREC_F32, flexible=flexible)
    for scale in (1e-30, 1e30):
        xs = torch.zeros_like(bt)
        rs = pc.solve(Dq, xs, bt * scale, tol=1e-10, precision=Q.PREC_F32, flexible=flexible)
        assert rs.status == Q.OK and rs.true_rel_res <= 1e-10, (scale, rs)
        assert abs(rs.iters - r1.iters) <= 2
        assert float((xs / scale - x1).norm() / x1.norm()) < 1e-8


@pytest.mark.parametrize("prec", [Q.PREC_F32, Q.PREC_BF16])
def test_streaming_pcg_n128_certified(cuda, prec):
    """n=128 (327,680 sites): above what the register-resident solver holds,
    so the preconditioner's blocks become tiles of <= 512 sites walked by a
    persistent grid (k_pcgs).  Trained briefly on pairs of the same lattice;
    certified at 1e-10 and fewer iterations than plain mixed-precision CG."""
    rng = np.random.default_rng(128)
    lat = Q.S2Trivalent(128)
    A, _ = Q.thermalized_links(lat, 1.4, seed=2, ntraj=10, init="uniform", device=cuda)
    D = Q.DiracS2Dual(lat, 1.0, 0.05)
    D.update(A)
    pc = Q.LearnedPreconditioner(D, channels=16, layers=2, seed=1)
    assert pc.info()["block_sites"] <= 512
    pc.collect(D, nsrc=4, seed=3, snapshots=(0, 5, 20, 60))
    pc.train(300, batch=8, lr=3e-3, seed=2)
    b = to_dev(rand_spinor(rng, lat.n_sites), cuda)
    x = torch.zeros_like(b)
    plain = D.solve(x, b, tol=1e-10, precision=prec)
    assert plain.status == Q.OK
    x = torch.zeros_like(b)
    rep = pc.solve(D, x, b, tol=1e-10, precision=prec)
    assert rep.status == Q.OK and rep.true_rel_res <= 1e-10
    q = torch.zeros_like(b)
    D.apply(q, x, Q.OP_DDAGD)
    assert float((b - q).norm() / b.norm()) <= 1.05e-10
    assert rep.iters < plain.iters
