"""Batched persistent solver: several lattices, right-hand sides and shifts in
one cooperative launch, each solution certified by its FP64 true residual and
compared with the oracle's CG (src/dual/matpoly.h:204-267 restated)."""
import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O
from tests.gpu_util import from_dev, to_dev

pytestmark = pytest.mark.gpu


def _systems(cuda, ns=(2, 4, 8), nrhs=(3, 2, 5), seed=50):
    rng = np.random.default_rng(seed)
    out = []
    for n, k in zip(ns, nrhs):
        g = O.geometry(n)
        lat = Q.S2Trivalent(n)
        A = rng.uniform(-np.pi, np.pi, g.n_links)
        M5 = float(rng.uniform(0.02, 0.2))
        Do = O.Dirac(g, 1.0, M5)
        Do.update(A)
        Dq = Q.DiracS2Dual(lat, 1.0, M5)
        Dq.update(A)
        b = rng.normal(size=(k, 2 * g.n_sites)) + 1j * rng.normal(size=(k, 2 * g.n_sites))
        out.append((g, lat, Do, Dq, b))
    return out


@pytest.mark.parametrize("sched", [Q.BATCH_STATIC, Q.BATCH_DYNAMIC])
@pytest.mark.parametrize("prec", [Q.PREC_F64, Q.PREC_F32, Q.PREC_BF16])
@pytest.mark.parametrize("tile,threads", [(1, 256), (2, 128), (4, 256), (8, 128)])
def test_batched_multi_lattice(cuda, prec, tile, threads, sched):
    sy = _systems(cuda)
    batch = Q.Batch([(s[3], s[4].shape[0]) for s in sy], precision=prec, rhs_tile=tile, threads=threads,
                    schedule=sched)
    assert batch.rhs_tile == tile and batch.threads == threads and batch.schedule == sched
    bs = [to_dev(s[4], cuda) for s in sy]
    xs = [b.clone() * 0 for b in bs]
    reps, ms = batch.solve(xs, bs, tol=1e-10, precision=prec)
    k = 0
    for (g, lat, Do, Dq, b), xt in zip(sy, xs):
        x = from_dev(xt)
        for r in range(b.shape[0]):
            rep = reps[k]
            k += 1
            assert rep.status == Q.OK, rep
            assert rep.true_rel_res <= 1e-10
            res = np.linalg.norm(b[r] - Do.apply(x[r], 2)) / np.linalg.norm(b[r])
            assert res <= 1.05e-10, (r, res)
            xr, _, _ = Do.cg(b[r], tol=1e-10)
            assert np.linalg.norm(x[r] - xr) / np.linalg.norm(xr) < 1e-7


def test_batched_shifts_and_autotune(cuda):
    sy = _systems(cuda, ns=(4, 8), nrhs=(4, 3), seed=51)
    batch = Q.Batch([(s[3], s[4].shape[0]) for s in sy], precision=Q.PREC_F32)  # autotuned
    assert batch.rhs_tile in (1, 2, 4, 8) and batch.threads in (128, 256)
    assert batch.schedule in (Q.BATCH_STATIC, Q.BATCH_DYNAMIC)
    shifts = [np.array([0.0, 0.1, 0.5, 2.0]), np.array([0.03, 0.3, 1.0])]
    bs = [to_dev(s[4], cuda) for s in sy]
    xs = [b.clone() * 0 for b in bs]
    reps, ms = batch.solve(xs, bs, shifts=shifts, tol=1e-11, precision=Q.PREC_F32)
    k = 0
    for (g, lat, Do, Dq, b), xt, sh in zip(sy, xs, shifts):
        x = from_dev(xt)
        for r in range(b.shape[0]):
            assert reps[k].status == Q.OK
            k += 1
            res = np.linalg.norm(b[r] - Do.apply(x[r], 2) - sh[r] * x[r]) / np.linalg.norm(b[r])
            assert res <= 1.1e-11


@pytest.mark.parametrize("sched", [Q.BATCH_STATIC, Q.BATCH_DYNAMIC])
def test_batched_zero_rhs_and_noconv(cuda, sched):
    sy = _systems(cuda, ns=(2, 4), nrhs=(2, 1), seed=52)
    batch = Q.Batch([(s[3], s[4].shape[0]) for s in sy], precision=Q.PREC_F32, rhs_tile=2, threads=128,
                    schedule=sched)
    bs = [to_dev(s[4], cuda) for s in sy]
    bs[0][1].zero_()
    xs = [b.clone() + 1 for b in bs]
    reps, _ = batch.solve(xs, bs, tol=1e-10, precision=Q.PREC_F32)
    assert reps[1].status == Q.OK and reps[1].iters == 0 and float(xs[0][1].abs().max()) == 0.0
    assert reps[0].status == Q.OK and reps[2].status == Q.OK
    reps, _ = batch.solve(xs, bs, tol=1e-14, maxiter=4, precision=Q.PREC_F32)
    assert reps[0].status == Q.ERR_NOCONV and reps[0].iters == 4


def test_batched_config_256_rhs(cuda):
    """Batched configuration of the benchmark spec: 256 right-hand sides, 64 on
    each of n = 16, 32, 48, 64, each lattice with its own seeded beta = 1.4
    configuration (pure-gauge HMC) and a mass drawn from U[0.02, 0.2], all
    solved to 1e-10 in ONE persistent launch with autotuned tile shapes; every
    solution certified by its FP64 true residual, recomputed here through the
    apply entry point for a sample of each lattice."""
    import torch
    rng = np.random.default_rng(256)
    systems, bs = [], []
    for n in (16, 32, 48, 64):
        lat = Q.S2Trivalent(n)
        A, _ = Q.thermalized_links(lat, 1.4, seed=300 + n, ntraj=10, init="uniform", device=cuda)
        M5 = float(rng.uniform(0.02, 0.2))
        D = Q.DiracS2Dual(lat, 1.0, M5)
        D.update(A)
        b = rng.normal(size=(64, 2 * lat.n_sites)) + 1j * rng.normal(size=(64, 2 * lat.n_sites))
        systems.append((D, 64))
        bs.append(to_dev(b, cuda))
    batch = Q.Batch(systems, precision=Q.PREC_F32)  # autotuner picks tile and threads
    xs = [torch.zeros_like(b) for b in bs]
    reps, ms = batch.solve(xs, bs, tol=1e-10, precision=Q.PREC_F32)
    assert len(reps) == 256
    assert all(r.status == Q.OK and r.true_rel_res <= 1e-10 for r in reps)
    for (D, _), b, x in zip(systems, bs, xs):
        for r in (0, 63):
            q = torch.zeros_like(b[r])
            D.apply(q, x[r].contiguous(), Q.OP_DDAGD)
            assert float((b[r] - q).norm() / b[r].norm()) <= 1.05e-10


@pytest.mark.parametrize("sched", [Q.BATCH_STATIC, Q.BATCH_DYNAMIC])
def test_batched_graph_capture_replay(cuda, sched):
    """The batched solve captured into a CUDA graph (set_shifts, then launch
    under torch.cuda.graph) and replayed with new right-hand sides written into
    the captured buffers: each replay is bit-identical to an ordinary
    synchronous solve of the same systems and certified against the oracle
    (with the dynamic schedule too: its sums run over fixed tile slots, so
    which block took which tile does not change a bit)."""
    import torch
    sy = _systems(cuda, ns=(4, 8), nrhs=(3, 2), seed=53)
    batch = Q.Batch([(s[3], s[4].shape[0]) for s in sy], precision=Q.PREC_F32, rhs_tile=2, threads=128,
                    schedule=sched)
    shifts = [np.array([0.0, 0.2, 1.0]), np.array([0.05, 0.5])]
    bs = [to_dev(s[4], cuda) for s in sy]
    xs = [torch.zeros_like(b) for b in bs]
    batch.set_shifts(shifts)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        batch.launch(xs, bs, tol=1e-10, stream=side)
    torch.cuda.current_stream().wait_stream(side)
    assert all(r.status == Q.OK for r in batch.reports(stream=side))
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        batch.launch(xs, bs, tol=1e-10, stream=torch.cuda.current_stream())
    rng = np.random.default_rng(54)
    for trial in range(3):
        bnew = [rng.normal(size=b.shape) + 1j * rng.normal(size=b.shape) for b in (s[4] for s in sy)]
        for bt, bn in zip(bs, bnew):
            bt.copy_(to_dev(bn, cuda))
        for x in xs:
            x.fill_(0)
        graph.replay()
        torch.cuda.synchronize()
        reps = batch.reports()
        assert all(r.status == Q.OK and r.true_rel_res <= 1e-10 for r in reps), reps
        xr = [torch.zeros_like(b) for b in bs]
        reps2, _ = batch.solve(xr, bs, shifts=shifts, tol=1e-10, precision=Q.PREC_F32)
        assert [r.iters for r in reps] == [r.iters for r in reps2]
        for x, y in zip(xs, xr):
            assert torch.equal(x, y)
        for (g, lat, Do, Dq, _), x, bn, sh in zip(sy, xs, bnew, shifts):
            xh = from_dev(x)
            for r in range(bn.shape[0]):
                res = np.linalg.norm(bn[r] - Do.apply(xh[r], 2) - sh[r] * xh[r]) / np.linalg.norm(bn[r])
                assert res <= 1.05e-10, (trial, r, res)


@pytest.mark.parametrize("sched", [Q.BATCH_STATIC, Q.BATCH_DYNAMIC])
@pytest.mark.parametrize("scale", [1e-30, 1e30])
def test_batched_scale_invariance(cuda, scale, sched):
    """Right-hand sides far from unit scale: the reduced-precision iterations run
    on b / |b|, so the solution is the unit-scale solution times the scale (to
    the tolerance) instead of an FP32 underflow or overflow."""
    sy = _systems(cuda, ns=(4,), nrhs=(3,), seed=55)
    g, lat, Do, Dq, b = sy[0]
    batch = Q.Batch([(Dq, 3)], precision=Q.PREC_F32, rhs_tile=4, threads=128, schedule=sched)
    bt = to_dev(b, cuda)
    x1 = [bt.clone() * 0]
    reps1, _ = batch.solve(x1, [bt], tol=1e-12, precision=Q.PREC_F32)
    xs = [bt.clone() * 0]
    reps, _ = batch.solve(xs, [bt * scale], tol=1e-12, precision=Q.PREC_F32)
    assert all(r.status == Q.OK and r.true_rel_res <= 1e-12 for r in reps), reps
    assert [r.iters for r in reps] == [r.iters for r in reps1]
    x, xr = from_dev(xs[0]), from_dev(x1[0]) * scale
    assert np.abs(x - xr).max() <= 1e-13 * np.abs(xr).max()
