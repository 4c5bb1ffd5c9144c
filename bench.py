"""Benchmark: D^dag D solves/s to 1e-10 at n=64 on one GB300, plus Dirac-apply GB/s.

Workload (the n=64 configuration of the benchmark spec): dual lattice n=64
(81,920 sites, 122,880 links); links theta ~ U[-pi, pi) (seed 2) smoothed by
50 pure-gauge HMC trajectories at beta=1.4 (compact action); Wilson r=1,
M5=0.05; one complex Gaussian source (seed 7).  A step is one full solve
of D^dag D x = b certified by the FP64 true residual <= 1e-10.  Inputs are
synthetic (seeded), no dataset.

Before the timed region the learned preconditioner is trained on the GPU
(the learned-preconditioner configuration of the spec): 2,000 residual/error
pairs from the plain solver on 40 seeded configurations at beta in
{1.0, 1.4, 2.0} (seeds 100-139, m = 0.05), then Adam steps.  The timed
workload's configuration (seed 2) is not among them.

`value` = solves/s of the learned-preconditioned mixed-precision solver
(device-resident b, x); the plain FP64 / FP32 / BF16 CG solves are timed
beside it (`solvers`, `speedup_vs_plain_f64`).  `e2e` = the same through the
public C-ABI call with b and x in pinned host memory (H2D of b and D2H of x
inside every timed step).  L2 (129 MB) is flushed between timed steps since
the n=64 working set fits in it.

`batched_256` (outside the headline): the multi-lattice batched configuration,
256 right-hand sides (64 on each of n = 16, 32, 48, 64) solved to 1e-10 in one
persistent launch per batch, beside the same 256 solves run one after another.
`multi_rhs_n64`: 64 right-hand sides of the headline operator in one batched
launch, beside the single-right-hand-side learned solver.

--impl reference times the reference's algorithm on the host cores: the
oracle's restatement of MatPoly::solve (src/dual/matpoly.h:204-267) over the
reference CSR operator, OpenMP over rows on every host core.  That arm builds
its workload with the oracle alone (the same seeded recipe: uniform links,
50 pure-gauge HMC trajectories, Gaussian source); it loads nothing of this
project's library.

Baseline legs of our arm (outside the timed region, like `cpu_baseline`):
`ref_gpu_baseline` runs the reference's GPU CG design on the same GPU -- one
thread per CSR row, separate axpy kernels, cuBLAS dot products read back by
the host, allocations per operator call (oracle/ref_gpu_cg.cu, restated from
src/both_3d/gpu_header.h:102-130 and src/both_3d/matpoly.h:62-267) -- over
the reference's CSR operator of the same configuration.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_REFINE = 64
BETA = 1.4
OV_MASS = 0.05  # overlap outer solve: D(m) = (1 - m/2) D_ov + m
M5 = 0.05
TOL = 1e-10
# FP32 solves: an FP64 reliable update when |r| fell 100x since the last one
# (delta = 0.01; each costs two FP64 stencil passes, the slow pipe on this
# GPU); measured: the same iterations as delta = 0.1 with half the updates.
# BF16 halo copies keep delta = 0.1: their rounding (~4e-3) needs the more
# frequent updates (at 0.01 the BF16 solvers stagnate).
RU_DELTA = 0.01


def ru_delta(Q, prec):
    return RU_DELTA if prec == Q.PREC_F32 else 0.1
# DRAM read + write bytes of one k_pcg launch at n=64 from an ncu capture
# (--set full, one launch): the operator and vectors are loaded once, the
# iterations run out of L2.
PCG_DRAM_BYTES_PER_LAUNCH = 53.06e6
METRIC = "D†D solves/s to 1e-10 at n=64: learned-PC mixed vs plain FP64 CG; apply GB/s"
WORKLOAD = ("n=64 dual lattice (81,920 sites), r=1, M5=0.05, links U[-pi,pi) seed 2 + 50 HMC traj beta=1.4, "
            "Gaussian source seed 7, CG on D^dag D to 1e-10 FP64 true residual")


def config(world):
    """The workload description both arms print (identical dicts)."""
    return {"workload": WORKLOAD, "l2": "flushed between timed steps (the n=64 working set is L2-resident)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons during the timed region:
    one `nvidia-smi -lms 100` child streams a line every 100 ms (a fresh
    nvidia-smi per sample takes a few hundred ms and gives only a handful of
    samples over a ~1 s region); stop() ends that child."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._proc = None
        self._t = None

    def start(self):
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                           "--format=csv,noheader,nounits", "-lms", "100"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self._proc = None
            return

        def run():
            for line in self._proc.stdout:
                line = line.strip()
                if line:
                    self.samples.append([v.strip() for v in line.split(",")])

        self._t = threading.Thread(target=run, daemon=True)
        self._t.start()

    def stop(self):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=10)
            except Exception:
                self._proc.kill()
        if self._t:
            self._t.join(timeout=10)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and s[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def make_workload(torch, dev):
    import qed3_gb300 as Q
    lat = Q.S2Trivalent(N_REFINE)
    A, acc = Q.thermalized_links(lat, BETA, seed=2, ntraj=50, init="uniform", device=dev)
    D = Q.DiracS2Dual(lat, 1.0, M5)
    D.update(A)
    b = Q.ParallelRng(lat, 7).gaussian_spinor()
    return Q, lat, A, D, b, acc


def make_workload_oracle():
    """The same seeded configuration built by the oracle alone (its pure-gauge
    HMC and random streams are the product's, pinned to the reference's own
    HMCPureGauge and ParallelRng2): no part of this project's library loads."""
    from oracle import oracle as O
    g = O.geometry(N_REFINE)
    A, acc = O.thermalized_links(g, BETA, 2, 50, init="uniform")
    b = O.Rng(g, 7).gaussian_spinor()
    return g, A, b, acc / 50


def train_preconditioner(torch, Q, lat, D, dev, n_cfg=40, n_src=10, steps=1500):
    """Pairs from the plain solver on n_cfg seeded configurations, then Adam on the GPU."""
    t0 = time.perf_counter()
    pc = Q.LearnedPreconditioner(D, channels=16, layers=2, seed=1)
    Dt = Q.DiracS2Dual(lat, 1.0, M5)
    betas = (1.0, 1.4, 2.0)
    for c in range(n_cfg):
        Ac, _ = Q.thermalized_links(lat, betas[c % 3], seed=100 + c, ntraj=50, init="uniform", device=dev)
        Dt.update(Ac)
        pc.collect(Dt, nsrc=n_src, seed=1000 + c, snapshots=(0, 5, 20, 60, 150))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    hist = pc.train(steps, batch=8, lr=3e-3, seed=2)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    info = pc.info()
    return pc, {"pairs": info["npairs"], "configs": n_cfg, "channels": 16, "layers": 2, "params": info["nparams"],
                "block_sites": info["block_sites"], "adam_steps": steps, "batch": 8,
                "loss_first50": float(np.mean(hist[:50])), "loss_last50": float(np.mean(hist[-50:])),
                "collect_s": t1 - t0, "train_s": t2 - t1}


def tc_training_timing(torch, pc, steps=40, batch=8):
    """Adam steps of the network with its 16 -> 16 channel mixing on the tensor
    cores (tcgen05, BF16 operands, FP32 accumulation) and on FP32 CUDA cores;
    the trained weights are restored afterwards."""
    w0 = pc.get_weights()
    out = {}
    for name, on in (("tcgen05_bf16", True), ("cuda_core_fp32", False)):
        pc.set_tensor_cores(on)
        pc.train(3, batch=batch, seed=9)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pc.train(steps, batch=batch, seed=9)
        torch.cuda.synchronize()
        out[name] = {"ms_per_adam_step": 1e3 * (time.perf_counter() - t0) / steps}
        pc.set_weights(w0)
    pc.set_tensor_cores(True)
    out["speedup"] = out["cuda_core_fp32"]["ms_per_adam_step"] / out["tcgen05_bf16"]["ms_per_adam_step"]
    out["config"] = f"batch {batch} residual/error pairs per step (forward, backward, Adam), n=64, 16 channels"
    return out


def host_pcg_iterations(torch, Q, D, pc, b, tol=TOL, maxiter=3000):
    """Iterations of a host-driven flexible PCG (FP64 vectors, Polak-Ribiere
    beta) with the network applied layer by layer (any depth), for comparing
    networks by iteration count outside the persistent solver."""
    x = torch.zeros_like(b)
    r = b.clone()
    z = torch.empty_like(b)
    q = torch.empty_like(b)
    pc.apply(z, r)
    p = z.clone()
    rz = torch.vdot(r, z).real
    bn = float(b.norm())
    for k in range(1, maxiter + 1):
        D.apply(q, p, Q.OP_DDAGD)
        al = rz / torch.vdot(p, q).real
        x += al * p
        r_new = r - al * q
        if float(r_new.norm()) <= tol * bn:
            break
        pc.apply(z, r_new)
        beta = torch.vdot(z, r_new - r).real / rz
        p = z + beta * p
        r = r_new
        rz = torch.vdot(r, z).real
    D.apply(q, x, Q.OP_DDAGD)
    return k, float((b - q).norm()) / bn


def network_depth_study(torch, Q, lat, D, pc2, dev, seeds=3):
    """The learned-preconditioner configuration names a 3-layer, 16-channel
    network; the solver runs the 2-layer one.  Trains the 3-layer network on
    the same pairs recipe and compares iteration counts of the two networks
    (host-driven flexible PCG, layer-by-layer application) on the benchmark
    configuration with several sources."""
    t0 = time.perf_counter()
    pc3 = Q.LearnedPreconditioner(D, channels=16, layers=3, seed=1)
    pc3.set_tensor_cores(True)  # its 16 -> 16 layers on tcgen05, as the 2-layer network's
    Dt = Q.DiracS2Dual(lat, 1.0, M5)
    betas = (1.0, 1.4, 2.0)
    for c in range(40):
        Ac, _ = Q.thermalized_links(lat, betas[c % 3], seed=100 + c, ntraj=50, init="uniform", device=dev)
        Dt.update(Ac)
        pc3.collect(Dt, nsrc=10, seed=1000 + c, snapshots=(0, 5, 20, 60, 150))
    hist = pc3.train(1500, batch=8, lr=3e-3, seed=2)
    torch.cuda.synchronize()
    out = {"train_s": time.perf_counter() - t0, "loss_last50": float(np.mean(hist[-50:])),
           "params_3layer": pc3.info()["nparams"], "params_2layer": pc2.info()["nparams"], "cases": [],
           "solver_words": {"layers2": 7, "layers3": 15}}
    # the network acts with the hop blocks of the operator it was created on
    # (the benchmark configuration): several sources on that configuration
    for src in (7,) + tuple(50 + s for s in range(seeds)):
        b = torch.from_numpy(Q.ParallelRng(lat, src).gaussian_spinor()).to(dev)
        row = {"source_seed": src}
        for name, p_ in (("layers2", pc2), ("layers3", pc3)):
            it, res = host_pcg_iterations(torch, Q, D, p_, b)
            row[name] = {"iters": it, "true_rel_res": res}
        out["cases"].append(row)
    out["iters_3_over_2"] = float(np.mean([c["layers3"]["iters"] / c["layers2"]["iters"] for c in out["cases"]]))
    return out


def heldout_iterations(torch, Q, lat, pc, dev, n=20):
    """Plain (FP64 and mixed) vs preconditioned mixed CG on 20 held-out
    configurations and sources, none used in training."""
    Dt = Q.DiracS2Dual(lat, 1.0, M5)
    out = []
    betas = (1.0, 1.4, 2.0)
    for s in range(n):
        Ac, _ = Q.thermalized_links(lat, betas[s % 3], seed=5000 + s, ntraj=50, init="uniform", device=dev)
        Dt.update(Ac)
        b = torch.from_numpy(Q.ParallelRng(lat, 50 + s).gaussian_spinor()).to(dev)
        x = torch.zeros_like(b)
        r64 = Dt.solve(x, b, tol=TOL, precision=Q.PREC_F64)
        r0 = Dt.solve(x, b, tol=TOL, precision=Q.PREC_F32, delta=RU_DELTA)
        r1 = pc.solve(Dt, x, b, tol=TOL, precision=Q.PREC_F32, delta=RU_DELTA)
        out.append({"beta": betas[s % 3], "seed": 5000 + s, "cg_f64_iters": r64.iters, "cg_f32_iters": r0.iters,
                    "pcg_f32_iters": r1.iters, "cg_f64_ms": r64.ms, "cg_f32_ms": r0.ms, "pcg_f32_ms": r1.ms,
                    "certified": r1.status == Q.OK and r1.true_rel_res <= TOL})
    return out


def heldout_summary(rows):
    g = lambda k: np.array([r[k] for r in rows], dtype=np.float64)
    return {"seeds": len(rows), "all_certified": all(r["certified"] for r in rows),
            "iters_pcg_over_cg": float(np.mean(g("pcg_f32_iters") / g("cg_f32_iters"))),
            "speedup_vs_cg_f32": float(np.mean(g("cg_f32_ms") / g("pcg_f32_ms"))),
            "speedup_vs_cg_f64": float(np.mean(g("cg_f64_ms") / g("pcg_f32_ms")))}


def flush_l2(torch, buf):
    buf.add_(1.0)


def time_solver(torch, Q, D, bt, prec, steps, warmup, flush, pc=None):
    """Per-step CUDA-event timing of device-resident solves (flush outside the events)."""
    st = torch.cuda.current_stream()
    x = torch.zeros_like(bt)
    reps = []

    def solve():
        if pc is not None:
            return pc.solve(D, x, bt, tol=TOL, precision=prec, delta=ru_delta(Q, prec))
        return D.solve(x, bt, tol=TOL, precision=prec, delta=ru_delta(Q, prec))

    for _ in range(warmup):
        solve()
    ms = []
    for _ in range(steps):
        flush_l2(torch, flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        rep = solve()
        e1.record(st)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        reps.append(rep)
    return ms, reps, x


def apply_bandwidth(torch, Q, n, prec, reps=50):
    """Device-internal D apply on an HBM-resident lattice; algorithmic bytes / time."""
    lat = Q.S2Trivalent(n)
    D = Q.DiracS2Dual(lat, 1.0, M5)
    A = torch.from_numpy(np.random.default_rng(3).uniform(-np.pi, np.pi, lat.n_links)).cuda()
    D.update(A)
    nb = D.field_bytes(prec, 1)
    fin = torch.zeros(nb, dtype=torch.uint8, device="cuda")
    fout = torch.zeros_like(fin)
    for _ in range(5):
        D.apply_field(fout, fin, Q.OP_D, prec)
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        D.apply_field(fout, fin, Q.OP_D, prec)
    e1.record(st)
    e1.synchronize()
    t = e0.elapsed_time(e1) / reps * 1e-3
    per_site = {Q.PREC_F64: 276, Q.PREC_F32: 144, Q.PREC_BF16: 128}[prec]
    gbs = per_site * lat.n_sites / t / 1e9
    return {"n": n, "prec": {0: "f64", 1: "f32", 2: "bf16"}[prec], "us": t * 1e6, "GB/s": gbs,
            "bytes_per_site": per_site}


def cpu_reference_solve(b, A, g=None):
    """The reference's algorithm on the host cores (oracle restatement)."""
    from oracle import oracle as O
    g = g or O.geometry(N_REFINE)
    D = O.Dirac(g, 1.0, M5)
    D.update(A)
    t = time.perf_counter()
    x, it, mu = D.cg(b, tol=TOL)
    dt = time.perf_counter() - t
    r = b - D.apply(x, 2)
    return dt, it, float(np.linalg.norm(r) / np.linalg.norm(b)), O.num_threads()


def _wall(torch, fn, reps):
    """Median wall time of fn() (host-driven paths: trajectories, host-looped CG)."""
    ts = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    return float(np.median(ts))


def paths_timings(torch, Q, dev, cpu=True):
    """The paths around the solver on the GPU, each beside the oracle's CPU
    restatement of the reference algorithm on the host cores (one bounded
    sample): Wilson-fermion HMC trajectory (n=16), overlap apply (n=16, order
    21), the S^2 x S^1 operator apply (n=64, Nt=16; HBM-resident, roofline),
    its FP64 CG (n=16, Nt=8) and HMC trajectory (n=8, Nt=8)."""
    from oracle import oracle as O
    peak, peak_kind = peaks()
    out = {}
    cores = O.num_threads()
    # -- Wilson-fermion HMC trajectory, ExplicitLeapfrogML, one pseudofermion
    n = 16
    lat = Q.S2Trivalent(n)
    A0, _ = Q.thermalized_links(lat, BETA, seed=3, ntraj=20, init="uniform", device=dev)
    D = Q.DiracS2Dual(lat, 1.0, 0.1)
    D.update(A0)
    kw = dict(tmax=1.0, nsteps=5, nsteps_inner=4, tol=1e-10)
    rng = Q.ParallelRng(lat, 11)
    A = A0.clone()
    its = []
    gpu_s = _wall(torch, lambda: its.append(Q.hmc_fermion(lat, D, rng, A, BETA, **kw)[2]), 4)
    row = {"gpu_ms": 1e3 * gpu_s, "cg_iters": its[-1], "config": "n=16, beta=1.4, r=1, M5=0.1, tau=1, 5 x 4 steps, "
           "tol 1e-10 (mixed FP32 solves, FP64 certificate)"}
    g = O.geometry(n) if cpu else None
    if cpu:
        Do = O.Dirac(g, 1.0, 0.1)
        Ao = A0.cpu().numpy().copy()
        t0 = time.perf_counter()
        O.hmc_fermion(g, Do, O.Rng(g, 11), Ao, BETA, **kw)
        row["cpu_baseline"] = {"ms": 1e3 * (time.perf_counter() - t0), "cores": cores, "kind": "port",
                               "sample": "one trajectory, same parameters, FP64 CSR CG"}
        row["gpu_vs_cpu"] = row["cpu_baseline"]["ms"] / row["gpu_ms"]
    out["hmc_fermion_n16"] = row
    # -- overlap apply (M5 = -1, Zolotarev order 41 = 20 poles, bounds from the operator update)
    Dw = Q.DiracS2Dual(lat, 1.0, -1.0)
    Dw.update(A0)
    ov = Q.Overlap(Dw, order=41)
    ov.update()
    inf = ov.info()
    v = torch.from_numpy(Q.ParallelRng(lat, 5).gaussian_spinor()).to(dev)
    w = torch.empty_like(v)
    gpu_s = _wall(torch, lambda: ov.apply(w, v, tol_inner=1e-10), 5)
    row = {"gpu_ms": 1e3 * gpu_s, "k": inf["k"], "config": "n=16, M5=-1, order 41 (20 poles), inner tol 1e-10 "
           "(all poles in one FP64 multi-shift CG)"}
    if cpu:
        Dow = O.Dirac(g, 1.0, -1.0)
        Dow.update(A0.cpu().numpy())
        vh = v.cpu().numpy()
        t0 = time.perf_counter()
        Dow.overlap(vh, inf["lambda_min"], inf["lambda_max"], 41, 0, 1e-10)
        row["cpu_baseline"] = {"ms": 1e3 * (time.perf_counter() - t0), "cores": cores, "kind": "port",
                               "sample": "one apply, one CG per pole"}
        row["gpu_vs_cpu"] = row["cpu_baseline"]["ms"] / row["gpu_ms"]
    out["overlap_apply_n16"] = row
    # -- S^2 x S^1 operator apply: HBM-resident at n=64, Nt=16
    n, Nt, at = 64, 16, 0.5
    lat = Q.S2Trivalent(n)
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, at)
    gen = torch.Generator(device=dev)
    gen.manual_seed(4)
    Ae = (torch.rand(Nt * (lat.n_links + lat.n_sites), dtype=torch.float64, device=dev, generator=gen) * 2 - 1) * np.pi
    De.update(Ae)
    ve = torch.randn(Nt * 2 * lat.n_sites, dtype=torch.complex128, device=dev, generator=gen)
    we = torch.empty_like(ve)
    st = torch.cuda.current_stream()
    for _ in range(3):
        De.apply(we, ve, Q.OP_D)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 20
    e0.record(st)
    for _ in range(reps):
        De.apply(we, ve, Q.OP_D)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / reps
    # per site and slice: spinor in 32 + out 32 + 3 slice hop blocks 192 + temporal angle 8,
    # plus the per-site tables (neighbours 12, permutation 4, diagonal 8, kappa_t 8) once per site
    bps = 32 + 32 + 192 + 8 + 32.0 / Nt
    gbs = bps * lat.n_sites * Nt / (ms * 1e-3) / 1e9
    row = {"gpu_ms": ms, "GB/s": gbs, "bytes_per_site_slice": bps, "frac_of_" + peak_kind: gbs / peak,
           "bound": "fp64 pipe (ncu: sm__pipe_fp64_cycles_active 92.5%, dram 22%)",
           "config": "n=64, Nt=16 (1.31M site-slices, 252 MB of hop blocks: HBM-resident), FP64, D"}
    if cpu:
        g = O.geometry(n)
        Ah, vh = Ae.cpu().numpy(), ve.cpu().numpy()
        t0 = time.perf_counter()
        O.dirac_ext_apply(g, 1.0, 0.1, Nt, at, Ah, vh, 0)
        row["cpu_baseline"] = {"ms": 1e3 * (time.perf_counter() - t0), "cores": cores, "kind": "port",
                               "sample": "one D apply (per-slice CSR restatement incl. its per-slice link update)"}
        row["gpu_vs_cpu"] = row["cpu_baseline"]["ms"] / row["gpu_ms"]
    out["ext_apply_n64_nt16"] = row
    # the same operator's FP64 and mixed-precision solve at the apply's size (FP64-pipe bound)
    be = torch.randn(Nt * 2 * lat.n_sites, dtype=torch.complex128, device=dev, generator=gen)
    xe = torch.empty_like(be)
    Ae.mul_(0.2)  # a smoother field: a few hundred iterations
    De.update(Ae)
    solves = {}
    for name, prec in (("f64", Q.PREC_F64), ("f32_mixed", Q.PREC_F32)):
        rr = []
        t_ = _wall(torch, lambda: rr.append(De.solve(xe, be, tol=1e-10, precision=prec)), 2)
        solves[name] = {"gpu_ms": 1e3 * t_, "iters": rr[-1].iters, "reliable_updates": rr[-1].reliable_updates,
                        "true_rel_res": rr[-1].true_rel_res}
    out["ext_cg_n64_nt16"] = dict(solves, config="n=64, Nt=16, at=0.5, links 0.2 U[-pi,pi), tol 1e-10, "
                                  "certified by the FP64 true residual")
    del De, Ae, ve, we, be, xe
    # -- S^2 x S^1 FP64 CG on D^dag D and the S^2 x S^1 HMC trajectory
    n, Nt, at = 16, 8, 0.5
    lat = Q.S2Trivalent(n)
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, at)
    Ae = (torch.rand(Nt * (lat.n_links + lat.n_sites), dtype=torch.float64, device=dev, generator=gen) - 0.5) * 0.6
    De.update(Ae)
    be = torch.randn(Nt * 2 * lat.n_sites, dtype=torch.complex128, device=dev, generator=gen)
    xe = torch.empty_like(be)
    reps_ = []
    gpu_s = _wall(torch, lambda: reps_.append(De.solve(xe, be, tol=1e-10)), 3)
    rm = []
    gpu_m = _wall(torch, lambda: rm.append(De.solve(xe, be, tol=1e-10, precision=Q.PREC_F32)), 3)
    row = {"gpu_ms": 1e3 * gpu_s, "iters": reps_[-1].iters, "true_rel_res": reps_[-1].true_rel_res,
           "mixed_f32": {"gpu_ms": 1e3 * gpu_m, "iters": rm[-1].iters, "reliable_updates": rm[-1].reliable_updates,
                         "true_rel_res": rm[-1].true_rel_res},
           "config": "n=16, Nt=8, at=0.5, links 0.6 U[-0.5,0.5), tol 1e-10; FP64 and FP32 + FP64 reliable updates"}
    if cpu:
        g = O.geometry(n)
        Ah, bh = Ae.cpu().numpy(), be.cpu().numpy()
        k = 10
        t0 = time.perf_counter()
        for _ in range(k):
            O.dirac_ext_apply(g, 1.0, 0.1, Nt, at, Ah, bh, 2)
        per = (time.perf_counter() - t0) / k
        row["cpu_baseline"] = {"ms": 1e3 * per * reps_[-1].iters, "cores": cores, "kind": "port",
                               "sample": f"{k} D^dag D applications of the restatement, times the GPU's "
                                         "iteration count (vector updates not counted)"}
        row["gpu_vs_cpu"] = row["cpu_baseline"]["ms"] / row["gpu_ms"]
    out["ext_cg_n16_nt8"] = row
    n, Nt = 8, 8
    lat = Q.S2Trivalent(n)
    De = Q.DiracExt(lat, 1.0, 0.1, Nt, at)
    Ae = (torch.rand(Nt * (lat.n_links + lat.n_sites), dtype=torch.float64, device=dev, generator=gen) - 0.5) * 0.6
    rng = Q.ParallelRng(lat, 21, n_slices=Nt)
    res = []
    gpu_s = _wall(torch, lambda: res.append(Q.hmc_ext(De, rng, Ae, 1.0, tmax=0.5, nsteps=4, nsteps_inner=4,
                                                       tol=1e-10)), 3)
    res32 = []
    gpu_m = _wall(torch, lambda: res32.append(Q.hmc_ext(De, rng, Ae, 1.0, tmax=0.5, nsteps=4, nsteps_inner=4,
                                                         tol=1e-10, precision=Q.PREC_F32)), 3)
    out["hmc_ext_n8_nt8"] = {"gpu_ms": 1e3 * gpu_s, "cg_iters": res[-1][2], "accepted": [r[0] for r in res],
                             "mixed_f32": {"gpu_ms": 1e3 * gpu_m, "cg_iters": res32[-1][2],
                                           "accepted": [r[0] for r in res32]},
                             "config": "n=8, Nt=8, at=0.5, g^2=1, tau=0.5, 4 x 4 steps, tol 1e-10; FP64 solves, "
                                       "then FP32 + FP64 reliable updates",
                             "cpu_baseline": None, "cpu_note": "the oracle's S^2 x S^1 HMC runs on a dense "
                             "operator (checked at n=2); no CPU sample at this size"}
    # -- overlap of the S^2 x S^1 operator (M5 = -1, order 21), Lanczos bounds
    Dw = Q.DiracExt(lat, 1.0, -1.0, Nt, at)
    Dw.update(Ae)
    ovx = Q.OverlapExt(Dw, 21)
    t_up = _wall(torch, lambda: ovx.update(tol=1e-10), 1)
    inf = ovx.info()
    ve = torch.randn(Nt * 2 * lat.n_sites, dtype=torch.complex128, device=dev, generator=gen)
    we = torch.empty_like(ve)
    pits = []
    t_ap = _wall(torch, lambda: pits.append(ovx.apply(we, ve, Q.OP_D, tol_inner=1e-10)), 3)
    out["overlap_ext_n8_nt8"] = {"gpu_ms": 1e3 * t_ap, "pole_iters": pits[-1], "lanczos_update_ms": 1e3 * t_up,
                                 "k": inf["k"], "config": "n=8, Nt=8, M5=-1, order 21 (10 poles, one FP64 "
                                 "multi-shift CG), inner tol 1e-10", "cpu_baseline": None,
                                 "cpu_note": "the oracle's S^2 x S^1 overlap is dense (checked at n=2)"}
    return out


def learned_hbm(torch, Q, dev, n=256, reps=3):
    """The learned preconditioner on an HBM-resident lattice: n=256 (1,310,720
    sites; ~0.4 GB of FP32 operator and state), where the preconditioned
    solver streams its state through HBM tile by tile (k_pcgs).  Links
    U[-pi,pi) seed 2 + 10 pure-gauge HMC trajectories at beta=1.4, M5=0.05,
    Gaussian source seed 7; the network (16 channels, 2 layers) is trained on
    pairs from this lattice (4 configurations x 4 sources, 400 Adam steps).
    Plain FP64 CG, plain mixed CG and the learned solver, each certified."""
    t0 = time.perf_counter()
    lat = Q.S2Trivalent(n)
    A, _ = Q.thermalized_links(lat, BETA, seed=2, ntraj=10, init="uniform", device=dev)
    D = Q.DiracS2Dual(lat, 1.0, M5)
    D.update(A)
    pc = Q.LearnedPreconditioner(D, channels=16, layers=2, seed=1)
    Dt = Q.DiracS2Dual(lat, 1.0, M5)
    for c in range(4):
        Ac, _ = Q.thermalized_links(lat, (1.0, 1.4, 2.0, 1.4)[c], seed=700 + c, ntraj=10, init="uniform", device=dev)
        Dt.update(Ac)
        pc.collect(Dt, nsrc=4, seed=900 + c, snapshots=(0, 5, 20, 60, 150))
    pc.train(400, batch=8, lr=3e-3, seed=2)
    torch.cuda.synchronize()
    out = {"n": n, "sites": lat.n_sites, "block_sites": pc.info()["block_sites"], "setup_s": time.perf_counter() - t0}
    b = torch.from_numpy(Q.ParallelRng(lat, 7).gaussian_spinor()).to(dev)
    x = torch.zeros_like(b)
    st = torch.cuda.current_stream()
    for name, fn in (("cg_f64", lambda: D.solve(x, b, tol=TOL, precision=Q.PREC_F64)),
                     ("cg_f32", lambda: D.solve(x, b, tol=TOL, precision=Q.PREC_F32, delta=RU_DELTA)),
                     ("pcg_f32", lambda: pc.solve(D, x, b, tol=TOL, precision=Q.PREC_F32, delta=RU_DELTA))):
        fn()
        ms, rep = [], None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            rep = fn()
            e1.record(st)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        out[name] = {"ms": float(np.mean(ms)), "iters": rep.iters, "true_rel_res": rep.true_rel_res,
                     "certified": rep.status == Q.OK and rep.true_rel_res <= TOL}
    out["speedup_vs_cg_f64"] = out["cg_f64"]["ms"] / out["pcg_f32"]["ms"]
    out["speedup_vs_cg_f32"] = out["cg_f32"]["ms"] / out["pcg_f32"]["ms"]
    # the streaming kernel's HBM bytes: D^dag D at 288 B/site + 7 FP32 state streams at 16 B
    gbs = 400 * lat.n_sites * out["pcg_f32"]["iters"] / (out["pcg_f32"]["ms"] * 1e-3) / 1e9
    peak, kind = peaks()
    out["pcg_roofline"] = {"kernel": "k_pcgs<F32,7>", "GB/s": gbs, "frac_of_" + kind: gbs / peak,
                           "bytes_per_site_iter": 400, "resident": "HBM"}
    return out


def topological_charge(torch, Q, lat, A):
    """Q = sum over dual faces of the plaquette angle wrapped to (-pi, pi], / 2 pi."""
    th = torch.empty(lat.n_faces, dtype=torch.float64, device=A.device)
    Q.plaquette(lat, A, th)
    return float(torch.remainder(th + np.pi, 2 * np.pi).sub(np.pi).sum()) / (2 * np.pi)


def dense_sign_error(torch, Q, dev, nev=16):
    """Sign-function check of the overlap configuration at n=8: D_ov from the
    dense FP64 eigendecomposition of H = gamma5 D_W (numpy eigh; D_W taken
    column by column from this library's apply) against the GPU D_ov (20
    poles), with and without the low-mode projection."""
    n = 8
    lat = Q.S2Trivalent(n)
    A, _ = Q.thermalized_links(lat, BETA, seed=2, ntraj=50, init="uniform", device=dev)
    D = Q.DiracS2Dual(lat, 1.0, -1.0)
    D.update(A)
    N = 2 * lat.n_sites
    E = torch.eye(N, dtype=torch.complex128, device=dev)
    M = torch.empty_like(E)
    for j in range(N):
        D.apply(M[j], E[j], Q.OP_D)  # row j of M = D e_j, i.e. column j of D
    Mh = M.T.cpu().numpy()
    g5 = np.tile([1.0, -1.0], N // 2)
    w, V = np.linalg.eigh(g5[:, None] * Mh)
    Dex = np.eye(N) + g5[:, None] * ((V * np.sign(w)) @ V.conj().T)
    ov = Q.Overlap(D, order=41)
    ov.update_lanczos()
    xi = np.random.default_rng(3).normal(size=N) + 1j * np.random.default_rng(4).normal(size=N)
    xt = torch.from_numpy(xi).to(dev)
    y = torch.empty_like(xt)
    ref = Dex @ xi
    out = {"n": n, "charge": topological_charge(torch, Q, lat, A), "dense": "numpy eigh of gamma5 D_W, FP64"}
    for nev_ in (0, nev):
        info = ov.project_low_modes(nev_)
        ov.apply(y, xt, Q.OP_D, tol_inner=1e-12)
        out[f"nev{nev_}"] = {"k": info["k"], "delta": info["delta"],
                             "rel_err_D_ov": float(np.abs(y.cpu().numpy() - ref).max() / np.abs(ref).max())}
    return out


def overlap_config(torch, Q, dev, nev=48):
    """The overlap configuration: n=32 (20,480 sites), links U[-pi,pi) seed 2 +
    50 pure-gauge HMC trajectories at beta=1.4, M5=-1, Zolotarev order 41 (20
    poles), outer solve of the propagator right-hand side to 1e-10 (certified
    with certified pole solves).  The configuration carries topological
    charge, so the massless D_ov^dag D_ov is singular (|Q| exact zero modes)
    and its near-zero modes make the outer CG ill-conditioned: the massless
    solve is reported after a fixed budget, the certified solve is that of
    the massive overlap D(m) = (1 - m/2) D_ov + m, m = 0.05.  The nev
    eigenmodes of gamma5 D_W nearest zero are treated exactly in the sign
    function (qed3_overlap_project_low_modes) and the outer CG runs per
    chirality sector."""
    n = 32
    lat = Q.S2Trivalent(n)
    A, _ = Q.thermalized_links(lat, BETA, seed=2, ntraj=50, init="uniform", device=dev)
    D = Q.DiracS2Dual(lat, 1.0, -1.0)
    D.update(A)
    ov = Q.Overlap(D, order=41)
    out = {"config": "n=32, beta=1.4 seed 2 (50 HMC trajectories from U[-pi,pi)), M5=-1, order 41 (20 poles), "
                     "outer CG on D_ov^dag D_ov to 1e-10, pole solves to 1e-12",
           "charge": topological_charge(torch, Q, lat, A)}
    out["bounds_s"] = _wall(torch, lambda: ov.update_lanczos(), 1)
    i0 = ov.info()
    out["unprojected"] = {"k": i0["k"], "delta": i0["delta"]}
    xi = torch.from_numpy(Q.ParallelRng(lat, 5).gaussian_spinor()).to(dev)
    y = torch.empty_like(xi)
    reps = []
    out["unprojected"]["apply_D_ms"] = 1e3 * _wall(torch, lambda: reps.append(ov.apply(y, xi, Q.OP_D,
                                                                                     tol_inner=1e-12)), 2)
    out["unprojected"]["pole_iters"] = reps[-1].iters
    info = {}
    out["project_s"] = _wall(torch, lambda: info.update(ov.project_low_modes(nev)), 1)
    out["projected"] = {"nev": nev, "k": info["k"], "delta": info["delta"], "max_residual": info["max_residual"],
                        "lanczos_applies": info["lanczos_steps"]}
    reps = []
    out["projected"]["apply_D_ms"] = 1e3 * _wall(torch, lambda: reps.append(ov.apply(y, xi, Q.OP_D,
                                                                                   tol_inner=1e-12)), 3)
    out["projected"]["pole_iters"] = reps[-1].iters
    # the same product with every pole its own mixed-precision CG (FP32 iterations,
    # FP64 reliable updates and certificates) in one batched launch
    ov.set_pole_solver(Q.POLES_BATCHED)
    reps = []
    out["projected"]["apply_D_ms_batched_mixed"] = 1e3 * _wall(
        torch, lambda: reps.append(ov.apply(y, xi, Q.OP_D, tol_inner=1e-12)), 3)
    out["projected"]["batched_mixed_worst_true_res"] = reps[-1].true_rel_res
    ov.set_pole_solver(Q.POLES_MULTISHIFT)
    b = torch.empty_like(xi)
    x = torch.zeros_like(b)
    # the massless outer solve within a fixed budget: singular (|Q| zero modes) and ill-conditioned
    ov.apply(b, xi, Q.OP_DDAG, tol_inner=1e-12)
    rr = []
    t = _wall(torch, lambda: rr.append(ov.solve(x, b, tol=TOL, tol_inner=1e-12, maxiter=400)), 1)
    out["outer_solve_massless_400_iters"] = {"s": t, "iters": rr[-1].iters, "true_rel_res": rr[-1].true_rel_res}
    # the massive overlap D(m) = (1 - m/2) D_ov + m, m = 0.05, per chirality sector, to 1e-10
    ov.set_mass(OV_MASS)
    ov.apply(b, xi, Q.OP_DDAG, tol_inner=1e-12)
    rr = []
    t = _wall(torch, lambda: rr.append(ov.solve(x, b, tol=TOL, tol_inner=1e-12, maxiter=20000,
                                                 flags=Q.OVSOLVE_CHIRAL)), 1)
    out["outer_solve"] = {"s": t, "iters": rr[-1].iters, "true_rel_res": rr[-1].true_rel_res,
                          "certified": rr[-1].status == Q.OK and rr[-1].true_rel_res <= TOL,
                          "max_pole_iters": rr[-1].reliable_updates, "mode": "chirality sectors",
                          "mass": OV_MASS}
    out["sign_check_n8"] = dense_sign_error(torch, Q, dev)
    return out


def batched_throughput(torch, Q, dev, reps=3):
    """The multi-lattice batched configuration: 256 right-hand sides, 64 on each
    of n = 16, 32, 48, 64 (each with its own beta = 1.4 configuration and a mass
    from U[0.02, 0.2]), solved to 1e-10 in ONE persistent launch per batch, vs
    the same 256 solves one after another with the single-system solver."""
    rng = np.random.default_rng(256)
    systems, bs = [], []
    for n in (16, 32, 48, 64):
        lat_n = Q.S2Trivalent(n)
        A_n, _ = Q.thermalized_links(lat_n, BETA, seed=300 + n, ntraj=10, init="uniform", device=dev)
        D_n = Q.DiracS2Dual(lat_n, 1.0, float(rng.uniform(0.02, 0.2)))
        D_n.update(A_n)
        b_n = rng.normal(size=(64, 2 * lat_n.n_sites)) + 1j * rng.normal(size=(64, 2 * lat_n.n_sites))
        systems.append((D_n, 64))
        bs.append(torch.from_numpy(b_n).to(dev))
    batch = Q.Batch(systems, precision=Q.PREC_F32)
    xs = [torch.zeros_like(b_) for b_ in bs]
    ms_b, ok, iters, rus = [], True, 0, 0
    for i in range(reps + 1):
        reps_, ms = batch.solve(xs, bs, tol=TOL, precision=Q.PREC_F32, delta=RU_DELTA)
        ok = ok and all(r.status == Q.OK and r.true_rel_res <= TOL for r in reps_)
        iters = max(iters, max(r.iters for r in reps_))
        rus = max(rus, max(r.reliable_updates for r in reps_))
        if i > 0:
            ms_b.append(ms)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    seq_ok = True
    for (D_n, _), b_ in zip(systems, bs):
        x_ = torch.zeros_like(b_[0])
        for r in range(64):
            rep = D_n.solve(x_, b_[r].contiguous(), tol=TOL, precision=Q.PREC_F32, delta=RU_DELTA)
            seq_ok = seq_ok and rep.status == Q.OK
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t0
    ms = float(np.mean(ms_b))
    return {"rhs": 256, "lattices": [16, 32, 48, 64], "rhs_tile": batch.rhs_tile, "threads": batch.threads,
            "blocks": batch.blocks, "schedule": {Q.BATCH_STATIC: "static", Q.BATCH_DYNAMIC: "dynamic"}[batch.schedule],
            "reliable_update_delta": RU_DELTA, "max_reliable_updates": rus,
            "ms_per_batch": ms, "solves_per_s": 256e3 / ms, "max_iters": iters,
            "certified": bool(ok), "sequential_single_solves_per_s": 256 / seq_s, "sequential_certified": seq_ok,
            "speedup_vs_sequential": (256e3 / ms) / (256 / seq_s)}


def multi_rhs_n64(torch, Q, dev, D, lat, single_ms, reps=3):
    """64 right-hand sides of the headline operator (n=64, m=0.05) in one
    batched persistent launch (autotuned tile, threads and schedule; plain CG,
    FP32 iterations with FP64 reliable updates, each solution certified by its
    FP64 true residual), against the single-right-hand-side learned solver."""
    rng = np.random.default_rng(64)
    b = torch.from_numpy(rng.normal(size=(64, 2 * lat.n_sites)) + 1j * rng.normal(size=(64, 2 * lat.n_sites))).to(dev)
    batch = Q.Batch([(D, 64)], precision=Q.PREC_F32)
    xs = [torch.zeros_like(b)]
    ms_l, ok, iters = [], True, 0
    for i in range(reps + 1):
        reps_, ms = batch.solve(xs, [b], tol=TOL, precision=Q.PREC_F32, delta=RU_DELTA)
        ok = ok and all(r.status == Q.OK and r.true_rel_res <= TOL for r in reps_)
        iters = max(iters, max(r.iters for r in reps_))
        if i > 0:
            ms_l.append(ms)
    ms = float(np.mean(ms_l))
    return {"rhs": 64, "n": N_REFINE, "rhs_tile": batch.rhs_tile, "threads": batch.threads,
            "schedule": {Q.BATCH_STATIC: "static", Q.BATCH_DYNAMIC: "dynamic"}[batch.schedule],
            "ms_per_batch": ms, "solves_per_s": 64e3 / ms, "max_iters": iters, "certified": bool(ok),
            "single_rhs_learned_solves_per_s": 1e3 / single_ms, "throughput_per_rhs_vs_single": (64e3 / ms) / (1e3 / single_ms)}


def ref_gpu_baseline(A, b, reps=3):
    """The reference's GPU CG design on this GPU (oracle/ref_gpu_cg.cu) over
    the reference CSR operator of the workload; host-vector solves as the
    reference's MatPoly::solve makes them (b copied in, x copied out)."""
    import ctypes
    from oracle import oracle as O
    g = O.geometry(N_REFINE)
    D = O.Dirac(g, 1.0, M5)
    D.update(A)
    rows, cols, val = D.csr()
    rowsT, colsT, valH = D.csr(dagger=True)
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_build", "librefgpu.so"))
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    x = np.zeros_like(b)
    ms = np.zeros(reps)
    it = L.refgpu_cg(ctypes.c_int(D.N), ctypes.c_int(cols.size), p(rows), p(cols), p(val), p(rowsT), p(colsT),
                     p(valH), p(b), p(x), ctypes.c_double(TOL), ctypes.c_int(100000), ctypes.c_int(1),
                     ctypes.c_int(reps), p(ms))
    if it < 0:
        return {"error": "refgpu_cg failed"}
    res = float(np.linalg.norm(b - D.apply(x, 2)) / np.linalg.norm(b))
    return {"ms": float(np.mean(ms)), "ms_min": float(np.min(ms)), "iters": int(it), "true_rel_res": res,
            "solves_per_s": 1e3 / float(np.mean(ms)), "kind": "reference GPU algorithm restated",
            "design": "CSR SpMV one thread per row + separate axpy kernels + cuBLAS Zdotc read back by the host "
                      "+ cudaMalloc/cudaFree per operator call, FP64, sm_103a (oracle/ref_gpu_cg.cu)",
            "timing": "host wall clock per host-vector solve (H2D of b and D2H of x inside)"}


def count_launches(torch, fn):
    """Kernel launches of one call of fn() (CUPTI runtime-API callbacks,
    qed3_gb300/launchcount.c): (this library's kernels, all kernels)."""
    import ctypes
    path = os.path.join(ROOT, "qed3_gb300", "liblaunchcount.so")
    if not os.path.exists(path):
        raise RuntimeError("launch counter not built (CUPTI headers missing)")
    L = ctypes.CDLL(path)
    torch.cuda.synchronize()
    if L.lc_start() != 0:
        raise RuntimeError("CUPTI subscription failed")
    fn()
    torch.cuda.synchronize()
    ours, tot = ctypes.c_longlong(), ctypes.c_longlong()
    L.lc_stop(ctypes.byref(ours), ctypes.byref(tot))
    return int(ours.value), int(tot.value)


def profile_case(torch, which):
    """Small cases for ncu captures (a few hundred MB on the device)."""
    import qed3_gb300 as Q
    if which == "apply":
        for prec in (Q.PREC_F32, Q.PREC_BF16, Q.PREC_F64):
            r = apply_bandwidth(torch, Q, 512, prec, reps=3)
            print(json.dumps(r))
    elif which == "ext":
        # the S^2 x S^1 operator at n=64, Nt=16 (0.5 GB of hop blocks, above L2): 3 D applies
        Nt = 16
        lat = Q.S2Trivalent(64)
        De = Q.DiracExt(lat, 1.0, 0.1, Nt, 0.5)
        g = torch.Generator(device="cuda")
        g.manual_seed(4)
        De.update((torch.rand(Nt * (lat.n_links + lat.n_sites), dtype=torch.float64, device="cuda", generator=g)
                   * 2 - 1) * np.pi)
        v = torch.randn(Nt * 2 * lat.n_sites, dtype=torch.complex128, device="cuda", generator=g)
        w = torch.empty_like(v)
        for _ in range(3):
            De.apply(w, v, Q.OP_D)
        # eight FP32 iterations of the mixed-precision CG (k_ext_apply32 and its BLAS)
        rep = De.solve(w, v, tol=1e-10, maxiter=8, precision=Q.PREC_F32)
        print(json.dumps({"norm": float(torch.linalg.vector_norm(w)), "iters": rep.iters}))
    elif which == "train":
        # a few Adam steps of the n=64 network (the tcgen05 mixing and weight-gradient kernels)
        lat = Q.S2Trivalent(N_REFINE)
        D = Q.DiracS2Dual(lat, 1.0, M5)
        D.update(torch.from_numpy(np.random.default_rng(2).uniform(-np.pi, np.pi, lat.n_links)).cuda())
        pc = Q.LearnedPreconditioner(D, channels=16, layers=2, seed=1)
        pc.collect(D, nsrc=2, seed=1000, snapshots=(0, 5, 20))
        hist = pc.train(4, batch=8, lr=3e-3, seed=2)
        print(json.dumps({"loss": [float(v) for v in hist]}))
    elif which in ("batched", "batched_static"):
        # a quarter of the 256-RHS configuration (16 right-hand sides on each
        # of n = 16, 32, 48, 64; ~0.4 GB of fields, above L2) with the tile,
        # threads and schedule the autotuner picks for the full one (or the
        # static schedule), so no tuning launches precede it
        rng = np.random.default_rng(256)
        systems, bs = [], []
        for n in (16, 32, 48, 64):
            lat_n = Q.S2Trivalent(n)
            D_n = Q.DiracS2Dual(lat_n, 1.0, float(rng.uniform(0.02, 0.2)))
            D_n.update(torch.from_numpy(rng.uniform(-np.pi, np.pi, lat_n.n_links)).cuda())
            b_n = rng.normal(size=(16, 2 * lat_n.n_sites)) + 1j * rng.normal(size=(16, 2 * lat_n.n_sites))
            systems.append((D_n, 16))
            bs.append(torch.from_numpy(b_n).cuda())
        if which == "batched":
            batch = Q.Batch(systems, precision=Q.PREC_F32, rhs_tile=2, threads=256, schedule=Q.BATCH_DYNAMIC)
        else:
            batch = Q.Batch(systems, precision=Q.PREC_F32, rhs_tile=1, threads=128, schedule=Q.BATCH_STATIC)
        xs = [torch.zeros_like(b_) for b_ in bs]
        for _ in range(2):
            reps, ms = batch.solve(xs, bs, tol=TOL, precision=Q.PREC_F32, delta=RU_DELTA)
        print(json.dumps({"ms": ms, "max_iters": max(r.iters for r in reps),
                          "certified": all(r.status == Q.OK and r.true_rel_res <= TOL for r in reps)}))
    else:
        lat = Q.S2Trivalent(N_REFINE)
        D = Q.DiracS2Dual(lat, 1.0, M5)
        A = torch.from_numpy(np.random.default_rng(2).uniform(-np.pi, np.pi, lat.n_links)).cuda()
        D.update(A)
        b = torch.from_numpy(Q.ParallelRng(lat, 7).gaussian_spinor()).cuda()
        x = torch.zeros_like(b)
        if which == "pcgs":  # the streaming kernel on an HBM-resident lattice, 200 iterations
            lat = Q.S2Trivalent(256)
            D = Q.DiracS2Dual(lat, 1.0, M5)
            D.update(torch.from_numpy(np.random.default_rng(2).uniform(-np.pi, np.pi, lat.n_links)).cuda())
            b = torch.from_numpy(Q.ParallelRng(lat, 7).gaussian_spinor()).cuda()
            x = torch.zeros_like(b)
            pc = Q.LearnedPreconditioner(D, channels=16, layers=2, seed=1)
            rep = pc.solve(D, x, b, tol=TOL, precision=Q.PREC_F32, maxiter=200)
        elif which in ("pcg", "ppcg"):  # untrained network: same per-iteration cost as a trained one
            pc = Q.LearnedPreconditioner(D, channels=16, layers=2, seed=1)
            rep = pc.solve(D, x, b, tol=TOL, precision=Q.PREC_F32, maxiter=300, pipelined=which == "ppcg")
        else:
            rep = D.solve(x, b, tol=TOL, precision=Q.PREC_F32)
        print(json.dumps(rep.__dict__))
    torch.cuda.synchronize()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-paths", action="store_true", help="skip the timings of the HMC, overlap and S^2 x S^1 paths")
    ap.add_argument("--profile", choices=["apply", "cg", "pcg", "ppcg", "pcgs", "batched", "batched_static", "ext", "train"],
                    default=None,
                    help="small self-contained case for ncu: 'apply' = D apply at n=512 (f32, bf16, f64; "
                         "HBM-resident), 'cg' = one n=64 mixed-precision solve, 'pcg' = 300 iterations of the "
                         "n=64 preconditioned solve, 'ppcg' = the same with the pipelined one-barrier kernel, "
                         "'batched' / 'batched_static' = 64 RHS over four lattices (dynamic / static schedule), "
                         "'ext' = S^2 x S^1 D apply at n=64, Nt=16, "
                         "'train' = four Adam steps of the n=64 network (tcgen05 channel mixing), 'pcgs' = 200 iterations "
                         "of the streaming preconditioned solver at n=256")
    args = ap.parse_args()
    rank, world, local = env_rank()
    warmup = max(3, args.warmup)

    import torch
    if args.profile:
        return profile_case(torch, args.profile)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    # ---- the reference arm: host-core CG of the reference algorithm ----------------
    if args.impl == "reference":
        if rank != 0:
            return
        g, A_h, b, acc = make_workload_oracle()
        times, its = [], []
        for i in range(warmup + args.steps):
            dt, it, res, cores = cpu_reference_solve(b, A_h, g)
            if i >= warmup:
                times.append(dt)
                its.append(it)
        v = len(times) / sum(times)
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": 0,
                "steps": args.steps, "warmup": warmup, "ms_per_step": 1e3 * sum(times) / len(times),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": config(world),
                "solver": "reference CG (MatPoly::solve) restated over the reference CSR operator",
                "iters": int(np.median(its)), "hmc_acceptance": acc,
                "cpu_baseline": {"value": v, "unit": "solves/s", "cores": cores, "kind": "port",
                                 "sample": "full n=64 solves to 1e-10 on all host cores"},
                "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    # ---- our arm -------------------------------------------------------------------
    Q, lat, A, D, b, acc = make_workload(torch, dev)
    bt = torch.from_numpy(b).to(dev)
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    pc, train_info = train_preconditioner(torch, Q, lat, D, dev)
    torch.cuda.synchronize()

    results = {}
    solvers = (("f64", Q.PREC_F64, None), ("f32", Q.PREC_F32, None), ("bf16", Q.PREC_BF16, None),
               ("pcg_f32", Q.PREC_F32, pc), ("pcg_bf16", Q.PREC_BF16, pc))
    clocks = Clocks(local)
    clocks.start()  # sampled over every timed solver and the e2e loop
    torch.cuda.nvtx.range_push("timed")  # the launch list of the timed region (ncu --nvtx-include timed/)
    for name, prec, p in solvers:
        ms, reps, x = time_solver(torch, Q, D, bt, prec, args.steps, warmup, flush, pc=p)
        ok = all(r.status == Q.OK and r.true_rel_res <= TOL for r in reps)
        results[name] = {"ms": float(np.mean(ms)), "ms_min": float(np.min(ms)), "iters": reps[-1].iters,
                         "reliable_updates": reps[-1].reliable_updates, "true_rel_res": reps[-1].true_rel_res,
                         "certified": ok}
    cands = [k for k in ("pcg_f32", "pcg_bf16") if results[k]["certified"]]
    if not cands:  # the learned solver is judged by plain CG's certificate; fall back to the best plain one
        cands = [k for k in ("f64", "f32", "bf16") if results[k]["certified"]]
    best = min(cands, key=lambda k: results[k]["ms"])
    ms_best = results[best]["ms"]
    if world > 1:
        t = torch.tensor([ms_best], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_best = float(t.item())
    value = world * 1e3 / ms_best

    # ---- e2e through the public C-ABI call with pinned host buffers ----------------
    prec_best = Q.PREC_BF16 if best.endswith("bf16") else (Q.PREC_F64 if best == "f64" else Q.PREC_F32)
    use_pc = best.startswith("pcg")
    hb = torch.from_numpy(b).pin_memory()
    hx = torch.zeros_like(hb).pin_memory()
    db = torch.empty_like(bt)
    dx = torch.empty_like(bt)
    st = torch.cuda.current_stream()
    e2e_ms = []
    for i in range(warmup + args.steps):
        flush_l2(torch, flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        db.copy_(hb, non_blocking=True)
        if use_pc:
            pc.solve(D, dx, db, tol=TOL, precision=prec_best, delta=ru_delta(Q, prec_best))
        else:
            D.solve(dx, db, tol=TOL, precision=prec_best, delta=ru_delta(Q, prec_best))
        hx.copy_(dx, non_blocking=True)
        e1.record(st)
        e1.synchronize()
        if i >= warmup:
            e2e_ms.append(e0.elapsed_time(e1))
    e2e = world * 1e3 / float(np.mean(e2e_ms))
    torch.cuda.nvtx.range_pop()
    clocks_info = clocks.stop()

    train_info["tensor_cores"] = tc_training_timing(torch, pc)
    train_info["depth_study"] = network_depth_study(torch, Q, lat, D, pc, dev)
    heldout = heldout_iterations(torch, Q, lat, pc, dev)
    batched = batched_throughput(torch, Q, dev)
    multi64 = multi_rhs_n64(torch, Q, dev, D, lat, results[best]["ms"])
    paths = None if args.no_paths else paths_timings(torch, Q, dev, cpu=rank == 0 and not args.no_cpu_baseline)
    overlap32 = None if args.no_paths else overlap_config(torch, Q, dev)
    hbm_pcg = None if args.no_paths else learned_hbm(torch, Q, dev)

    # ---- roofline of the dominant kernel ----------------------------------------------
    # algorithmic HBM bytes per site per iteration (the measurement rule: each array once):
    #   D^dag D = 2 x (2 S_psi + 3 (4 + S_H) + S_diag) with S_psi the stored spinor size,
    #   plus 7 spinor streams of the solver state (read x, r, p, q; write x, r, p).
    # The learned preconditioner's neighbour passes run in shared memory on the
    # block's own sites and add no HBM bytes.
    S = {"f64": 32, "f32": 16, "bf16": 8, "pcg_f32": 16, "pcg_bf16": 8}[best]
    if best == "f64":
        per_site_iter = 2 * (2 * 32 + 3 * (4 + 64) + 8) + 7 * 32
    else:
        per_site_iter = 2 * (2 * S + 3 * (4 + 32) + 4) + 7 * 16
    iters = results[best]["iters"]
    alg_bytes = per_site_iter * lat.n_sites * iters
    achieved = alg_bytes / (results[best]["ms"] * 1e-3) / 1e9
    peak, peak_kind = peaks()
    sweep = []
    # the apply sweep over n = 32 ... 512 in FP32 (L2-resident below n ~ 100), BF16 and FP64 at the large end
    for n, p in tuple((n_, Q.PREC_F32) for n_ in (32, 48, 64, 96, 128, 192, 256, 384, 512)) + (
            (512, Q.PREC_BF16), (256, Q.PREC_F64), (512, Q.PREC_F64)):
        s_ = apply_bandwidth(torch, Q, n, p)
        s_["frac_of_" + peak_kind] = s_["GB/s"] / peak
        s_["resident"] = "L2" if s_["bytes_per_site"] * 20 * n * n < 100e6 else "HBM"
        sweep.append(s_)
    hbm_apply = next(s_ for s_ in sweep if s_["n"] == 512 and s_["prec"] == "f32")

    # ---- launches of this library's kernels in the timed region ------------------------
    def one_step():
        if use_pc:
            pc.solve(D, dx, db, tol=TOL, precision=prec_best, delta=ru_delta(Q, prec_best))
        else:
            D.solve(dx, db, tol=TOL, precision=prec_best, delta=ru_delta(Q, prec_best))
    try:
        ours1, all1 = count_launches(torch, one_step)
        launches = {"per_step": ours1, "per_step_all_kernels": all1,
                    "source": "CUPTI launch callbacks on one extra step (qed3_gb300/launchcount.c), times the "
                              "timed steps"}
    except Exception as e:  # the profiler is unavailable: the solve's launch sequence, counted by hand
        ours1 = 4  # |b| partials, unit-norm import, solver, scaled export
        launches = {"per_step": ours1, "source": f"launch sequence of the solve (trace unavailable: {e})"}
    n_timed = args.steps  # the headline's timed steps (the e2e loop repeats them through host buffers)
    ref_gpu = ref_gpu_baseline(A.cpu().numpy(), b) if rank == 0 and not args.no_cpu_baseline else None
    if ref_gpu and "ms" in ref_gpu:
        ref_gpu["learned_speedup"] = ref_gpu["ms"] / results[best]["ms"]
        ref_gpu["learned_e2e_speedup"] = ref_gpu["ms"] / float(np.mean(e2e_ms))
        ref_gpu["plain_f64_speedup"] = ref_gpu["ms"] / results["f64"]["ms"]
    kernel = "k_pcg" if use_pc else ("k_cg_v2")
    dtype = {"f64": "f64", "f32": "f32", "bf16": "f32 (bf16 halo copies)", "pcg_f32": "f32",
             "pcg_bf16": "f32 (bf16 halo copies)"}[best]

    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": warmup, "ms_per_step": ms_best, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": config(world),
            "solver": (f"learned-preconditioned persistent CG, {best[4:]} inner, FP64 reliable updates"
                       if use_pc else f"persistent CG, {best} inner, FP64 reliable updates"),
            "hmc_acceptance": acc,
            "solvers": results, "reliable_update_delta": {"f32": RU_DELTA, "bf16": 0.1},
            "speedup_vs_plain_f64": results["f64"]["ms"] / results[best]["ms"],
            "preconditioner": train_info,
            "heldout": heldout,
            "heldout_summary": heldout_summary(heldout),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": PCG_DRAM_BYTES_PER_LAUNCH if use_pc else None, "kernel": kernel,
                         "resident": "L2", "note": "L2-resident effective bandwidth: the n=64 working set stays "
                         "in the 129 MB L2, so `traffic` (ncu DRAM bytes per launch) is far below the algorithmic "
                         f"bytes; {per_site_iter} B/site/iteration (D^dag D + 7 solver-state streams) x "
                         f"{lat.n_sites} sites x {iters} iterations per launch; the solver is grid-barrier "
                         "latency bound",
                         "hbm_apply": {"kernel": "k_apply32<F32>", "n": 512, "GB/s": hbm_apply["GB/s"],
                                       "frac": hbm_apply["frac_of_" + peak_kind]}},
            "apply_sweep": sweep,
            "batched_256": batched,
            "multi_rhs_n64": multi64,
            "overlap_n32": overlap32,
            "learned_pc_n256": hbm_pcg,
            "paths": paths,
            "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": b.nbytes, "d2h_bytes_per_step": b.nbytes},
            "gpu_launches": ours1 * n_timed,
            "gpu_launches_detail": dict(launches, timed_steps=n_timed),
            "ref_gpu_baseline": ref_gpu,
            "clocks": clocks_info}
    if rank == 0 and not args.no_cpu_baseline:
        dt, it, res, cores = cpu_reference_solve(b, A.cpu().numpy())
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "solves/s", "cores": cores, "kind": "port",
                                "sample": f"one full n=64 solve to 1e-10 ({it} iterations, true res {res:.1e})"}
    if world > 1:
        torch.distributed.barrier()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
