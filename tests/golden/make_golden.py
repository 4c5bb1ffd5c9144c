"""Regenerates the golden fixtures in this folder.

zolotarev_ref.json: Zolotarev coefficients produced by the REFERENCE's own
code (src/both_3d/overlap.h:7-134), compiled in place by `make -C oracle ref`
into oracle/_ref/libzolo_ref.so.  Needs the reference tree, so it runs only in
the development container; the fixture travels with the repo.

rng_ref.json: the REFERENCE's own ParallelRng2 streams (src/both/rng.h:76-125),
compiled in place by the same `make -C oracle ref` into oracle/_ref/librng_ref.so:
per-link Gaussians (two sweeps), the per-site Gaussians in fill_gaussian's
order, master uniforms and per-site Z2 draws, for two lattice sizes and seeds.

gauge_ref.json: the REFERENCE's own gauge side compiled in place by the same
`make -C oracle ref` into oracle/_ref/libgauge_ref.so -- U1onS2 plaquette
angles and average plaquette (src/both/gauge.h), U1Wilson action and force
(src/both/action.h), and HMCPureGauge trajectories driven by ParallelRng2
(src/both/hmc.h:115-200, src/both/rng.h) -- on the oracle's lattice tables
(faces, dual-face areas, link orientation) for n = 2 and 4, compact and
non-compact.

rng_ckpoint_ref.txt / rng_ckpoint_ref.json: a checkpoint written by the
REFERENCE's ParallelRngExt::ckpoint (src/both_3d/rng.h:131-168, Nt = 1; built
in place by `make -C oracle ref` into oracle/_ref/librng3d_ref.so) after one
sweep of link and site Gaussians and three master uniforms (3 links, 2 sites,
seed 5), and the reference's continuation draws after it.

analyze_corr_ref.json: the REFERENCE's correlator analysis program
(src/both_3d/analyze_corr.cpp, built in place by `make -C oracle ref` into
oracle/_ref/analyze_corr) run on seeded synthetic correlator files (stored in
the fixture): its complete standard output for three argument sets (two
streams with one cut short, binsize 1 and 3, one stream).

free_spectrum.json: the known answers of analysis/ev_dual.ipynb (cells 33-34),
typed in from the notebook's output cells.

dirac_ref.npz: the REFERENCE's own operator pipeline compiled in place by
`make -C oracle ref` into oracle/_ref/libdirac_ref_n<n>_t<Nt>.so
(oracle/ref_dirac.cu): S2Simp / S2Trivalent reading this project's lattice
from .dat tables in the reference's layout (qed3_gb300.dats.write), the
reference's spin-structure tables and check, DiracS2Dual kappa / gamma /
Omega, DiracExt::coo_format, DWDevice's CSR assembly and the host SpMV
`matmul`.  Per case (key prefix "n<n>_t<Nt>/"): the link angles A, the source
v, D v, D^dag v, D^dag D v, D's CSR values (n=2 only), the CG iterates of
MatPoly::solve's iteration (restated on the host over the reference's matmul)
after the counts in `iters_at`, and the converged x at tol 1e-10 with its
iteration count.
"""
import ctypes
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

CASES = [(0.01, 21), (0.01, 31), (0.01, 41), (0.003, 41), (0.05, 41), (0.2, 11), (0.1, 51)]


def zolotarev_fixture():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libzolo_ref.so"))
    dp = ctypes.POINTER(ctypes.c_double)
    out = []
    for k, n in CASES:
        size = n // 2 + 1
        c, cp, A, sc = np.zeros(size), np.zeros(size), np.zeros(size), np.zeros(4)
        L.ref_zolotarev(ctypes.c_double(k), n, *[a.ctypes.data_as(dp) for a in (c, cp, A, sc)])
        out.append(dict(k=k, n=n, c=[float.hex(v) for v in c], cp=[float.hex(v) for v in cp],
                        A=[float.hex(v) for v in A], M=float.hex(sc[0]), lambda_inv=float.hex(sc[1]),
                        E=float.hex(sc[2]), C=float.hex(sc[3])))
    with open(os.path.join(HERE, "zolotarev_ref.json"), "w") as f:
        json.dump(dict(source="reference src/both_3d/overlap.h:7-134 compiled by oracle/Makefile `ref`",
                       cases=out), f, indent=1)


RNG_CASES = [(30, 20, 1), (120, 80, 7), (480, 320, 12345)]


def rng_fixture():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "librng_ref.so"))
    dp = ctypes.POINTER(ctypes.c_double)
    out = []
    for nl, ns, seed in RNG_CASES:
        links2, sites4, unif5, z2 = np.zeros(2 * nl), np.zeros(4 * ns), np.zeros(5), np.zeros(4 * ns)
        L.ref_rng_streams(nl, ns, seed, *[a.ctypes.data_as(dp) for a in (links2, sites4, unif5, z2)])
        out.append(dict(n_links=nl, n_sites=ns, seed=seed, links2=[float.hex(v) for v in links2],
                        sites4=[float.hex(v) for v in sites4], uniform5=[float.hex(v) for v in unif5],
                        z2=[int(v) for v in z2]))
    with open(os.path.join(HERE, "rng_ref.json"), "w") as f:
        json.dump(dict(source="reference src/both/rng.h:76-125 (ParallelRng2) compiled by oracle/Makefile `ref`",
                       cases=out), f, indent=0)


GAUGE_CASES = [(2, False, 1.4, 9), (2, True, 1.4, 9), (4, True, 1.4, 5), (4, False, 2.0, 6)]


def gauge_fixture():
    import sys
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libgauge_ref.so"))
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    hx = lambda a: [float.hex(float(v)) for v in a]
    out = []
    for n, compact, beta, seed in GAUGE_CASES:
        g = O.geometry(n)
        A = np.random.default_rng(100 + n).normal(size=g.n_links) * 0.5
        fo = np.ascontiguousarray(g.face_offsets, np.int32)
        fs = np.ascontiguousarray(g.face_sites, np.int32)
        links = np.ascontiguousarray(g.links, np.int32).ravel()
        vols = np.ascontiguousarray(g.vols)
        ntraj, tmax, nsteps = 3, 1.0, 20
        th, F, Aout = np.zeros(g.n_faces), np.zeros(g.n_links), np.zeros(g.n_links)
        dH, acc = np.zeros(ntraj), np.zeros(ntraj, np.int32)
        avg, S = ctypes.c_double(), ctypes.c_double()
        L.ref_gauge_run(g.n_sites, g.n_links, g.n_faces, fo.ctypes.data_as(ip), fs.ctypes.data_as(ip),
                        vols.ctypes.data_as(dp), ctypes.c_double(g.mean_vol), links.ctypes.data_as(ip), int(compact),
                        ctypes.c_double(beta), A.ctypes.data_as(dp), th.ctypes.data_as(dp), ctypes.byref(avg),
                        ctypes.byref(S), F.ctypes.data_as(dp), seed, ctypes.c_double(tmax), nsteps, ntraj,
                        Aout.ctypes.data_as(dp), dH.ctypes.data_as(dp), acc.ctypes.data_as(ip))
        out.append(dict(n=n, compact=compact, beta=beta, A=hx(A), theta=hx(th), avg_plaquette=float.hex(avg.value),
                        action=float.hex(S.value), force=hx(F), hmc=dict(seed=seed, tmax=tmax, nsteps=nsteps,
                        dH=hx(dH), accepted=[int(v) for v in acc], A_final=hx(Aout))))
    with open(os.path.join(HERE, "gauge_ref.json"), "w") as f:
        json.dump(dict(source="reference src/both/{gauge,action,hmc,rng}.h compiled by oracle/Makefile `ref` on the "
                              "oracle's lattice tables; the force is the reference's (theta, not sin theta)",
                       cases=out), f, indent=0)


def rng_ckpoint_fixture():
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "librng3d_ref.so"))
    nl, ns, seed = 3, 2, 5
    cont = np.zeros(nl + 4 * ns + 2 + 4 * ns)
    path = os.path.join(HERE, "rng_ckpoint_ref.txt")
    dp = ctypes.POINTER(ctypes.c_double)
    L.ref_rng3d_run(nl, ns, seed, path.encode(), None, cont.ctypes.data_as(dp), None)
    with open(os.path.join(HERE, "rng_ckpoint_ref.json"), "w") as f:
        json.dump(dict(source="reference src/both_3d/rng.h ParallelRngExt<.,1>::ckpoint compiled by oracle/Makefile "
                              "`ref`; draws before: links, 4 x sites, 3 uniforms; after: links, 4 x sites, "
                              "2 uniforms, 4 x sites z2",
                       n_links=nl, n_sites=ns, seed=seed, continuation=[float.hex(float(v)) for v in cont]), f,
                  indent=0)


def spectrum_fixture():
    data = dict(source="analysis/ev_dual.ipynb cells 33-34: [n, |Im lambda| (j=3/2), |Im lambda| (j=1/2)]",
                rows=[[2, 1.89453, 0.995597], [4, 1.97081, 0.997657], [6, 1.98474, 0.998488],
                      [8, 1.98955, 0.998865]])
    with open(os.path.join(HERE, "free_spectrum.json"), "w") as f:
        json.dump(data, f, indent=1)


def analyze_corr_fixture():
    import tempfile
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    exe = os.path.join(ROOT, "oracle", "_ref", "analyze_corr")
    rng = np.random.default_rng(17)
    Nt = 6
    files = {}
    # stream 1: confs 10, 12, ..., 48; stream 2 stops at 40
    for prefix, last in ((1, 48), (2, 40)):
        for conf in range(10, last + 1, 2):
            decay = np.exp(-0.4 * np.arange(Nt)) + np.exp(-0.4 * (Nt - np.arange(Nt)))
            files[f"corr/s{prefix}/C{conf}.dat"] = [float(v) for v in decay * (1 + 0.1 * rng.normal(size=Nt))]
    cases = [["corr/s", "C", 10, 60, 2, Nt, 2, 2], ["corr/s", "C", 10, 60, 2, Nt, 3, 2],
             ["corr/s", "C", 12, 44, 2, Nt, 1, 1]]
    out = []
    with tempfile.TemporaryDirectory() as d:
        for rel, vals in files.items():
            os.makedirs(os.path.join(d, os.path.dirname(rel)), exist_ok=True)
            with open(os.path.join(d, rel), "w") as f:
                f.write("".join(f"{v!r} {0.5 * v!r}\n" for v in vals))
        for c in cases:
            r = subprocess.run([exe] + [str(a) for a in c], cwd=d, capture_output=True, text=True, check=True)
            out.append(dict(args=c, stdout=r.stdout.splitlines()))
    with open(os.path.join(HERE, "analyze_corr_ref.json"), "w") as f:
        json.dump(dict(source="src/both_3d/analyze_corr.cpp built in place; files: first column read, second ignored",
                       files=files, runs=out), f, indent=1)


# (n, Nt, r, M5, at, iterates recorded after these CG iteration counts, store D/D^dag outputs)
DIRAC_CASES = [(2, 1, 1.0, 0.1, 1.0, (1, 2, 5, 20), True), (4, 1, 1.0, 0.05, 1.0, (1, 5, 20), True),
               (8, 1, 1.0, 0.1, 1.0, (), False), (2, 2, 1.0, 0.1, 0.5, (1, 5, 20), True),
               (4, 4, 1.0, -0.5, 0.5, (), False)]


def dirac_fixture():
    import sys
    import tempfile
    sys.path.insert(0, ROOT)
    import qed3_gb300 as Q
    from qed3_gb300 import dats
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"])
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    out = {}
    for n, Nt, r, M5, at, iters_at, full in DIRAC_CASES:
        L = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", f"libdirac_ref_n{n}_t{Nt}.so"))
        lat = Q.S2Trivalent(n)
        Ns, Nl = lat.n_sites, lat.n_links
        N = 2 * Ns * Nt
        rng = np.random.default_rng(1000 * n + Nt)
        A = rng.uniform(-np.pi, np.pi, Nt * (Nl + Ns))
        v = rng.normal(size=N) + 1j * rng.normal(size=N)
        Dv, DHv, DHDv, xf = (np.zeros(N, np.complex128) for _ in range(4))
        rows, cols = np.zeros(N + 1, np.int32), np.zeros(12 * N, np.int32)
        val = np.zeros(12 * N, np.complex128)
        kappa = np.zeros(Nl)
        its = np.array(iters_at, np.int32)
        x_at = np.zeros((max(1, len(its)), N), np.complex128)
        with tempfile.TemporaryDirectory() as d:
            dats.write(lat, d)
            k = L.ref_dirac_run(d.encode(), ctypes.c_double(r), ctypes.c_double(M5), ctypes.c_double(at),
                                A.ctypes.data_as(dp), v.ctypes.data_as(dp), Dv.ctypes.data_as(dp),
                                DHv.ctypes.data_as(dp), DHDv.ctypes.data_as(dp), rows.ctypes.data_as(ip),
                                cols.ctypes.data_as(ip), val.ctypes.data_as(dp), kappa.ctypes.data_as(dp),
                                ctypes.c_double(1e-10), 100000, len(its), its.ctypes.data_as(ip),
                                x_at.ctypes.data_as(dp), xf.ctypes.data_as(dp))
        assert k > 0, (n, Nt, k)
        key = f"n{n}_t{Nt}/"
        out[key + "params"] = np.array([r, M5, at])
        out[key + "A"] = A
        out[key + "v"] = v
        out[key + "DHDv"] = DHDv
        out[key + "x_final"] = xf
        out[key + "cg_iters"] = np.array([k], np.int32)
        out[key + "kappa"] = kappa
        if full:
            out[key + "Dv"] = Dv
            out[key + "DHv"] = DHv
        if len(its):
            out[key + "iters_at"] = its
            out[key + "x_at"] = x_at
        if n == 2 and Nt == 1:
            out[key + "csr_rows"] = rows
            out[key + "csr_cols"] = cols
            out[key + "csr_val"] = val
    np.savez_compressed(os.path.join(HERE, "dirac_ref.npz"), **out)


if __name__ == "__main__":
    zolotarev_fixture()
    rng_fixture()
    gauge_fixture()
    rng_ckpoint_fixture()
    spectrum_fixture()
    analyze_corr_fixture()
    dirac_fixture()
