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


if __name__ == "__main__":
    zolotarev_fixture()
    rng_fixture()
    gauge_fixture()
    rng_ckpoint_fixture()
    spectrum_fixture()
    analyze_corr_fixture()
