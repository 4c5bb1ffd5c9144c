"""Regenerates the golden fixtures in this folder.

zolotarev_ref.json: Zolotarev coefficients produced by the REFERENCE's own
code (src/both_3d/overlap.h:7-134), compiled in place by `make -C oracle ref`
into oracle/_ref/libzolo_ref.so.  Needs the reference tree, so it runs only in
the development container; the fixture travels with the repo.

rng_ref.json: the REFERENCE's own ParallelRng2 streams (src/both/rng.h:76-125),
compiled in place by the same `make -C oracle ref` into oracle/_ref/librng_ref.so:
per-link Gaussians (two sweeps), the per-site Gaussians in fill_gaussian's
order, master uniforms and per-site Z2 draws, for two lattice sizes and seeds.

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


def spectrum_fixture():
    data = dict(source="analysis/ev_dual.ipynb cells 33-34: [n, |Im lambda| (j=3/2), |Im lambda| (j=1/2)]",
                rows=[[2, 1.89453, 0.995597], [4, 1.97081, 0.997657], [6, 1.98474, 0.998488],
                      [8, 1.98955, 0.998865]])
    with open(os.path.join(HERE, "free_spectrum.json"), "w") as f:
        json.dump(data, f, indent=1)


if __name__ == "__main__":
    zolotarev_fixture()
    rng_fixture()
    spectrum_fixture()
