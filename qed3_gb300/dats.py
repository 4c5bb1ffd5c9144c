"""The reference's geometry and spin-structure text tables.

The reference generates its lattice offline and reads it from `.dat` files:
  * written by integrator/get_geometry.cc:352-439 (pts, pts_dual, nns,
    nns_dual, links, dual_links, face, face_dual)
  * written by integrator/test_sorting.cc:430-456 (omega_dual, alpha_dual)
  * read by src/both_3d/s2n_simp.h:43-190, src/both_3d/s2n_dual.h:49-106 and
    src/both_3d/dirac_dual.h:15-60.

`write` stores a lattice in that layout.  This project's O(N) builder can
then feed the reference at refinements its O(N^2) generator cannot reach.
`read` builds a lattice from a directory of such files.  The lattice keeps
the files' site numbering (matched through pts_dual), link numbering and
orientation (dual_links), and spin connection (omega_dual, alpha_dual, when
present).  A gauge configuration saved by the reference therefore indexes
the lattice unchanged.
"""
from __future__ import annotations

import os

import numpy as np

from . import S2Trivalent

_W, _P = 50, 25  # get_geometry.cc: std::setw(50), std::scientific, setprecision(25)
_WS, _PS = 25, 15  # test_sorting.cc: std::setw(25), setprecision(15)


def _name(kind: str, n: int) -> str:
    if kind == "face_dual":
        return f"face_dual_n{n}.dat"
    return f"{kind}_n{n}_singlepatch.dat"


def _write_rows(path, rows, fmt):
    with open(path, "w") as f:
        for r in rows:
            f.write("".join(fmt(v) + " " for v in r) + "\n")


def _f(v):
    return f"{float(v):{_W}.{_P}e}"


def _i(v):
    return f"{int(v):{_W}d}"


def write(lattice: S2Trivalent, directory: str, n_refine: int | None = None) -> list[str]:
    """Writes the lattice's tables in the reference's file layout; returns the paths."""
    n = lattice.n_refine if n_refine is None else n_refine
    if n < 1:
        raise ValueError("pass n_refine for a lattice built from a mesh")
    os.makedirs(directory, exist_ok=True)
    v, tri = lattice.mesh()
    t = lattice.tables()
    # simplicial neighbours of each vertex, ascending
    nb = [set() for _ in range(v.shape[0])]
    for a, b, c in tri:
        nb[a].update((b, c))
        nb[b].update((a, c))
        nb[c].update((a, b))
    faces = [t["face_sites"][t["face_offsets"][i]:t["face_offsets"][i + 1]] for i in range(lattice.n_faces)]
    out = []

    def p(kind):
        out.append(os.path.join(directory, _name(kind, n)))
        return out[-1]

    _write_rows(p("pts"), v, _f)
    _write_rows(p("pts_dual"), t["sites"], _f)
    _write_rows(p("nns_dual"), t["nns"], _i)
    _write_rows(p("links"), t["simp_links"], _i)
    _write_rows(p("dual_links"), t["links"], _i)
    _write_rows(p("face"), tri, _i)
    _write_rows(p("nns"), [sorted(s) for s in nb], _i)
    _write_rows(p("face_dual"), faces, _i)
    links = t["links"]
    slot = {(int(x), int(y)): k for x in range(lattice.n_sites) for k, y in enumerate(t["nns"][x])}
    with open(p("omega_dual"), "w") as f:
        for (i, j), om in zip(links, t["omega"]):
            f.write(f"{int(i):{_WS}d} {int(j):{_WS}d} {float(om):{_WS}.{_PS}e}\n")
    with open(p("alpha_dual"), "w") as f:
        for i, j in links:
            i, j = int(i), int(j)
            f.write(f"{i:{_WS}d} {j:{_WS}d} {t['alpha'][i][slot[(i, j)]]:{_WS}.{_PS}e}\n")
            f.write(f"{j:{_WS}d} {i:{_WS}d} {t['alpha'][j][slot[(j, i)]]:{_WS}.{_PS}e}\n")
    return out


def _load(path, dtype):
    with open(path) as f:
        return [np.array(line.split(), dtype=dtype) for line in f if line.strip()]


def _circumcentres(v, tri):
    a, b, c = v[tri[:, 0]], v[tri[:, 1]], v[tri[:, 2]]
    ab, ac = b - a, c - a
    n = np.cross(ab, ac)
    p = a + (np.cross(n, ab) * (ac * ac).sum(1)[:, None] + np.cross(ac, n) * (ab * ab).sum(1)[:, None]) / (
        2.0 * (n * n).sum(1)[:, None])
    return p / np.linalg.norm(p, axis=1)[:, None]


def read(directory: str, n_refine: int, spin_structure: bool = True) -> S2Trivalent:
    """Builds a lattice from the reference's files in `directory` (see the
    module docstring); `lattice.max_site_deviation` records how far the files'
    dual sites are from the rebuilt circumcentres."""
    g = lambda kind: os.path.join(directory, _name(kind, n_refine))
    v = np.vstack(_load(g("pts"), np.float64))
    tri = np.vstack(_load(g("face"), np.int64)).astype(np.int32)
    links = np.vstack(_load(g("dual_links"), np.int64)).astype(np.int32)
    # dual site s of the files is the triangle whose circumcentre it is
    sites = np.vstack(_load(g("pts_dual"), np.float64)) if os.path.exists(g("pts_dual")) else None
    if sites is not None:
        cc = _circumcentres(v / np.linalg.norm(v, axis=1)[:, None], tri)
        try:
            from scipy.spatial import cKDTree
            d, idx = cKDTree(cc).query(sites)
        except ImportError:  # small lattices: brute force
            dist = ((sites[:, None, :] - cc[None, :, :]) ** 2).sum(-1)
            idx = dist.argmin(1)
            d = np.sqrt(dist[np.arange(len(idx)), idx])
        if len(np.unique(idx)) != len(idx):
            raise ValueError("pts_dual does not match the triangles' circumcentres one to one")
        tri = tri[idx]
    lat = S2Trivalent.from_mesh(v, tri, links)
    lat.max_site_deviation = float(np.abs(lat.tables()["sites"] - sites).max()) if sites is not None else None
    if spin_structure and os.path.exists(g("omega_dual")) and os.path.exists(g("alpha_dual")):
        t = lat.tables()
        om_rows = _load(g("omega_dual"), np.float64)
        om_map = {(int(r[0]), int(r[1])): r[2] for r in om_rows}
        omega = np.empty(lat.n_links)
        for l, (i, j) in enumerate(t["links"]):
            i, j = int(i), int(j)
            omega[l] = om_map[(i, j)] if (i, j) in om_map else -om_map[(j, i)]
        al_map = {(int(r[0]), int(r[1])): r[2] for r in _load(g("alpha_dual"), np.float64)}
        alpha = np.array([[al_map[(x, int(y))] for y in t["nns"][x]] for x in range(lat.n_sites)])
        lat.set_spin_structure(omega, alpha)
    return lat
