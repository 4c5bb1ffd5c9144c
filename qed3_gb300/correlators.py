"""Propagator profiles and correlator analysis of the S^2 x S^1 extension.

* `site_angles`, `prop_profiles`, `write_prop_files`: the measurement end of
  the reference's propagator driver (src/both_3d/prop.cu:272-410).  The sink
  comes from `DiracExt.propagator` (the point-source solve on the GPU); this
  module turns it into the spatial profile on the slice of the source (sites
  with 0 <= phi <= width, against theta) and the temporal profile at site 0,
  both divided by at * mean_ell (mean_ell alone at Nt = 1), in the driver's
  text files.
* `Corr`, `jackknife`, `analyze_corr`: the binned jackknife of
  src/both_3d/analyze_corr.cpp:15-211 over files of one value per line,
  with its text output.
"""
from __future__ import annotations

import math
import os

import numpy as np

_TOLMOD = 1.0e-5  # integrator/geodesic.h:13


def _acos(x: float) -> float:
    """Geodesic::_acos (integrator/geodesic.h:113-121): clamps outside [-1, 1]."""
    if x < -1.0:
        return math.pi
    if x > 1.0:
        return 0.0
    return math.acos(x)


def _mod(a: float, b: float) -> float:
    """Geodesic::Mod (integrator/geodesic.h:36-41)."""
    return a - int(math.floor(a / b)) * b


def _is_moddable(v: float, q: float) -> bool:
    """Geodesic::isModdable (integrator/geodesic.h:86-90)."""
    return _mod(abs(v), q) < _TOLMOD or _mod(-abs(v), q) < _TOLMOD


def projection_s2(x) -> tuple[float, float]:
    """Geodesic::projectionS2 (integrator/geodesic.h:131-170): (theta, phi) of
    a point of R^3; phi = 0 at the poles, negative for y < 0."""
    r = math.sqrt(float(x[0]) ** 2 + float(x[1]) ** 2 + float(x[2]) ** 2)
    theta = _acos(float(x[2]) / r)
    phi = 0.0
    if not _is_moddable(theta, math.pi):
        phi = _acos(float(x[0]) / (r * math.sin(theta)))
        if float(x[1]) < 0.0:
            phi = -phi
    return theta, phi


def site_angles(lattice) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(theta, phi, geodesic length from site 0) of every dual site, reference numbering."""
    sites = lattice.tables()["sites"]
    th = np.empty(len(sites))
    ph = np.empty(len(sites))
    ln = np.empty(len(sites))
    x0 = sites[0]
    for i, p in enumerate(sites):
        th[i], ph[i] = projection_s2(p)
        ln[i] = _acos(float(x0[0] * p[0] + x0[1] * p[1] + x0[2] * p[2]))
    return th, ph, ln


def prop_profiles(lattice, sink, Nt: int, at: float, width: float = 0.05):
    """The rows prop.cu writes (src/both_3d/prop.cu:336-410): spatial rows
    (theta, Re, Im) for spin 0 then 1 of each site of slice 0 with
    0 <= phi <= width, in site order; temporal rows (at s, Re, Im) for spin 0
    then 1 of site 0 at each slice; values divided by at * mean_ell
    (mean_ell at Nt = 1).  sink: complex [Nt][n_sites][2] (host or device)."""
    if hasattr(sink, "detach"):
        sink = sink.detach().cpu().numpy()
    v = np.asarray(sink)
    if v.dtype != np.complex128:
        v = v.view(np.complex128) if v.dtype == np.float64 else v.astype(np.complex128)
    v = v.reshape(Nt, lattice.n_sites, 2)
    th, ph, _ = site_angles(lattice)
    mean_ell = float(lattice.tables()["means"][0])
    factor = at * mean_ell if Nt != 1 else mean_ell
    spatial = []
    for ix in range(lattice.n_sites):
        if ph[ix] > width or ph[ix] < 0.0:
            continue
        for a in (0, 1):
            e = v[0, ix, a]
            spatial.append((th[ix], e.real / factor, e.imag / factor))
    temporal = []
    for s in range(Nt):
        for a in (0, 1):
            e = v[s, 0, a]
            temporal.append((at * s, e.real / factor, e.imag / factor))
    return np.array(spatial).reshape(-1, 3), np.array(temporal).reshape(-1, 3)


def _tdiv(a: int, b: int) -> int:
    """C++ integer division (truncation toward zero)."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b >= 0) else -q


def _g(x: float) -> str:
    """A double through a default-formatted std::ostream (precision 6, %g)."""
    return f"{x:.6g}"


def write_prop_files(lattice, sink, Nt: int, at: float, n_refine: int, directory: str = ".", width: float = 0.05,
                     overlap: bool = False, dagger: bool = False) -> list[str]:
    """Writes prop.cu's two files for the dual lattice,
    [dagger_][ov_]dual_prop_spacial_L<n>_Nt<Nt>.dat1 and ..._temporal_..., each
    row three setw(25) columns in the stream's default format."""
    spatial, temporal = prop_profiles(lattice, sink, Nt, at, width)
    out = []
    for kind, rows in (("spacial", spatial), ("temporal", temporal)):
        name = "dual_" + f"prop_{kind}_L{n_refine}_Nt{Nt}.dat1"
        if overlap:
            name = "ov_" + name
        if dagger:
            name = "dagger_" + name
        path = os.path.join(directory, name)
        with open(path, "w") as f:
            for r in rows:
                f.write(f"{_g(r[0]):>25} {_g(r[1]):>25} {_g(r[2]):>25}\n")
        out.append(path)
    return out


class Corr:
    """Corr (src/both_3d/analyze_corr.cpp:15-96): the first number of each line of a file."""

    def __init__(self, path: str | None = None):
        self.data = np.zeros(0)
        if path is not None:
            vals = []
            with open(path) as f:
                for line in f:
                    tok = line.split()
                    if not tok:
                        raise ValueError(f"{path}: empty line (the reference reads an indeterminate value)")
                    vals.append(float(tok[0]))
            self.data = np.array(vals)


def jackknife(binavgs: list[np.ndarray]) -> tuple[np.ndarray, np.ndarray]:
    """Jackknife::do_it (src/both_3d/analyze_corr.cpp:100-145): leave-one-out
    bin averages, their mean and (nbins-1)/nbins times the sum of squared
    deviations, accumulated in the reference's order."""
    nb = len(binavgs)
    jack = []
    for i in range(nb):
        acc = None
        for j in range(nb):
            if i == j:
                continue
            acc = binavgs[j].copy() if acc is None else acc + binavgs[j]
        jack.append(acc / (nb - 1.0))
    est = None
    for i in range(nb):
        est = jack[i].copy() if est is None else est + jack[i]
    est = est / nb
    var = None
    for i in range(nb):
        d = jack[i] - est
        var = d * d if var is None else var + d * d
    var = var / nb
    var = var * (nb - 1.0)
    return est, var


def analyze_corr(path: str, header: str, conf_min: int, conf_max: int, interval: int, Nt: int, binsize: int,
                 prefix_max: int) -> tuple[np.ndarray, np.ndarray, list[str]]:
    """analyze_corr's main (src/both_3d/analyze_corr.cpp:151-211): files
    path<prefix>/<header><conf>.dat for prefix 1..prefix_max; conf_max is
    lowered to the last conf present in every stream; bins of binsize
    configurations (interval apart); jackknife over all streams' bins.
    Returns (estimate, error, the program's output lines)."""
    lines = [f"# path = {path}", f"# header = {header}", f"# conf_min = {conf_min}", f"# interval = {interval}",
             f"# Nt = {Nt}", f"# binsize = {binsize}"]
    fname = lambda prefix, conf: path + str(prefix) + "/" + header + str(conf) + ".dat"
    min_min = conf_max
    for prefix in range(1, prefix_max + 1):
        tmp = 0
        for conf in range(conf_min, conf_max, interval):
            f = fname(prefix, conf)
            lines.append(f"# file = {f}")
            if not os.path.exists(f):
                break
            tmp = conf
        min_min = min(min_min, tmp)
    conf_max = min_min
    nbins = _tdiv(_tdiv(conf_max - conf_min, interval), binsize)
    lines.append(f"# nbins = {nbins}")
    binavgs = []
    for prefix in range(1, prefix_max + 1):
        for ib in range(nbins):
            acc = None
            c0 = conf_min + ib * interval * binsize
            for conf in range(c0, conf_min + (ib + 1) * interval * binsize, interval):
                f = fname(prefix, conf)
                if not os.path.exists(f):
                    raise FileNotFoundError(f)
                d = Corr(f).data
                acc = d.copy() if acc is None else acc + d
            binavgs.append(acc / binsize)
    est, var = jackknife(binavgs)
    lines.append("# test ")
    err = np.sqrt(var)
    lines += [f"{_g(e)} {_g(s)}" for e, s in zip(est, err)]
    return est, err, lines
