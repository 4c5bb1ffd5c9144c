"""Correlator analysis and propagator profiles of the S^2 x S^1 extension:
the jackknife restatement against the reference's own analyze_corr program
(built in place, output stored in tests/golden/analyze_corr_ref.json), the
angles of Geodesic::projectionS2, and the rows prop.cu writes."""
import json
import math
import os

import numpy as np
import pytest

import qed3_gb300 as Q
from qed3_gb300 import correlators as C

HERE = os.path.dirname(os.path.abspath(__file__))


def test_analyze_corr_matches_reference_output(tmp_path, monkeypatch):
    with open(os.path.join(HERE, "golden", "analyze_corr_ref.json")) as f:
        g = json.load(f)
    for rel, vals in g["files"].items():
        p = tmp_path / rel
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text("".join(f"{v!r} {0.5 * v!r}\n" for v in vals))
    monkeypatch.chdir(tmp_path)
    for run in g["runs"]:
        est, err, lines = C.analyze_corr(*run["args"])
        assert lines == run["stdout"], run["args"]
        assert est.shape == err.shape == (run["args"][5],)


def test_jackknife_of_constant_bins_has_zero_error():
    bins = [np.array([1.5, -2.0, 3.25])] * 5
    est, var = C.jackknife(bins)
    assert np.allclose(est, bins[0]) and np.all(var < 1e-28)
    # two bins: jackknife error = |b0 - b1| / 2 * sqrt(1) * ... = the standard error of the mean
    b = [np.array([1.0]), np.array([3.0])]
    est, var = C.jackknife(b)
    assert est[0] == 2.0 and math.isclose(math.sqrt(var[0]), 1.0)


def test_projection_s2():
    th, ph = C.projection_s2([0.0, 0.0, 2.0])
    assert th == 0.0 and ph == 0.0
    th, ph = C.projection_s2([0.0, 0.0, -1.0])
    assert th == math.pi and ph == 0.0
    th, ph = C.projection_s2([1.0, 1.0, 0.0])
    assert math.isclose(th, math.pi / 2) and math.isclose(ph, math.pi / 4)
    th, ph = C.projection_s2([1.0, -1.0, 0.0])
    assert math.isclose(ph, -math.pi / 4)
    th, ph = C.projection_s2([-1.0, 1e-300, 0.0])
    assert math.isclose(ph, math.pi)


def test_prop_profiles_rows():
    lat = Q.S2Trivalent(4)
    Nt, at = 3, 0.5
    rng = np.random.default_rng(1)
    sink = rng.normal(size=(Nt, lat.n_sites, 2)) + 1j * rng.normal(size=(Nt, lat.n_sites, 2))
    sp, tp = C.prop_profiles(lat, sink, Nt, at, width=0.3)
    th, ph, ln = C.site_angles(lat)
    assert ln[0] < 1e-7 and np.all(ln >= 0) and np.all(ln <= math.pi)
    sel = [i for i in range(lat.n_sites) if 0.0 <= ph[i] <= 0.3]
    fac = at * lat.tables()["means"][0]
    assert sp.shape == (2 * len(sel), 3) and len(sel) > 0
    assert np.allclose(sp[0::2, 0], th[sel]) and np.allclose(sp[1::2, 1], sink[0, sel, 1].real / fac)
    assert tp.shape == (2 * Nt, 3)
    assert np.allclose(tp[0::2, 0], at * np.arange(Nt)) and np.allclose(tp[1::2, 2], sink[:, 0, 1].imag / fac)


def test_write_prop_files_names_and_format(tmp_path):
    lat = Q.S2Trivalent(2)
    Nt, at = 2, 0.5
    sink = np.arange(Nt * lat.n_sites * 2, dtype=np.float64).astype(np.complex128) * (1 - 0.5j)
    paths = C.write_prop_files(lat, sink, Nt, at, 2, str(tmp_path), width=0.5, overlap=True, dagger=True)
    assert [os.path.basename(p) for p in paths] == ["dagger_ov_dual_prop_spacial_L2_Nt2.dat1",
                                                    "dagger_ov_dual_prop_temporal_L2_Nt2.dat1"]
    rows = open(paths[1]).read().splitlines()
    assert len(rows) == 2 * Nt and all(len(r) == 3 * 25 + 2 for r in rows)
    _, tp = C.prop_profiles(lat, sink, Nt, at, width=0.5)
    assert [float(x) for x in rows[2].split()] == [float(f"{v:.6g}") for v in tp[2]]
