"""Product lattice builder vs the oracle: integer tables, coordinates and areas
bit-exact; the spin connection (closed form vs quadrature) to 1e-14."""
import os

import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O


def wrap(a):
    return np.mod(a + np.pi, 2 * np.pi) - np.pi


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 16, 32])
def test_tables_match_oracle(n):
    lat = Q.S2Trivalent(n)
    t = lat.tables()
    g = O.geometry(n)
    for k in ("sites", "nns", "links", "simp_links", "face_offsets", "face_sites", "ell", "link_volume", "vols"):
        assert np.array_equal(t[k], getattr(g, k)), k
    assert np.array_equal(t["means"], [g.mean_ell, g.mean_link_volume, g.mean_vol])
    assert np.abs(t["omega"] - g.omega).max() < 1e-14
    assert np.abs(wrap(t["alpha"] - g.alpha)).max() < 1e-14
    # reference ranges: alpha(x<y) in [-pi, pi], alpha(x>y) in [0, 2pi)
    x = np.arange(lat.n_sites)[:, None]
    hi = t["nns"] < x
    assert (t["alpha"][hi] >= 0).all() and (t["alpha"][hi] < 2 * np.pi).all()


def test_permutation_is_a_bijection():
    lat = Q.S2Trivalent(16)
    p = lat.permutation()
    assert np.array_equal(np.sort(p), np.arange(lat.n_sites))


def test_large_lattice_sizes():
    lat = Q.S2Trivalent(128)
    assert (lat.n_sites, lat.n_links, lat.n_faces) == (327680, 491520, 163842)
    t = lat.tables()
    assert abs(t["link_volume"].sum() - 4 * np.pi) < 1e-9


def test_invalid_refinement_is_an_error():
    with pytest.raises(Q.Qed3Error) as e:
        Q.S2Trivalent(0)
    assert e.value.status == Q.ERR_ARG


def test_zolotarev_against_reference_fixture():
    """Product Zolotarev (A&S AGM Jacobi functions) vs the reference's own code.

    The reference evaluates cn as sqrt(1 - sn^2), which loses relative accuracy
    ~eps/cn^2 on the poles near K'; the product keeps ~eps/cn.  So coefficients
    agree to 1e-9 relative, and the product's r(x) is at least as close to
    sign(x) on [k, 1] as the reference's (at the Zolotarev bound Delta when
    FP64 allows)."""
    import json
    import os
    data = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "zolotarev_ref.json")))
    h = lambda v: np.array([float.fromhex(s) for s in v])

    def r(z, x):
        res = np.ones_like(x)
        for m in range(1, z["size"]):
            res = res + z["A"][m] / (x * x - z["k"] ** 2 / z["cp"][m])
        return res * z["C"] * x

    for c in data["cases"]:
        z = Q.zolotarev(c["k"], c["n"])
        ref = dict(c=h(c["c"]), cp=h(c["cp"]), A=h(c["A"]), size=z["size"], k=c["k"],
                   **{key: float.fromhex(c[key]) for key in ("M", "lambda_inv", "E", "C")})
        for key in ("c", "cp", "A"):
            assert np.allclose(z[key], ref[key], rtol=1e-9, atol=0), (c["k"], c["n"], key)
        for key in ("M", "lambda_inv", "E", "C"):
            assert abs(z[key] - ref[key]) <= 1e-9 * abs(ref[key]), key
        x = np.geomspace(c["k"], 1.0, 20001)
        delta = (ref["lambda_inv"] - 1) / (ref["lambda_inv"] + 1)
        err_q = np.abs(r(z, x) - 1).max()
        err_ref = np.abs(r(ref, x) - 1).max()
        assert err_q <= max(1.01 * err_ref, 2 * abs(delta), 1e-13), (c["k"], c["n"], err_q, err_ref, delta)


def _relabelled_mesh(n, seed):
    """The n-refined mesh with its vertices and triangles renumbered at random and
    every other triangle's winding reversed: how another generator (the
    reference's QFE-based tables) may number the same sphere."""
    lat = Q.S2Trivalent(n)
    v, t = lat.mesh()
    rng = np.random.default_rng(seed)
    pv = rng.permutation(v.shape[0])          # new vertex k = old vertex pv[k]
    inv_v = np.argsort(pv)
    pt = rng.permutation(t.shape[0])          # new triangle (dual site) s = old triangle pt[s]
    t2 = inv_v[t[pt]]
    t2[::2] = t2[::2, ::-1]
    return lat, v[pv], t2, pv, pt


def test_mesh_round_trip_is_identical():
    lat = Q.S2Trivalent(6)
    v, t = lat.mesh()
    lat2 = Q.S2Trivalent.from_mesh(v, t)
    a, b = lat.tables(), lat2.tables()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(lat.permutation(), lat2.permutation())


def test_mesh_in_a_callers_numbering():
    """Sites, links and faces follow the caller's numbering; lengths and areas
    are those of the same geometric objects; omega(x, y) and alpha keep the
    reference's conventions for the new labels (equal up to orientation and 2 pi)."""
    lat, v2, t2, pv, pt = _relabelled_mesh(4, 1)
    lat2 = Q.S2Trivalent.from_mesh(v2, t2)
    a, b = lat.tables(), lat2.tables()
    assert np.abs(b["sites"] - a["sites"][pt]).max() < 1e-15
    inv_t = np.argsort(pt)
    old_links = {tuple(l): i for i, l in enumerate(a["links"])}
    for i, (x, y) in enumerate(b["links"]):
        ox, oy = pt[x], pt[y]
        j = old_links[(min(ox, oy), max(ox, oy))]
        sgn = 1.0 if ox < oy else -1.0
        assert abs(b["ell"][i] - a["ell"][j]) < 1e-14
        assert abs(b["link_volume"][i] - a["link_volume"][j]) < 1e-15
        assert abs(wrap(b["omega"][i] - sgn * a["omega"][j])) < 1e-13
    assert np.abs(b["vols"] - a["vols"][pv]).max() < 1e-15
    for s in range(lat2.n_sites):
        for k in range(3):
            o = pt[s]
            ko = list(a["nns"][o]).index(pt[b["nns"][s][k]])
            assert abs(wrap(b["alpha"][s][k] - a["alpha"][o][ko])) < 1e-13
    assert abs(b["means"][2] - a["means"][2]) < 1e-15


def test_mesh_with_a_link_order():
    lat = Q.S2Trivalent(3)
    v, t = lat.mesh()
    a = lat.tables()
    order = np.random.default_rng(2).permutation(lat.n_links)
    lat2 = Q.S2Trivalent.from_mesh(v, t, links=a["links"][order])
    b = lat2.tables()
    assert np.array_equal(b["links"], a["links"][order])
    for k in ("simp_links", "ell", "link_volume", "omega"):
        assert np.array_equal(b[k], a[k][order]), k
    for k in ("sites", "nns", "face_offsets", "face_sites", "vols", "alpha"):
        assert np.array_equal(b[k], a[k]), k


def test_bad_meshes_are_errors():
    lat = Q.S2Trivalent(2)
    v, t = lat.mesh()
    bad = [t[:-2],                                   # open surface (and V - E + F != 2)
           np.concatenate([t[:-1], t[:1]]),          # a triangle twice, one missing
           np.where(np.arange(t.size).reshape(t.shape) == 4, t[0, 0], t)]   # repeated vertex
    for tb in bad:
        with pytest.raises(Q.Qed3Error) as e:
            Q.S2Trivalent.from_mesh(v, tb)
        assert e.value.status == Q.ERR_ARG
    links = lat.tables()["links"].copy()
    for lb in (np.concatenate([links[:-1], links[:1]]), np.concatenate([links[:-1], [[0, 0]]])):
        with pytest.raises(Q.Qed3Error) as e:
            Q.S2Trivalent.from_mesh(v, t, links=lb)
        assert e.value.status == Q.ERR_ARG


def test_caller_spin_structure_is_used():
    lat = Q.S2Trivalent(3)
    t = lat.tables()
    om = t["omega"] + 0.25
    al = t["alpha"] - 0.5
    lat.set_spin_structure(om, al)
    t2 = lat.tables()
    assert np.array_equal(t2["omega"], om) and np.array_equal(t2["alpha"], al)
    lat.set_spin_structure(omega=t["omega"])
    assert np.array_equal(lat.tables()["omega"], t["omega"]) and np.array_equal(lat.tables()["alpha"], al)
    bad = t["omega"].copy()
    bad[3] = np.nan
    with pytest.raises(Q.Qed3Error):
        lat.set_spin_structure(bad)


def test_mesh_with_oriented_links():
    """Links listed (j, i) point j -> i: the tables keep that orientation, omega
    changes sign, and the hop signs follow the stored direction."""
    lat = Q.S2Trivalent(3)
    v, t = lat.mesh()
    a = lat.tables()
    flip = np.zeros(lat.n_links, bool)
    flip[::3] = True
    links = a["links"].copy()
    links[flip] = links[flip][:, ::-1]
    b = Q.S2Trivalent.from_mesh(v, t, links=links).tables()
    assert np.array_equal(b["links"], links)
    assert np.array_equal(b["omega"][flip], -a["omega"][flip])
    assert np.array_equal(b["omega"][~flip], a["omega"][~flip])
    for k in ("sites", "nns", "face_sites", "ell", "link_volume", "vols", "alpha"):
        assert np.array_equal(b[k], a[k]), k


def test_reference_dat_files_round_trip(tmp_path):
    """The reference's .dat layout (get_geometry.cc / test_sorting.cc writers,
    s2n_simp.h / dirac_dual.h readers): write, read back, same lattice."""
    from qed3_gb300 import dats
    lat = Q.S2Trivalent(4)
    paths = dats.write(lat, str(tmp_path))
    assert len(paths) == 10
    names = sorted(os.path.basename(p) for p in paths)
    assert "face_dual_n4.dat" in names and "pts_dual_n4_singlepatch.dat" in names
    # row shapes as the reference's readers parse them
    first = open(os.path.join(str(tmp_path), "nns_dual_n4_singlepatch.dat")).readline().split()
    assert len(first) == 3 and all(s.lstrip("-").isdigit() for s in first)
    lat2 = dats.read(str(tmp_path), 4)
    assert lat2.max_site_deviation == 0.0
    a, b = lat.tables(), lat2.tables()
    for k in ("sites", "nns", "links", "simp_links", "face_offsets", "face_sites", "ell", "link_volume", "vols"):
        assert np.array_equal(a[k], b[k]), k
    assert np.abs(a["omega"] - b["omega"]).max() < 1e-14
    assert np.abs(a["alpha"] - b["alpha"]).max() < 1e-14


def test_reference_dat_files_in_another_numbering(tmp_path):
    """Files whose sites, vertices and link orientations differ from this
    project's numbering (a relabelled mesh, some links listed j -> i): the read
    lattice follows the files."""
    from qed3_gb300 import dats
    lat0, v2, t2, pv, pt = _relabelled_mesh(3, 11)
    links = Q.S2Trivalent.from_mesh(v2, t2).tables()["links"].copy()
    links[::5] = links[::5][:, ::-1]
    lat = Q.S2Trivalent.from_mesh(v2, t2, links=links)
    dats.write(lat, str(tmp_path), n_refine=3)
    # shuffle the triangle rows of face_n: the reader re-pairs them with pts_dual
    fp = os.path.join(str(tmp_path), "face_n3_singlepatch.dat")
    rows = open(fp).readlines()
    perm = np.random.default_rng(0).permutation(len(rows))
    open(fp, "w").writelines([rows[i] for i in perm])
    lat2 = dats.read(str(tmp_path), 3)
    a, b = lat.tables(), lat2.tables()
    assert np.abs(a["sites"] - b["sites"]).max() < 1e-15
    assert np.array_equal(a["links"], b["links"]) and np.array_equal(a["nns"], b["nns"])
    assert np.abs(a["omega"] - b["omega"]).max() < 1e-14
