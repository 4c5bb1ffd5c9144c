"""Product lattice builder vs the oracle: integer tables, coordinates and areas
bit-exact; the spin connection (closed form vs quadrature) to 1e-14."""
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
