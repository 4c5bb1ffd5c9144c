"""Host-side sources (FermionVector, src/dual/valence.h:47-60): Z2 noise
streams and point sources against the oracle's restatement of ParallelRng2."""
import numpy as np
import pytest

import qed3_gb300 as Q
from oracle import oracle as O


def test_z2_spinor_stream_matches_oracle():
    g = O.geometry(4)
    lat = Q.S2Trivalent(4)
    r1, r2 = O.Rng(g, 11), Q.ParallelRng(lat, 11)
    a, b = r1.z2_spinor(), r2.z2_spinor()
    assert np.array_equal(a, b)
    scaled = np.concatenate([a.real, a.imag]) * np.sqrt(2 * g.n_sites)
    assert set(np.round(scaled).astype(int)) <= {1, 2}
    # the site engines advance: a second draw differs and still agrees
    a2, b2 = r1.z2_spinor(), r2.z2_spinor()
    assert np.array_equal(a2, b2) and not np.array_equal(a, a2)


def test_point_source():
    lat = Q.S2Trivalent(2)
    v = Q.point_source(lat, 5, 1)
    assert v.shape == (2 * lat.n_sites,)
    assert v[2 * 5 + 1] == 1.0 and np.count_nonzero(v) == 1
    with pytest.raises(Q.Qed3Error):
        Q.point_source(lat, lat.n_sites, 0)
