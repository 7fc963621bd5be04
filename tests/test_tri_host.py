"""Host side of the TRI core (no GPU): the coefficient tables the kernels evaluate equal the
oracle's (and so the reference's generated flow equations), and the initial condition of
spn_tri_initial_state equals the oracle's."""
import os

import numpy as np

import spinparser_gb300 as spn
from oracle import TriOracle, tri_initial_state as oracle_initial_state

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def kitaev_gamma():
    z = np.load(os.path.join(GOLDEN, "reference3_tri.npz"))
    lat = spn.Lattice("honeycomb", 3, "honeycomb-kitaev-gamma",
                      {"j": str(float(z["j"])), "k": str(float(z["k"])), "g": str(float(z["g"]))},
                      resource_dir=os.path.join(GOLDEN, "res_honeycomb"))
    return z, lat


def test_device_tables_equal_the_oracle_tables():
    z, lat = kitaev_gamma()
    mine = spn.tri_tables()
    ref = TriOracle(lat.tables(), lat.spin_tables(), np.sort(z["frequencies"])).tables()
    assert mine.shape == ref.shape == (1152, 6)
    # the egg table keeps its zero-coefficient slots; the oracle writes b = 0 there as well
    np.testing.assert_array_equal(mine, ref)


def test_initial_state_matches_oracle():
    z, lat = kitaev_gamma()
    v2, v4 = spn.tri_initial_state(lat, 14)
    o2, o4 = oracle_initial_state(lat.tables(), 14)
    np.testing.assert_array_equal(v2, o2)
    np.testing.assert_array_equal(v4, o4)


def test_initial_state_normalization():
    z, lat = kitaev_gamma()
    _, a = spn.tri_initial_state(lat, 4, 1.0)
    _, b = spn.tri_initial_state(lat, 4, 2.0)
    np.testing.assert_allclose(b, a / np.float32(2.0), rtol=1e-7)
