"""GPU parity of the XYZ core (spn_xyz_*) against the oracle and the reference's golden output.

Tolerances as for the SU(2) core: one RHS within normwise relative error 1e-5 per component,
correlations within 1e-5 absolute of test_reference2.ref (the reference's comparator,
test/scripted/assets/test_eval.py:12-27).
"""
import os

import numpy as np
import pytest

import spinparser_gb300 as spn
from oracle import XyzOracle, xyz_initial_state as oracle_initial_state, xyz_scatter

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RHS_TOL = 1e-5


def normwise(g, r):
    return float(np.max(np.abs(np.asarray(g, np.float64) - r)) / max(float(np.max(np.abs(r))), 1e-300))


def kitaev():
    z = np.load(os.path.join(GOLDEN, "reference2_xyz.npz"))
    lat = spn.Lattice("hyperhoneycomb", 3, "hyperhoneycomb-kitaev", {"j": str(float(z["j"])), "k": str(float(z["k"]))},
                      resource_dir=os.path.join(GOLDEN, "res_hyperhoneycomb"))
    return z, lat


def oracle_state(orc, cut, v2, v4, steps):
    c = np.float32(cut[0])
    for k in range(steps):
        d2, d4 = orc.rhs(c, v2, v4)
        st = np.float32(np.float32(cut[k + 1]) - c)
        v2 = (v2 + st * d2).astype(np.float32)
        v4 = (v4 + st * d4).astype(np.float32)
        c = np.float32(cut[k + 1])
    return c, v2, v4


def test_initial_state_matches_oracle():
    z, lat = kitaev()
    tab = lat.tables()
    v2, v4 = spn.xyz_initial_state(lat, 14)
    o2, o4 = oracle_initial_state(tab, 14)
    np.testing.assert_array_equal(v2, o2)
    np.testing.assert_array_equal(v4, o4)


@pytest.mark.parametrize("case", ["kitaev", "square-r11", "square-r15"])
def test_xyz_rhs_matches_oracle(case):
    if case == "kitaev":
        z, lat = kitaev()
        freq = np.sort(z["frequencies"])
        cut = z["cutoffs"]
        steps = 5
    elif case == "square-r15":  # 72 sites: four sites per lane
        lat = spn.Lattice("square", 15, "square-heisenberg", {"j": "1.0"})
        freq = spn.frequency_exponential(0.01, 30.0, 4)
        cut = spn.cutoff_exponential(30.0, 0.05, 0.9)
        steps = 2
    else:  # 42 sites: two sites per lane
        lat = spn.Lattice("square", 11, "square-heisenberg", {"j": "1.0"})
        freq = spn.frequency_exponential(0.01, 30.0, 6)
        cut = spn.cutoff_exponential(30.0, 0.05, 0.9)
        steps = 2
    tab, st = lat.tables(), lat.spin_tables()
    orc = XyzOracle(tab, st, freq)
    c, v2, v4 = oracle_state(orc, cut, *oracle_initial_state(tab, len(freq)), steps)
    flow = spn.XyzFlow(tab, st, freq)
    flow.set_state(float(c), v2, v4)
    flow.compute_step()
    g2, g4 = flow.get_flow()
    r2, r4 = orc.rhs(c, v2, v4)
    assert normwise(g2, r2) <= RHS_TOL
    for q in range(4):
        assert normwise(g4[q], r4[q]) <= RHS_TOL, q
    assert not flow.is_diverged()
    # measurement at the same state
    corr, chi = flow.measure_correlation()
    ochi = orc.correlation(c, v2, v4)
    np.testing.assert_allclose(chi, ochi, rtol=1e-5, atol=1e-6)
    ocorr = xyz_scatter(ochi, tab, st).reshape(4, -1)
    np.testing.assert_allclose(corr, ocorr, rtol=1e-5, atol=1e-6)


def test_xyz_flow_matches_reference2_golden():
    """The XYZ task of test_reference2.sh on the GPU, all 34 cutoffs, against the .ref values."""
    z, lat = kitaev()
    tab, st = lat.tables(), lat.spin_tables()
    freq = np.sort(z["frequencies"])
    cs = z["cutoff_spec"]
    cut = spn.cutoff_exponential(float(cs[0]), float(cs[1]), float(cs[2]))
    flow = spn.XyzFlow(tab, st, freq)
    measured, corr, diverged = flow.run(cut, *spn.xyz_initial_state(lat, len(freq)))
    assert not diverged and len(measured) == len(z["cutoffs"])
    np.testing.assert_array_equal(measured, z["cutoffs"])
    corr = corr.reshape(len(measured), 4, tab.n_basis, tab.n_range)
    for q, name in enumerate(("xx", "yy", "zz", "dd")):
        np.testing.assert_allclose(corr[:, q], z[name], rtol=0, atol=1e-5)


def test_xyz_state_round_trip():
    z, lat = kitaev()
    tab, st = lat.tables(), lat.spin_tables()
    freq = np.sort(z["frequencies"])
    flow = spn.XyzFlow(tab, st, freq)
    rng = np.random.default_rng(3)
    v2 = rng.standard_normal(len(freq)).astype(np.float32)
    v4 = rng.standard_normal((4, flow.fn * flow.nl)).astype(np.float32)
    flow.set_state(2.5, v2, v4)
    c, g2, g4 = flow.get_state()
    assert c == np.float32(2.5)
    np.testing.assert_array_equal(g2, v2)
    np.testing.assert_array_equal(g4, v4)
