"""GPU parity of the TRI core (spn_tri_*) against the oracle and the reference's golden output.

Tolerances as for the SU(2) and XYZ cores: one RHS within normwise relative error 1e-5 (the
16 components together, and each component against the largest magnitude of the vertex),
correlations within 1e-5 absolute of test_reference3.ref / test_reference2.ref (the
reference's comparator, test/scripted/assets/test_eval.py:12-27).
"""
import os

import numpy as np
import pytest

import spinparser_gb300 as spn
from oracle import TriOracle, tri_initial_state as oracle_initial_state, tri_scatter

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RHS_TOL = 1e-5


def kitaev_gamma(rng=3):
    z = np.load(os.path.join(GOLDEN, "reference3_tri.npz"))
    lat = spn.Lattice("honeycomb", rng, "honeycomb-kitaev-gamma",
                      {"j": str(float(z["j"])), "k": str(float(z["k"])), "g": str(float(z["g"]))},
                      resource_dir=os.path.join(GOLDEN, "res_honeycomb"))
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
    _, lat = kitaev_gamma()
    v2, v4 = spn.tri_initial_state(lat, 14)
    o2, o4 = oracle_initial_state(lat.tables(), 14)
    np.testing.assert_array_equal(v2, o2)
    np.testing.assert_array_equal(v4, o4)


@pytest.mark.parametrize("case", ["kitaev-gamma-r3", "kitaev-gamma-r11", "square-r11", "square-r15"])
def test_tri_rhs_matches_oracle(case):
    if case == "kitaev-gamma-r3":
        z, lat = kitaev_gamma()
        freq = np.sort(z["frequencies"])
        cut = z["cutoffs"]
        steps = 5
    elif case == "kitaev-gamma-r11":  # more than 32 sites, permuted spin components
        _, lat = kitaev_gamma(11)
        freq = spn.frequency_exponential(0.02, 20.0, 6)
        cut = spn.cutoff_exponential(20.0, 0.1, 0.85)
        steps = 2
    elif case == "square-r15":  # 72 sites: three site blocks per warp
        lat = spn.Lattice("square", 15, "square-heisenberg", {"j": "1.0"})
        freq = spn.frequency_exponential(0.01, 30.0, 4)
        cut = spn.cutoff_exponential(30.0, 0.05, 0.9)
        steps = 2
    else:  # 42 sites of an SU(2)-symmetric model
        lat = spn.Lattice("square", 11, "square-heisenberg", {"j": "1.0"})
        freq = spn.frequency_exponential(0.01, 30.0, 6)
        cut = spn.cutoff_exponential(30.0, 0.05, 0.9)
        steps = 2
    tab, st = lat.tables(), lat.spin_tables()
    orc = TriOracle(tab, st, freq)
    c, v2, v4 = oracle_state(orc, cut, *oracle_initial_state(tab, len(freq)), steps)
    flow = spn.TriFlow(tab, st, freq)
    flow.set_state(float(c), v2, v4)
    flow.compute_step()
    g2, g4 = flow.get_flow()
    r2, r4 = orc.rhs(c, v2, v4)
    scale = float(np.max(np.abs(r4)))
    assert scale > 0
    np.testing.assert_allclose(g2, r2, rtol=RHS_TOL, atol=RHS_TOL * float(np.max(np.abs(r2))))
    assert float(np.max(np.abs(g4 - r4))) <= RHS_TOL * scale
    g4 = g4.reshape(-1, 16, tab.n_sites)
    r4 = r4.reshape(-1, 16, tab.n_sites)
    for q in range(16):
        sq = float(np.max(np.abs(r4[:, q])))
        assert float(np.max(np.abs(g4[:, q] - r4[:, q]))) <= RHS_TOL * max(sq, 1e-3 * scale), q
    assert not flow.is_diverged()
    # measurement at the same state
    corr, chi = flow.measure_correlation()
    ochi = orc.correlation(c, v2, v4)
    np.testing.assert_allclose(chi, ochi, rtol=1e-5, atol=1e-6)
    ocorr = tri_scatter(ochi, tab, st).reshape(10, -1)
    np.testing.assert_allclose(corr, ocorr, rtol=1e-5, atol=1e-6)


def test_tri_flow_matches_reference3_golden():
    """test_reference3.sh on the GPU, all 34 cutoffs, against the .ref values."""
    z, lat = kitaev_gamma()
    tab, st = lat.tables(), lat.spin_tables()
    freq = np.sort(z["frequencies"])
    cs = z["cutoff_spec"]
    cut = spn.cutoff_exponential(float(cs[0]), float(cs[1]), float(cs[2]))
    flow = spn.TriFlow(tab, st, freq)
    measured, corr, diverged = flow.run(cut, *spn.tri_initial_state(lat, len(freq)))
    assert not diverged and len(measured) == len(z["cutoffs"])
    np.testing.assert_array_equal(measured, z["cutoffs"])
    corr = corr.reshape(len(measured), 10, tab.n_basis, tab.n_range)
    for q, name in enumerate(spn.TRI_COMPONENTS):
        np.testing.assert_allclose(corr[:, q], z[name], rtol=0, atol=1e-5)


def test_tri_flow_matches_reference2_golden():
    """test_reference2.sh's TRI run: the hyperhoneycomb Kitaev model through the TRI core."""
    z = np.load(os.path.join(GOLDEN, "reference2_xyz.npz"))
    lat = spn.Lattice("hyperhoneycomb", 3, "hyperhoneycomb-kitaev", {"j": str(float(z["j"])), "k": str(float(z["k"]))},
                      resource_dir=os.path.join(GOLDEN, "res_hyperhoneycomb"))
    tab, st = lat.tables(), lat.spin_tables()
    freq = np.sort(z["frequencies"])
    flow = spn.TriFlow(tab, st, freq)
    measured, corr, diverged = flow.run(z["cutoffs"], *spn.tri_initial_state(lat, len(freq)))
    assert not diverged and len(measured) == len(z["cutoffs"])
    corr = corr.reshape(len(measured), 10, tab.n_basis, tab.n_range)
    for q, name in ((0, "xx"), (4, "yy"), (8, "zz"), (9, "dd")):
        np.testing.assert_allclose(corr[:, q], z[name], rtol=0, atol=1e-5)


def test_tri_state_round_trip():
    z, lat = kitaev_gamma()
    tab, st = lat.tables(), lat.spin_tables()
    freq = np.sort(z["frequencies"])
    flow = spn.TriFlow(tab, st, freq)
    rng = np.random.default_rng(5)
    v2 = rng.standard_normal(len(freq)).astype(np.float32)
    v4 = rng.standard_normal(flow.size).astype(np.float32)
    flow.set_state(1.5, v2, v4)
    c, g2, g4 = flow.get_state()
    assert c == np.float32(1.5)
    np.testing.assert_array_equal(g2, v2)
    np.testing.assert_array_equal(g4, v4)
