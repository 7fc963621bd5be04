"""Oracle pin of the TRI core (time-reversal-invariant models with general couplings).

The reference's test_reference3.sh runs a honeycomb Heisenberg-Kitaev-Gamma model (j = 0.2,
k = 1, g = -0.1, range 3, 14 manual frequencies, cutoff 10 -> 0.3 x0.9) with the TRI core and
compares the ten correlation groups of its .obs (TRICorXX ... TRICorZZ, TRICorDD) with
test/scripted/assets/test_reference3.ref; test_reference2.sh runs the same script's Kitaev
model through both the XYZ and the TRI core against one .ref.  The comparator allows 1e-5
absolute (test/scripted/assets/test_eval.py:12-27).  The restatement builds the flow
equations' coefficient tables from the Pauli algebra and reproduces test_reference3.ref bit
for bit.
"""
import os

import numpy as np

import spinparser_gb300 as spn
from oracle import TRI_COMPONENTS, TriOracle, tri_initial_state, tri_scatter

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def reference3(g=None):
    z = np.load(os.path.join(GOLDEN, "reference3_tri.npz"))
    g = float(z["g"]) if g is None else g
    lat = spn.Lattice("honeycomb", 3, "honeycomb-kitaev-gamma",
                      {"j": str(float(z["j"])), "k": str(float(z["k"])), "g": str(g)},
                      resource_dir=os.path.join(GOLDEN, "res_honeycomb"))
    return z, lat.tables(), lat.spin_tables()


def test_coefficient_tables_follow_the_reference_terms():
    """Known terms of the generated flow equations, read from the reference source."""
    z, tab, st = reference3()
    rows = TriOracle(tab, st, np.sort(z["frequencies"])).tables()
    tabs = {k: rows[rows[:, 0] == k] for k in range(6)}
    assert [len(tabs[k]) for k in range(6)] == [256, 256, 64, 256, 256, 64]
    # every ladder term pairs A(a) with B(a ^ c ^ 15) (Pauli product of the two components)
    for k in (0, 1):
        t = tabs[k]
        assert np.array_equal(t[:, 4], t[:, 3] ^ t[:, 1] ^ 15)
        assert set(np.unique(t[:, 5])) == {-1, 1}
    # density-density output of the particle-particle ladder, a = 15 .. 0
    # (TRIFrgCore.cpp:199-230: multAdd for a = 15, 10, 9, 8, 6, 5, 4, 2, 1, 0)
    pp15 = tabs[0][tabs[0][:, 1] == 15]
    assert pp15[:, 3].tolist() == list(range(15, -1, -1))
    assert pp15[:, 5].tolist() == [1, -1, -1, -1, -1, 1, 1, 1, -1, 1, 1, 1, -1, 1, 1, 1]
    # the particle-hole ladder starts with minus A(DD) B(DD) for DD (TRIFrgCore.cpp:2390)
    ph15 = tabs[1][tabs[1][:, 1] == 15]
    assert ph15[0, 3:].tolist() == [15, 15, -1]
    # RPA of XX: minus the density inner index, plus the spin ones (TRIFrgCore.cpp:740-770)
    rpa0 = tabs[2][tabs[2][:, 1] == 0]
    assert rpa0[:, 3:].tolist() == [[3, 12, -1], [2, 8, 1], [1, 4, 1], [0, 0, 1]]
    # egg diagram of the measurement, XY: + vdz - vzd + vyx + vxy
    # (TRIMeasurementCorrelation.cpp:219-222)
    egg1 = tabs[5][tabs[5][:, 1] == 1]
    assert egg1[:, 3].tolist() == [14, 11, 4, 1] and egg1[:, 5].tolist() == [1, -1, 1, 1]


def test_tri_oracle_reproduces_reference3_golden():
    z, tab, st = reference3()
    assert (tab.n_basis, tab.n_range) == z["xx"].shape[1:]
    np.testing.assert_allclose(tab.site_pos, z["sites"], atol=1e-5)
    freq = np.sort(z["frequencies"])
    cs = z["cutoff_spec"]
    cut = spn.cutoff_exponential(float(cs[0]), float(cs[1]), float(cs[2]))
    np.testing.assert_array_equal(cut, z["cutoffs"])
    orc = TriOracle(tab, st, freq)
    n, chi, _ = orc.flow(cut, *tri_initial_state(tab, len(freq)))
    assert n == len(cut)
    corr = np.stack([tri_scatter(chi[k], tab, st) for k in range(n)])
    for q, name in enumerate(TRI_COMPONENTS):
        np.testing.assert_allclose(corr[:, q], z[name], rtol=0, atol=1e-5)
        assert np.abs(corr[:, q] - z[name]).max() == 0.0  # bit-exact restatement


def test_tri_oracle_reproduces_reference2_golden():
    """test_reference2.sh's TRI run: the Kitaev model through the TRI core against the
    same .ref as the XYZ core."""
    z = np.load(os.path.join(GOLDEN, "reference2_xyz.npz"))
    lat = spn.Lattice("hyperhoneycomb", 3, "hyperhoneycomb-kitaev", {"j": str(float(z["j"])), "k": str(float(z["k"]))},
                      resource_dir=os.path.join(GOLDEN, "res_hyperhoneycomb"))
    tab, st = lat.tables(), lat.spin_tables()
    orc = TriOracle(tab, st, np.sort(z["frequencies"]))
    n, chi, _ = orc.flow(z["cutoffs"], *tri_initial_state(tab, len(z["frequencies"])))
    assert n == len(z["cutoffs"])
    corr = np.stack([tri_scatter(chi[k], tab, st) for k in range(n)])
    for q, name in ((0, "xx"), (4, "yy"), (8, "zz"), (9, "dd")):
        np.testing.assert_allclose(corr[:, q], z[name], rtol=0, atol=1e-5)
    # no off-diagonal correlations for a diagonal model
    assert np.abs(corr[:, [1, 2, 3, 5, 6, 7]]).max() == 0.0


def test_tri_oracle_fails_on_sign_flipped_gamma():
    """Negative control in the spirit of test_referenceFail.sh: g -> -g must not match."""
    z, tab, st = reference3(g=-float(np.load(os.path.join(GOLDEN, "reference3_tri.npz"))["g"]))
    freq = np.sort(z["frequencies"])
    cut = z["cutoffs"][:16]
    n, chi, _ = TriOracle(tab, st, freq).flow(cut, *tri_initial_state(tab, len(freq)))
    corr = tri_scatter(chi[n - 1], tab, st)
    assert np.abs(corr[1] - z["xy"][n - 1]).max() > 1e-3


def test_initial_state_holds_the_full_coupling_matrix():
    z, tab, st = reference3()
    v2, v4 = tri_initial_state(tab, 4)
    v4 = v4.reshape(-1, 4, 4, tab.n_sites)
    assert not v2.any() and not v4[:, 3].any() and not v4[:, :, 3].any()
    # the Gamma coupling puts off-diagonal spin components on the nearest-neighbour bond
    assert np.abs(v4[0, :3, :3]).max() > 0 and any(v4[0, a, b].any() for a in range(3) for b in range(3) if a != b)
    np.testing.assert_array_equal(v4[0], v4[-1])
