"""Oracle pin of the XYZ core and the spin-permutation lattice tables it needs.

The reference's test_reference2.sh runs a hyperhoneycomb Heisenberg-Kitaev model (j = 0.1,
k = -1, range 3, 14 manual frequencies, cutoff 10 -> 0.3 x0.9) with the XYZ core and compares
its .obs with test/scripted/assets/test_reference2.ref.  The committed fixture holds those
golden correlations (XYZCorXX/YY/ZZ/DD at all 34 cutoffs); the oracle must reproduce them
(the reference's comparator allows 1e-5 absolute, test/scripted/assets/test_eval.py:12-27;
the restatement matches bit for bit).
"""
import os

import numpy as np

import spinparser_gb300 as spn
from oracle import SPIN_PERMUTATIONS, XyzOracle, xyz_initial_state, xyz_scatter

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def reference2():
    z = np.load(os.path.join(GOLDEN, "reference2_xyz.npz"))
    lat = spn.Lattice("hyperhoneycomb", 3, "hyperhoneycomb-kitaev", {"j": str(float(z["j"])), "k": str(float(z["k"]))},
                      resource_dir=os.path.join(GOLDEN, "res_hyperhoneycomb"))
    return z, lat.tables(), lat.spin_tables()


def test_spin_tables_of_the_kitaev_lattice():
    z, tab, st = reference2()
    assert (tab.n_basis, tab.n_range) == z["xx"].shape[1:]
    # the Kitaev couplings single out bond directions: some maps exchange spin components
    assert st.corr_perm.any() and st.overlap_perm1.any()
    assert np.all((st.corr_perm >= 0) & (st.corr_perm < 6))
    # the representative of every class is reached without a permutation
    assert not st.sites_perm.any()
    # positions of the correlation entries equal the reference's meta/sites
    np.testing.assert_allclose(tab.site_pos, z["sites"], atol=1e-5)


def test_spin_tables_are_trivial_for_su2_models():
    st = spn.Lattice("cubic", 3, "cubic-j1j2heisenberg", {"j1": "1", "j2": "0.25"}).spin_tables()
    for v in (st.sites_perm, st.inv_sites_perm, st.overlap_perm1, st.overlap_perm2, st.corr_perm):
        assert not v.any()


def test_xyz_oracle_reproduces_reference2_golden():
    z, tab, st = reference2()
    freq = np.sort(z["frequencies"])
    cs = z["cutoff_spec"]
    cut = spn.cutoff_exponential(float(cs[0]), float(cs[1]), float(cs[2]))
    np.testing.assert_array_equal(cut, z["cutoffs"])
    orc = XyzOracle(tab, st, freq)
    v2, v4 = xyz_initial_state(tab, len(freq))
    n, chi, _ = orc.flow(cut, v2, v4)
    assert n == len(cut)
    corr = np.stack([xyz_scatter(chi[k], tab, st) for k in range(n)])
    for c, name in enumerate(("xx", "yy", "zz", "dd")):
        np.testing.assert_allclose(corr[:, c], z[name], rtol=0, atol=1e-5)
        assert np.abs(corr[:, c] - z[name]).max() == 0.0  # bit-exact restatement


def test_xyz_oracle_fails_on_sign_flipped_kitaev():
    """Negative control in the spirit of test_referenceFail.sh: k -> -k must not match."""
    z, _, _ = reference2()
    lat = spn.Lattice("hyperhoneycomb", 3, "hyperhoneycomb-kitaev", {"j": str(float(z["j"])), "k": str(-float(z["k"]))},
                      resource_dir=os.path.join(GOLDEN, "res_hyperhoneycomb"))
    tab, st = lat.tables(), lat.spin_tables()
    freq = np.sort(z["frequencies"])
    cut = z["cutoffs"][:16]
    orc = XyzOracle(tab, st, freq)
    n, chi, _ = orc.flow(cut, *xyz_initial_state(tab, len(freq)))
    corr = xyz_scatter(chi[n - 1], tab, st)
    # the reference's comparator (1e-5 absolute) rejects it well before the end of the flow
    assert np.abs(corr[0] - z["xx"][n - 1]).max() > 1e-3


def test_spin_permutation_table_is_the_reference_enumeration():
    assert SPIN_PERMUTATIONS.tolist() == [[0, 1, 2], [0, 2, 1], [1, 0, 2], [1, 2, 0], [2, 0, 1], [2, 1, 0]]
