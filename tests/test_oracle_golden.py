"""The CPU oracle is pinned to the reference's own golden data before it is trusted:
  * test/scripted/assets/test_reference1.ref (hyperkagome r3, all 34 cutoffs, ZZ and DD);
  * the numeric expectations of test/scripted/assets/test_python_obs.py (honeycomb r3);
  * the J -> -J negative control of test_referenceFail.sh must fail the same comparison.
"""
import json
import os

import numpy as np

import spinparser_gb300 as spn
from oracle import Oracle
from obs_queries import evaluate_query

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _hyperkagome():
    tab = spn.LatticeTables.from_npz(os.path.join(GOLDEN, "hyperkagome_r3_tables.npz"))
    g = np.load(os.path.join(GOLDEN, "reference1_su2.npz"))
    return tab, g


def test_reference1_cutoff_grid_bit_exact():
    _, g = _hyperkagome()
    cmax, cmin, step = (float(x) for x in g["cutoff_spec"])
    assert np.array_equal(spn.cutoff_exponential(cmax, cmin, step), g["cutoffs"])


def test_reference1_lattice_metadata_matches_golden_file():
    tab, g = _hyperkagome()
    assert np.allclose(tab.lattice_vectors, g["lattice_vectors"], atol=1e-6)
    assert np.allclose(tab.basis_pos, g["basis"], atol=1e-6)
    assert np.allclose(tab.site_pos, g["sites"], atol=1e-6)


def test_oracle_reproduces_reference1_golden():
    tab, g = _hyperkagome()
    orc = Oracle(tab, g["frequencies"])
    n, cs, cd, _ = orc.flow(g["cutoffs"], *tab.initial_state(len(g["frequencies"])))
    assert n == len(g["cutoffs"])
    corr = tab.corr_rid.reshape(tab.n_basis, tab.n_range)
    # the comparator of the reference's scripted tests: absolute 1e-5 (test_eval.py)
    assert float(np.abs(cs[:, corr] - g["zz"]).max()) < 1e-5
    assert float(np.abs(cd[:, corr] - g["dd"]).max()) < 1e-5


def test_oracle_negative_control_fails_reference1():
    tab, g = _hyperkagome()
    tab.interaction_J = -tab.interaction_J
    orc = Oracle(tab, g["frequencies"])
    n, cs, _, _ = orc.flow(g["cutoffs"], *tab.initial_state(len(g["frequencies"])))
    corr = tab.corr_rid.reshape(tab.n_basis, tab.n_range)
    assert float(np.abs(cs[:n, corr] - g["zz"][:n]).max()) > 1e-5


def test_oracle_reproduces_python_obs_expectations():
    spec = json.load(open(os.path.join(GOLDEN, "python_obs_honeycomb.json")))
    t = spec["task"]
    tab = spn.Lattice(t["lattice"], t["range"], t["model"], {"j": str(t["j"])}).tables()
    freq = np.array(t["frequencies"], np.float32)
    cut = spn.cutoff_exponential(t["cutoff_max"], t["cutoff_min"], t["cutoff_step"])
    orc = Oracle(tab, freq)
    n, cs, _, _ = orc.flow(cut, *tab.initial_state(len(freq)))
    zz = cs[:, tab.corr_rid].reshape(n, tab.n_basis, tab.n_range)
    for q in spec["queries"]:
        got = evaluate_query(q, cut[:n], zz, tab)
        assert np.isclose(got, np.array(q["expect"]), rtol=1e-5, atol=1e-16).all(), q["what"]


def test_oracle_fp64_close_to_fp32_on_one_rhs():
    """The FP64 instantiation follows the same code path: on one RHS it agrees with the
    FP32 reference-order result to FP32 rounding."""
    tab = spn.Lattice("square", 3, "square-heisenberg", {"j": "1.0"}).tables()
    freq = spn.frequency_exponential(0.05, 20.0, 8)
    orc = Oracle(tab, freq)
    v2, ss, dd = tab.initial_state(8)
    a = orc.rhs(1.0, v2, ss, dd)
    b = orc.rhs(1.0, v2, ss, dd, fp64=True)
    for x, y in zip(a, b):
        assert float(np.abs(x - y).max()) <= 1e-5 * float(np.abs(y).max())
