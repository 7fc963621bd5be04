"""GPU parity: the sm_103a kernels (through the C ABI) against the CPU oracle and against the
reference's golden outputs.

Tolerances
  * one RHS evaluation: normwise relative error max|gpu - oracle| / max|oracle| <= 1e-5 per
    array (self-energy flow, spin vertex flow, density vertex flow);
  * Euler update: bit-exact (same float operations);
  * correlations: absolute 1e-5, the reference's own comparator tolerance
    (test/scripted/assets/test_eval.py:12-27), and rtol 1e-5 for the test_python_obs values.
"""
import json
import os

import numpy as np
import pytest

import spinparser_gb300 as spn
from spinparser_gb300.driver import run_flow
from oracle import Oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
pytestmark = pytest.mark.gpu

RHS_TOL = 1e-5


def normwise(g, r):
    return float(np.max(np.abs(np.asarray(g, np.float64) - r)) / max(float(np.max(np.abs(r))), 1e-300))


def oracle_state(orc, cutoffs, v2, ss, dd, steps):
    """Advances the initial state by `steps` oracle Euler steps; returns (cutoff, state)."""
    c = np.float32(cutoffs[0])
    for k in range(steps):
        d2, dss, ddd = orc.rhs(c, v2, ss, dd)
        nxt = np.float32(cutoffs[k + 1])
        st = np.float32(nxt - c)
        v2 = (v2 + st * d2).astype(np.float32)
        ss = (ss + st * dss).astype(np.float32)
        dd = (dd + st * ddd).astype(np.float32)
        c = nxt
    return c, v2, ss, dd


@pytest.fixture(scope="module")
def square_r3():
    lat = spn.Lattice("square", 3, "square-heisenberg", {"j": "1.0"})
    return lat.tables()


def test_rhs_square_r3_n32_matches_oracle(square_r3):
    """Config-1 shape (square r3, 32 frequencies in [0.005, 50]) from a state 3 steps into the flow."""
    tab = square_r3
    freq = spn.frequency_exponential(0.005, 50.0, 32)
    cut = spn.cutoff_exponential(50.0, 0.05, 0.98)
    orc = Oracle(tab, freq)
    c, v2, ss, dd = oracle_state(orc, cut, *tab.initial_state(32), steps=3)
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(float(c), v2, ss, dd)
    flow.compute_step()
    g2, gss, gdd = flow.get_flow()
    r2, rss, rdd = orc.rhs(c, v2, ss, dd)
    assert normwise(g2, r2) <= RHS_TOL
    assert normwise(gss, rss) <= RHS_TOL
    assert normwise(gdd, rdd) <= RHS_TOL
    assert not flow.is_diverged()


@pytest.mark.parametrize("lattice,rng,model,params,n", [
    ("square", 3, "square-heisenberg", {"j": "1.0"}, 14),
    ("cubic", 3, "cubic-j1j2heisenberg", {"j1": "1.0", "j2": "0.25"}, 14),
    ("square", 11, "square-heisenberg", {"j": "1.0"}, 8),   # 42 sites: a CTA per triple, w = 48
    ("square", 13, "square-heisenberg", {"j": "1.0"}, 6),   # 56 sites: w = 64
    ("square", 15, "square-heisenberg", {"j": "1.0"}, 6),   # 72 sites: w = 80, 256 threads
    ("square", 17, "square-heisenberg", {"j": "1.0"}, 4),   # 90 sites: w = 96
    ("square", 20, "square-heisenberg", {"j": "1.0"}, 4),   # 121 sites: w = 128
])
def test_every_vertex_variant_matches_oracle(lattice, rng, model, params, n):
    """Each kernel variant the autotuner may pick (1 or 2 nodes per site-group iteration, RPA
    schedule in shared or global memory) reproduces the oracle, and all variants give the
    same bits (a group takes its nodes in the same order whatever the variant), so autotuning
    never changes a result.  Lattices of 6 and 8 sites run the warp-per-triple kernel, of 42,
    56, 72, 90 and 121 sites the CTA-per-triple kernel (w = 48, 64, 80, 96, 128), which has no
    variants."""
    tab = spn.Lattice(lattice, rng, model, params).tables()
    freq = spn.frequency_exponential(0.01, 30.0, n)
    orc = Oracle(tab, freq)
    cut = np.array([3.0, 2.0, 1.0, 0.4], np.float32)
    c, v2, ss, dd = oracle_state(orc, cut, *tab.initial_state(n), steps=2)
    r2, rss, rdd = orc.rhs(c, v2, ss, dd)
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(float(c), v2, ss, dd)
    first = None
    ran = 0
    for npi in (1, 2):
        for sm in (False, True):
            try:
                flow.set_variant(npi, sm)
            except spn.SpnError as e:  # a variant whose shared memory does not fit this lattice
                assert e.code == -8, e
                continue
            ran += 1
            flow.compute_step()
            g2, gss, gdd = flow.get_flow()
            assert normwise(gss, rss) <= RHS_TOL, (npi, sm)
            assert normwise(gdd, rdd) <= RHS_TOL, (npi, sm)
            if first is None:
                first = (gss.copy(), gdd.copy())
            assert np.array_equal(gss, first[0]) and np.array_equal(gdd, first[1]), (npi, sm)
    assert ran >= 1
    choice = flow.autotune(2)
    assert choice["nodes_per_iteration"] in (1, 2) and choice["grid"] > 0
    flow.compute_step()
    _, gss, gdd = flow.get_flow()
    assert normwise(gss, rss) <= RHS_TOL and normwise(gdd, rdd) <= RHS_TOL


def test_rhs_small_mesh_late_cutoff(square_r3):
    """Small cutoff (below the smallest frequency) exercises the clamped interpolation and
    all three Katanin ranges."""
    tab = square_r3
    freq = spn.frequency_exponential(0.05, 20.0, 12)
    orc = Oracle(tab, freq)
    cut = np.array([0.5, 0.3, 0.1, 0.03], np.float32)
    c, v2, ss, dd = oracle_state(orc, cut, *tab.initial_state(12), steps=3)
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(float(c), v2, ss, dd)
    flow.compute_step()
    g2, gss, gdd = flow.get_flow()
    r2, rss, rdd = orc.rhs(c, v2, ss, dd)
    for g, r in ((g2, r2), (gss, rss), (gdd, rdd)):
        assert normwise(g, r) <= RHS_TOL


@pytest.mark.parametrize("lattice,rng,model,params,n", [
    ("cubic", 6, "cubic-j1j2heisenberg", {"j1": "1.0", "j2": "0.25"}, 64),
    ("pyrochlore", 5, "pyrochlore-heisenberg", {"j": "1.0"}, 64),
])
def test_rhs_large_configs_sampled(lattice, rng, model, params, n):
    """Full-size configurations: GPU advances the state two steps, then one RHS is checked
    on sampled triple ranges against the oracle (the full oracle RHS takes minutes)."""
    tab = spn.Lattice(lattice, rng, model, params).tables()
    freq = spn.frequency_exponential(0.005 if lattice == "cubic" else 0.002, 100.0, n)
    cut = spn.cutoff_exponential(100.0, 0.05, 0.98)
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(float(cut[0]), *tab.initial_state(n))
    for k in range(2):
        flow.compute_step()
        flow.finalize_step(float(cut[k + 1]))
    c, v2, ss, dd = flow.get_state()
    flow.compute_step()
    g2, gss, gdd = flow.get_flow()
    orc = Oracle(tab, freq)
    r2 = orc.self_energy(c, v2, ss, dd)
    assert normwise(g2, r2) <= RHS_TOL
    nl, fn = tab.n_sites, flow.fn
    rng_ = np.random.default_rng(1234)
    starts = sorted(rng_.choice(fn - 16, size=6, replace=False).tolist()) + [0, fn - 16]
    # normwise: the error on the sampled triples relative to the largest flow entry
    scale_s, scale_d = float(np.abs(gss).max()), float(np.abs(gdd).max())
    for s in starts:
        rss, rdd = orc.vertex_range(c, v2, r2, ss, dd, s, s + 16)
        a, b = s * nl, (s + 16) * nl
        assert float(np.abs(gss[a:b] - rss).max()) <= RHS_TOL * scale_s
        assert float(np.abs(gdd[a:b] - rdd).max()) <= RHS_TOL * scale_d


def test_rhs_largest_mesh_sampled(square_r3):
    """The largest supported mesh (N = 256: 8 421 376 triples, up to 2N + 8 = 520 nodes per
    channel) at a late cutoff: the whole self-energy flow and sampled vertex triples (the first,
    the last and random ones) against the oracle."""
    tab = square_r3
    n = 256
    freq = spn.frequency_exponential(0.005, 50.0, n)
    cut = np.array([0.2, 0.1, 0.05, 0.02], np.float32)
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(float(cut[0]), *tab.initial_state(n))
    for k in range(2):
        flow.compute_step()
        flow.finalize_step(float(cut[k + 1]))
    assert not flow.is_diverged()
    c, v2, ss, dd = flow.get_state()
    flow.compute_step()
    g2, gss, gdd = flow.get_flow()
    assert int(flow.node_counts().max()) > 2 * 64, "late cutoff: long node lists"
    orc = Oracle(tab, freq)
    r2 = orc.self_energy(c, v2, ss, dd)
    assert normwise(g2, r2) <= RHS_TOL
    nl, fn = tab.n_sites, flow.fn
    assert fn == n * n * (n + 1) // 2
    rng_ = np.random.default_rng(4321)
    starts = sorted(rng_.choice(fn - 8, size=6, replace=False).tolist()) + [0, fn - 8]
    scale_s, scale_d = float(np.abs(gss).max()), float(np.abs(gdd).max())
    for s in starts:
        rss, rdd = orc.vertex_range(c, v2, r2, ss, dd, s, s + 8)
        a, b = s * nl, (s + 8) * nl
        assert float(np.abs(gss[a:b] - rss).max()) <= RHS_TOL * scale_s
        assert float(np.abs(gdd[a:b] - rdd).max()) <= RHS_TOL * scale_d
    flow.close()


def test_euler_update_bit_exact(square_r3):
    tab = square_r3
    freq = spn.frequency_exponential(0.05, 50.0, 10)
    orc = Oracle(tab, freq)
    v2, ss, dd = tab.initial_state(10)
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(5.0, v2, ss, dd)
    flow.compute_step()
    d2, dss, ddd = flow.get_flow()
    flow.finalize_step(4.9)
    c, n2, nss, ndd = flow.get_state()
    step = np.float32(np.float32(4.9) - np.float32(5.0))
    assert c == np.float32(4.9)
    assert np.array_equal(n2, (v2 + step * d2).astype(np.float32))
    assert np.array_equal(nss, (ss + step * dss).astype(np.float32))
    assert np.array_equal(ndd, (dd + step * ddd).astype(np.float32))


def test_correlation_matches_oracle(square_r3):
    tab = square_r3
    freq = spn.frequency_exponential(0.005, 50.0, 16)
    orc = Oracle(tab, freq)
    cut = spn.cutoff_exponential(50.0, 0.05, 0.9)
    c, v2, ss, dd = oracle_state(orc, cut, *tab.initial_state(16), steps=4)
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(float(c), v2, ss, dd)
    zz, ddc, cz, cd = flow.measure_correlation()
    rs, rd = orc.correlation(c, v2, ss, dd)
    assert normwise(cz, rs) <= RHS_TOL
    assert normwise(cd, rd) <= RHS_TOL
    assert np.array_equal(zz, cz[tab.corr_rid])


def test_hyperkagome_flow_matches_golden_reference():
    """test_reference1.sh: hyperkagome r3, SU2 core, 34 cutoffs, against test_reference1.ref."""
    tab = spn.LatticeTables.from_npz(os.path.join(GOLDEN, "hyperkagome_r3_tables.npz"))
    g = np.load(os.path.join(GOLDEN, "reference1_su2.npz"))
    freq = g["frequencies"]
    cmax, cmin, step = (float(x) for x in g["cutoff_spec"])
    cut = spn.cutoff_exponential(cmax, cmin, step)
    assert np.array_equal(cut, g["cutoffs"])
    flow = spn.Su2Flow(tab, freq)
    measured, zz, dd, _, _, div = run_flow(flow, cut, tab.initial_state(len(freq)))
    assert not div and np.array_equal(measured, g["cutoffs"])
    nb, nr = g["zz"].shape[1:]
    assert float(np.abs(zz.reshape(-1, nb, nr) - g["zz"]).max()) < 1e-5
    assert float(np.abs(dd.reshape(-1, nb, nr) - g["dd"]).max()) < 1e-5


def test_hyperkagome_antiferro_sign_control_fails_golden():
    """test_referenceFail.sh: the same task with J = -1 must NOT reproduce the golden data."""
    tab = spn.LatticeTables.from_npz(os.path.join(GOLDEN, "hyperkagome_r3_tables.npz"))
    tab.interaction_J = -tab.interaction_J
    g = np.load(os.path.join(GOLDEN, "reference1_su2.npz"))
    cut = g["cutoffs"]
    flow = spn.Su2Flow(tab, g["frequencies"])
    _, zz, _, _, _, _ = run_flow(flow, cut, tab.initial_state(len(g["frequencies"])))
    nb, nr = g["zz"].shape[1:]
    n = min(len(zz), len(cut))
    assert float(np.abs(zz[:n].reshape(-1, nb, nr) - g["zz"][:n]).max()) > 1e-5


def test_honeycomb_flow_matches_python_obs_expectations():
    """test_pythonObs.sh: honeycomb r3 SU2 correlations queried as test_python_obs.py does."""
    spec = json.load(open(os.path.join(GOLDEN, "python_obs_honeycomb.json")))
    t = spec["task"]
    tab = spn.Lattice(t["lattice"], t["range"], t["model"], {"j": str(t["j"])}).tables()
    freq = np.array(t["frequencies"], np.float32)
    cut = spn.cutoff_exponential(t["cutoff_max"], t["cutoff_min"], t["cutoff_step"])
    flow = spn.Su2Flow(tab, freq)
    measured, zz, _, _, _, _ = run_flow(flow, cut, tab.initial_state(len(freq)))
    zz = zz.reshape(len(measured), tab.n_basis, tab.n_range)
    from obs_queries import evaluate_query

    for q in spec["queries"]:
        got = evaluate_query(q, measured, zz, tab)
        atol = 1e-16
        if q["what"] == "structure_factor":
            # a sum over sites with strong cancellation at k = 0: the error budget of a sum is
            # rtol times the sum of the magnitudes of its terms, not times its (small) result
            atol = 1e-5 * float(np.max(evaluate_query(q, measured, np.abs(zz), tab)))
        assert np.isclose(got, np.array(q["expect"]), rtol=1e-5, atol=atol).all(), q["what"]


def test_repeated_step_is_bit_identical(square_r3):
    """Run-to-run determinism of the vertex kernel (no atomics in the accumulation)."""
    tab = square_r3
    freq = spn.frequency_exponential(0.005, 50.0, 24)
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(3.0, *tab.initial_state(24))
    flow.compute_step()
    a = flow.get_flow()
    flow.compute_step()
    b = flow.get_flow()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_nan_state_reports_divergence(square_r3):
    """isDiverged: a NaN injected on the host into the state propagates into the flow.
    (The local site column is read by every channel; a single entry may never be read.)"""
    tab = square_r3
    freq = spn.frequency_exponential(0.05, 50.0, 8)
    v2, ss, dd = tab.initial_state(8)
    ss = ss.copy()
    ss[::tab.n_sites] = np.nan
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(2.0, v2, ss, dd)
    flow.compute_step()
    assert flow.is_diverged()
    flow.set_state(2.0, *tab.initial_state(8))
    flow.compute_step()
    assert not flow.is_diverged()
