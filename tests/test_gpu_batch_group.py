"""Grouped batches: flows with the same frequency mesh, lattice tables and cutoff list that stand
at the same cutoff share the vertex flow's node supports (spn_batch_set_grouping).  Every flow's
measurements and final state must be bit-identical to the same flow run alone through spn_su2_*
(the single-flow kernel): groups of every grouped class (6, 12, 20 and 30 sites: 8, 16 and 32
lanes per flow), subgroups split in parts, a group whose first member diverges at its first
step, flows that join a running batch (not grouped with the flows already there) and a flow
with a different cutoff list (never grouped)."""
import numpy as np
import pytest

import spinparser_gb300 as spn
from spinparser_gb300.batch import Su2Batch
from spinparser_gb300.driver import run_flow

pytestmark = pytest.mark.gpu

FREQ = (0.05, 50.0)
CUT = (20.0, 1.0, 0.85)
# (range, flows, N): 6 sites x 18 flows (two subgroups of 9 of at most 16), 12 sites x 9 (5 + 4
# of at most 8), 20 sites x 5 (3 + 2 of at most 4), 30 sites x 4 (one subgroup)
GROUPS = [(3, 18, 10), (5, 9, 8), (7, 5, 8), (9, 4, 6)]

_tab = {}


def tables(rng, j2):
    key = (rng, j2)
    if key not in _tab:
        _tab[key] = spn.Lattice("square", rng, "square-j1j2heisenberg", {"j1": "1", "j2": f"{j2:.3f}"}).tables()
    return _tab[key]


def members():
    out = []
    for rng, k, n in GROUPS:
        for i in range(k):
            out.append((rng, round(0.05 + 0.9 * i / max(k - 1, 1), 3), n))
    return out


def poisoned(state, nl):
    v2, ss, dd = state
    ss = ss.copy()
    ss[::nl] = np.nan
    return v2, ss, dd


def alone(rng, j2, n, cut, poison=False):
    tab = tables(rng, j2)
    freq = spn.frequency_exponential(*FREQ, n)
    flow = spn.Su2Flow(tab, freq)
    flow.set_variant(1, False)
    state = tab.initial_state(n)
    if poison:
        state = poisoned(state, tab.n_sites)
    measured, zz, dd, cz, cd, div = run_flow(flow, cut, state)
    st = flow.get_state()
    flow.close()
    return {"cut": measured, "zz": zz, "dd": dd, "cz": cz, "cd": cd, "div": div, "state": st}


def add(b, rng, j2, n, cut, poison=False):
    tab = tables(rng, j2)
    freq = spn.frequency_exponential(*FREQ, n)
    state = tab.initial_state(n)
    if poison:
        state = poisoned(state, tab.n_sites)
    return b.add(tab, freq, cut, state)


def assert_same(b, fid, ref, what):
    r = b.result(fid)
    assert r.diverged == ref["div"], what
    assert np.array_equal(r.cutoffs, ref["cut"]), what
    for key, got in (("zz", r.zz), ("dd", r.dd), ("cz", r.chi_zz), ("cd", r.chi_dd)):
        assert np.array_equal(got, ref[key].reshape(got.shape), equal_nan=True), (what, key)
    if not ref["div"]:
        c, v2, ss, dd = b.state(fid)
        rc, rv2, rss, rdd = ref["state"]
        assert c == rc and np.array_equal(v2, rv2) and np.array_equal(ss, rss) and np.array_equal(dd, rdd), what


@pytest.mark.parametrize("cap_divisor,use_graph", [(1, True), (2, False)])
def test_grouped_flows_equal_flows_alone(cap_divisor, use_graph):
    cut = spn.cutoff_exponential(*CUT)
    b = Su2Batch(nodes_per_iteration=1, use_graph=use_graph)
    b.set_grouping(2, cap_divisor)
    specs = members()
    ids = [add(b, *sp, cut) for sp in specs]
    assert b.grouped_flows() == len(specs)
    b.run()
    for sp, fid in zip(specs, ids):
        assert_same(b, fid, alone(*sp, cut), sp)
    b.close()


def test_group_with_diverging_first_member():
    cut = spn.cutoff_exponential(*CUT)
    b = Su2Batch()
    b.set_grouping(2)
    specs = [(5, j2, 8) for j2 in (0.1, 0.3, 0.5, 0.7, 0.9)]
    ids = [add(b, *sp, cut, poison=(i == 0)) for i, sp in enumerate(specs)]
    assert b.grouped_flows() == 5
    b.run()
    for i, (sp, fid) in enumerate(zip(specs, ids)):
        ref = alone(*sp, cut, poison=(i == 0))
        assert ref["div"] == (i == 0)
        assert_same(b, fid, ref, (i, sp))
    b.close()


def test_late_joiners_and_other_cutoff_lists_are_not_grouped_with_running_flows():
    cut = spn.cutoff_exponential(*CUT)
    other = spn.cutoff_exponential(20.0, 1.0, 0.8)
    b = Su2Batch()
    b.set_grouping(2)
    first = [(3, j2, 10) for j2 in (0.2, 0.4, 0.6)]
    ids = [add(b, *sp, cut) for sp in first]
    fid_other = add(b, 3, 0.5, 10, other)
    assert b.grouped_flows() == 3
    b.step()
    b.step()
    late = [(3, j2, 10) for j2 in (0.3, 0.7)]
    late_ids = [add(b, *sp, cut) for sp in late]
    assert b.grouped_flows() == 5  # the running three, and the two late joiners among themselves
    b.run()
    for sp, fid in zip(first + late, ids + late_ids):
        assert_same(b, fid, alone(*sp, cut), sp)
    assert_same(b, fid_other, alone(3, 0.5, 10, other), "other cutoffs")
    b.close()


def test_autotuned_batch_keeps_results():
    cut = spn.cutoff_exponential(*CUT)
    b = Su2Batch()
    b.set_grouping(2)  # sharing enabled: the autotuner weighs it against the per-flow kernel
    specs = [(3, j2, 10) for j2 in (0.1, 0.3, 0.5, 0.7)] + [(7, j2, 8) for j2 in (0.2, 0.8)] + [(11, 0.4, 6)]
    ids = [add(b, *sp, cut) for sp in specs]
    b.step()  # the autotuner runs between steps, on states a step has produced
    choice = b.autotune(2)
    assert choice["nodes_per_iteration"] in (1, 2) and choice["min_group"] in (0, 2)
    assert choice["cap_divisor"] in (1, 2) and choice["vertex_ms"] > 0
    b.run()
    for sp, fid in zip(specs, ids):
        assert_same(b, fid, alone(*sp, cut), sp)
    b.close()
