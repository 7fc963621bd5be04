"""Batched flows (spn_batch_*): every flow's measurements and final state are bit-identical to
the same flow run alone through spn_su2_* with the same vertex-flow variant, whatever else is
in the batch, when it joined, whether the step is replayed as a CUDA graph, and whether a
neighbour diverges.  Flows of all three site classes (<= 32, <= 64, <= 128 sites) are mixed.
"""
import numpy as np
import pytest

import spinparser_gb300 as spn
from spinparser_gb300.batch import PHASE_DONE, Su2Batch
from spinparser_gb300.driver import run_flow

pytestmark = pytest.mark.gpu

# (lattice, range, model, params, N frequencies, (cutoff max, min, step), flags)
CASES = {
    "square-r3": ("square", 3, "square-j1j2heisenberg", {"j1": "1", "j2": "0.4"}, 12, (50.0, 0.5, 0.9), 0),
    "honeycomb-r3": ("honeycomb", 3, "honeycomb-heisenberg", {"j": "1"}, 10, (20.0, 0.5, 0.85), 0),
    "cubic-r3-fp64": ("cubic", 3, "cubic-heisenberg", {"j": "1"}, 8, (30.0, 1.0, 0.8), spn.FP64_SELF_ENERGY),
    "square-r11": ("square", 11, "square-heisenberg", {"j": "1"}, 6, (10.0, 1.0, 0.8), 0),
    "pyrochlore-r2": ("pyrochlore", 2, "pyrochlore-heisenberg", {"j": "1"}, 8, (10.0, 0.5, 0.9), 0),
    "square-r17": ("square", 17, "square-heisenberg", {"j": "1"}, 4, (5.0, 1.0, 0.8), 0),
}

_tables = {}


def case(name):
    lat, rng, model, params, n, (cmax, cmin, step), flags = CASES[name]
    if name not in _tables:
        _tables[name] = spn.Lattice(lat, rng, model, params).tables()
    tab = _tables[name]
    freq = spn.frequency_exponential(0.05, 50.0, n)
    cut = spn.cutoff_exponential(cmax, cmin, step)
    return tab, freq, cut, flags


def alone(name, npi=1, poison=False):
    tab, freq, cut, flags = case(name)
    flow = spn.Su2Flow(tab, freq, flags=flags)
    flow.set_variant(npi, False)
    state = list(tab.initial_state(len(freq)))
    if poison:
        state[1] = state[1].copy()
        state[1][::tab.n_sites] = np.nan
    measured, zz, dd, cz, cd, div = run_flow(flow, cut, tuple(state))
    c, v2, ss, sd = flow.get_state()
    return {"cut": measured, "zz": zz, "dd": dd, "cz": cz, "cd": cd, "div": div, "state": (c, v2, ss, sd)}


def add(batch, name, poison=False):
    tab, freq, cut, flags = case(name)
    state = list(tab.initial_state(len(freq)))
    if poison:
        state[1] = state[1].copy()
        state[1][::tab.n_sites] = np.nan
    return batch.add(tab, freq, cut, tuple(state), flags=flags)


def assert_same(batch, fid, ref, name):
    r = batch.result(fid)
    assert r.diverged == ref["div"], name
    assert np.array_equal(r.cutoffs, ref["cut"]), name
    for key, got in (("zz", r.zz), ("dd", r.dd), ("cz", r.chi_zz), ("cd", r.chi_dd)):
        assert np.array_equal(got, ref[key].reshape(got.shape), equal_nan=True), (name, key)
    if not ref["div"]:
        c, v2, ss, sd = batch.state(fid)
        rc, rv2, rss, rsd = ref["state"]
        assert c == rc and np.array_equal(v2, rv2) and np.array_equal(ss, rss) and np.array_equal(sd, rsd), name


@pytest.fixture(scope="module")
def reference():
    return {name: alone(name) for name in CASES}


@pytest.mark.parametrize("use_graph", [True, False])
def test_mixed_batch_equals_flows_alone(reference, use_graph):
    b = Su2Batch(nodes_per_iteration=1, use_graph=use_graph)
    ids = {name: add(b, name) for name in CASES}
    steps = b.run()
    assert steps == max(len(case(n)[2]) for n in CASES)
    for name, fid in ids.items():
        assert b.poll(fid)[0] == PHASE_DONE
        assert_same(b, fid, reference[name], name)
    st = b.stats()
    assert st["flows"] == len(CASES)
    if use_graph:
        # a graph is built only when the set of flows or a phase changes
        assert st["graph_builds"] < st["steps"]


def test_continuous_admission_and_removal(reference):
    b = Su2Batch()
    first = {name: add(b, name) for name in ("square-r3", "honeycomb-r3")}
    for _ in range(5):
        b.step()
    later = {name: add(b, name) for name in ("cubic-r3-fp64", "square-r11")}
    b.run()
    for name, fid in {**first, **later}.items():
        assert_same(b, fid, reference[name], name)
    # finished flows leave, their slots are reused by new arrivals
    b.remove(first["square-r3"])
    again = add(b, "pyrochlore-r2")
    assert again == first["square-r3"]
    b.run()
    assert_same(b, again, reference["pyrochlore-r2"], "pyrochlore-r2")


def test_diverging_flow_does_not_disturb_its_neighbours(reference):
    poisoned = alone("honeycomb-r3", poison=True)
    assert poisoned["div"] and len(poisoned["cut"]) == 1
    b = Su2Batch()
    good = add(b, "square-r3")
    bad = add(b, "honeycomb-r3", poison=True)
    b.run()
    assert_same(b, bad, poisoned, "poisoned")
    assert_same(b, good, reference["square-r3"], "square-r3")


def test_other_variant_gives_the_same_bits(reference):
    """A batch with the other kernel variant (2 nodes per iteration) against the flows run
    alone with the default variant."""
    names = ("square-r3", "square-r11", "pyrochlore-r2", "cubic-r3-fp64")
    b = Su2Batch(nodes_per_iteration=2)
    ids = {n: add(b, n) for n in names}
    b.run()
    for n, fid in ids.items():
        assert_same(b, fid, reference[n], n)


def test_server_admits_by_footprint_and_results_do_not_change(reference):
    """Continuous batching under a memory budget (the largest flow plus a little) and under a
    two-flow slot limit (arrival order and least work first): requests wait, are admitted as
    others finish, and every result equals the flow alone."""
    from spinparser_gb300.serve import FlowServer, FlowSpec

    def spec(name):
        lat, rng, model, params, n, (cmax, cmin, step), flags = CASES[name]
        return FlowSpec(lat, rng, model, tuple(params.items()), n, 0.05, 50.0, cmax, cmin, step, flags)

    names = list(CASES)
    feet = sorted(Su2Batch.footprint(*case(n)[:2], len(case(n)[2])) for n in names)
    for budget, slots, policy in ((feet[-1] + feet[0] // 2, None, "fifo"), (10 * feet[-1], 2, "fifo"),
                                  (10 * feet[-1], 2, "sjf")):
        srv = FlowServer(memory_budget=budget, max_flows=slots, policy=policy)
        tickets = {n: srv.submit(spec(n)) for n in names}
        most = 0
        while srv.pump():
            most = max(most, len(srv.active))
            assert srv.used <= srv.budget
            assert slots is None or len(srv.active) <= slots
        assert 1 <= most < len(names)  # requests had to wait for memory / slots
        for n, t in tickets.items():
            assert t.t_admit is not None and t.t_done is not None and t.time_to_result > 0
            r = t.result
            ref = reference[n]
            assert r.diverged == ref["div"] and np.array_equal(r.cutoffs, ref["cut"])
            assert np.array_equal(r.zz, ref["zz"].reshape(r.zz.shape)) and np.array_equal(r.dd, ref["dd"].reshape(r.dd.shape))
        srv.close()
