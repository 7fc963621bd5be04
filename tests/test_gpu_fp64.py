"""FP64 flows on the GPU (SPN_SU2_FP64) against the FP64 oracle.

An FP64 flow evaluates every operation of the right-hand side, the Euler step and the
measurement in double precision on the device.  It is the precision reference for FP32 flows
of the same task, so it has to agree with the CPU FP64 oracle to near double rounding:
normwise relative error <= 1e-11 for one right-hand side, and <= 1e-10 for correlations after
a short flow (the two evaluate the same sums with different association and node weights
that differ in the last bit).
"""
import numpy as np
import pytest

import spinparser_gb300 as spn
from spinparser_gb300._capi import SpnError
from oracle import Oracle

pytestmark = pytest.mark.gpu

RHS_TOL_F64 = 1e-11
FLOW_TOL_F64 = 1e-10


def normwise(g, r):
    return float(np.max(np.abs(np.asarray(g, np.float64) - r)) / max(float(np.max(np.abs(r))), 1e-300))


def f64_state(orc, cutoffs, v2, ss, dd, steps):
    """The initial state advanced by `steps` FP64 oracle Euler steps."""
    v2, ss, dd = (np.asarray(x, np.float64) for x in (v2, ss, dd))
    c = float(np.float32(cutoffs[0]))
    for k in range(steps):
        d2, dss, ddd = orc.rhs(np.float64(c), v2, ss, dd, fp64=True)
        nxt = float(np.float32(cutoffs[k + 1]))
        v2, ss, dd = v2 + (nxt - c) * d2, ss + (nxt - c) * dss, dd + (nxt - c) * ddd
        c = nxt
    return c, v2, ss, dd


@pytest.mark.parametrize("lattice,rng,model,params,n", [
    ("square", 3, "square-heisenberg", {"j": "1.0"}, 16),                     # 6 sites
    ("cubic", 6, "cubic-j1j2heisenberg", {"j1": "1.0", "j2": "0.25"}, 8),     # 23 sites
    ("square", 11, "square-heisenberg", {"j": "1.0"}, 6),                     # 42 sites
    ("square", 15, "square-heisenberg", {"j": "1.0"}, 6),                     # 72 sites
])
def test_fp64_rhs_matches_fp64_oracle(lattice, rng, model, params, n):
    tab = spn.Lattice(lattice, rng, model, params).tables()
    freq = spn.frequency_exponential(0.01, 30.0, n)
    cut = spn.cutoff_exponential(30.0, 0.05, 0.9)
    orc = Oracle(tab, freq)
    c, v2, ss, dd = f64_state(orc, cut, *tab.initial_state(n), steps=2)
    flow = spn.Su2Flow(tab, freq, flags=spn.FP64)
    flow.set_state_f64(c, v2, ss, dd)
    flow.compute_step()
    g2, gss, gdd = flow.get_flow_f64()
    r2, rss, rdd = orc.rhs(np.float64(c), v2, ss, dd, fp64=True)
    assert normwise(g2, r2) <= RHS_TOL_F64
    assert normwise(gss, rss) <= RHS_TOL_F64
    assert normwise(gdd, rdd) <= RHS_TOL_F64
    assert not flow.is_diverged()
    # the float view of the same flow is the double one rounded
    f2, fss, fdd = flow.get_flow()
    np.testing.assert_array_equal(fss, gss.astype(np.float32))
    np.testing.assert_array_equal(f2, g2.astype(np.float32))


def test_fp64_flow_matches_fp64_oracle_flow():
    """Twelve cutoff steps with a measurement at every cutoff, as the task driver runs them."""
    tab = spn.Lattice("square", 3, "square-heisenberg", {"j": "1.0"}).tables()
    n = 16
    freq = spn.frequency_exponential(0.01, 30.0, n)
    cut = spn.cutoff_exponential(30.0, 0.05, 0.9)[:13]
    orc = Oracle(tab, freq)
    v2, ss, dd = tab.initial_state(n)
    n_meas, ocs, ocd, (ov2, oss, odd) = orc.flow(cut, v2, ss, dd, fp64=True)
    assert n_meas == len(cut)
    flow = spn.Su2Flow(tab, freq, flags=spn.FP64)
    flow.set_state(float(cut[0]), v2, ss, dd)  # float state widened on the device side
    gcs = np.zeros_like(ocs)
    gcd = np.zeros_like(ocd)
    for k in range(len(cut)):
        _, _, gcs[k], gcd[k] = flow.measure_correlation_f64()
        if k + 1 < len(cut):
            flow.compute_step()
            flow.finalize_step(float(cut[k + 1]))
    assert normwise(gcs, ocs) <= FLOW_TOL_F64
    assert normwise(gcd, ocd) <= FLOW_TOL_F64
    c, g2, gss, gdd = flow.get_state_f64()
    assert c == float(np.float32(cut[-1]))
    assert normwise(gss, oss) <= FLOW_TOL_F64
    assert normwise(gdd, odd) <= FLOW_TOL_F64
    assert normwise(g2, ov2) <= FLOW_TOL_F64


def test_fp64_flow_api_limits():
    tab = spn.Lattice("square", 3, "square-heisenberg", {"j": "1.0"}).tables()
    freq = spn.frequency_exponential(0.01, 30.0, 8)
    f32 = spn.Su2Flow(tab, freq)
    with pytest.raises(SpnError):
        f32.get_state_f64()  # not an FP64 flow
    f64 = spn.Su2Flow(tab, freq, flags=spn.FP64)
    with pytest.raises(SpnError):
        f64.set_variant(2, False)  # one FP64 kernel
    assert f64.autotune()["nodes_per_iteration"] == 1
    b = spn.Su2Batch(0)
    try:
        with pytest.raises(SpnError):
            b.add(tab, freq, spn.cutoff_exponential(30.0, 0.05, 0.9), flags=spn.FP64)
    finally:
        b.close()
