"""Precision of whole flows against the FP64 oracle (every operation in double precision).

The bar is a relative error <= 1e-4 on the final correlations (normwise over the
correlation array).  Both GPU modes are checked: plain FP32 (the reference's types, Kahan
sums, FP64 node coefficients) and FP64 self-energy (Sigma and its flow kept in FP64 on the
device).  The FP32 oracle -- the reference's own arithmetic -- is measured the same way for
context; the GPU must not be worse than it by more than the bar.
"""
import numpy as np
import pytest

import spinparser_gb300 as spn
from spinparser_gb300.driver import run_flow
from oracle import Oracle

pytestmark = pytest.mark.gpu


def rel(a, ref):
    """Normwise relative error; where the reference is identically zero (the first cutoff
    equals the largest frequency, so no integration range exists) the result must be zero."""
    scale = float(np.max(np.abs(ref)))
    err = float(np.max(np.abs(np.asarray(a, np.float64) - ref)))
    return err / scale if scale > 0 else err


@pytest.mark.parametrize("lattice,rng,model,params,n", [
    ("square", 3, "square-j1j2heisenberg", {"j1": "1.0", "j2": "0.5"}, 24),
    ("cubic", 3, "cubic-j1j2heisenberg", {"j1": "1.0", "j2": "0.25"}, 16),
])
def test_final_correlations_against_fp64_oracle(lattice, rng, model, params, n):
    tab = spn.Lattice(lattice, rng, model, params).tables()
    freq = spn.frequency_exponential(0.005, 50.0, n)
    cut = spn.cutoff_exponential(50.0, 0.05, 0.95)
    state = tab.initial_state(n)
    orc = Oracle(tab, freq)
    n64, c64, _, _ = orc.flow(cut, *state, fp64=True)
    n32, c32, _, _ = orc.flow(cut, *state)
    assert n64 == n32 == len(cut)
    ref = c64[-1]
    errors = {"oracle_fp32": rel(c32[-1], ref)}
    for name, flags in (("gpu_fp32", 0), ("gpu_fp64_self_energy", spn.FP64_SELF_ENERGY)):
        flow = spn.Su2Flow(tab, freq, flags=flags)
        measured, _, _, cz, _, div = run_flow(flow, cut, state)
        assert not div and len(measured) == len(cut)
        errors[name] = rel(cz[-1], ref)
        # error growth along the flow stays within the bar at every cutoff
        growth = [rel(cz[k], c64[k]) for k in range(0, len(cut), 10)]
        assert max(growth) <= 1e-4, (name, growth)
    print(f"\n{lattice} r{rng} N={n}: final-correlation relative error vs FP64 oracle: {errors}")
    assert errors["gpu_fp32"] <= 1e-4
    assert errors["gpu_fp64_self_energy"] <= 1e-4
