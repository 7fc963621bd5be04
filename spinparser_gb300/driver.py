"""Cutoff loop over a GPU-resident flow, as SpinParser::runCore drives an FrgCore
(src/SpinParser.cpp:126-187): at every cutoff the flow and the correlation measurement are
computed from the same state, the flow is checked for NaN, then the explicit Euler step
moves the state to the next cutoff; a final measurement is taken at the last cutoff.
"""
from __future__ import annotations

import numpy as np

from .core import Su2Flow


def run_flow(flow: Su2Flow, cutoffs, state=None, measure: bool = True):
    """Runs the whole cutoff list.  Returns (measured_cutoffs, zz[n, n_corr], dd[n, n_corr],
    chi_zz[n, Nl], chi_dd[n, Nl], diverged)."""
    cut = np.asarray(cutoffs, np.float32)
    if state is not None:
        flow.set_state(float(cut[0]), *state)
    zz, dd, cz, cd, measured = [], [], [], [], []
    diverged = False
    k = 0
    for k in range(len(cut) - 1):
        flow.compute_step()
        if measure:
            z, d, a, b = flow.measure_correlation()
            zz.append(z), dd.append(d), cz.append(a), cd.append(b), measured.append(cut[k])
        if flow.is_diverged():
            diverged = True
            break
        flow.finalize_step(float(cut[k + 1]))
    if measure and not diverged:
        z, d, a, b = flow.measure_correlation()
        zz.append(z), dd.append(d), cz.append(a), cd.append(b), measured.append(cut[-1])
    if not measure:
        return np.array([], np.float32), None, None, None, None, diverged
    return (np.array(measured, np.float32), np.array(zz), np.array(dd), np.array(cz), np.array(cd), diverged)
