"""The CPU baseline is timed on the oracle's sources built with the reference's own flags
(-O3, the compiler's default floating-point contraction); the checker is the -O2
-ffp-contract=off build.  The two must compute the same flow: one RHS agrees within the
parity tolerance (1e-5 normwise), on CPU only."""
import numpy as np

import spinparser_gb300 as spn
from oracle import Oracle


def normwise(g, r):
    return float(np.max(np.abs(np.asarray(g, np.float64) - r)) / max(float(np.max(np.abs(r))), 1e-300))


def test_timing_build_computes_the_checker_flow():
    tab = spn.Lattice("cubic", 3, "cubic-j1j2heisenberg", {"j1": "1.0", "j2": "0.25"}).tables()
    freq = spn.frequency_exponential(0.01, 30.0, 12)
    chk, tim = Oracle(tab, freq), Oracle(tab, freq, timing=True)
    v2, ss, dd = tab.initial_state(12)
    c = np.float32(2.0)
    for nxt in (np.float32(1.5), np.float32(1.0)):  # a non-trivial state: two checker steps
        d2, dss, ddd = chk.rhs(c, v2, ss, dd)
        chk.euler(c, nxt, v2, d2)
        chk.euler(c, nxt, ss, dss)
        chk.euler(c, nxt, dd, ddd)
        c = nxt
    a = chk.rhs(c, v2, ss, dd)
    b = tim.rhs(c, v2, ss, dd)
    for x, y in zip(b, a):
        assert normwise(x, y) <= 1e-5
    ca, cb = chk.correlation(c, v2, ss, dd), tim.correlation(c, v2, ss, dd)
    for x, y in zip(cb, ca):
        assert normwise(x, y) <= 1e-5
