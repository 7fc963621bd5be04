"""Seeded multi-flow workloads: the parameter scan and the serving stream.

Scan: 128 square-lattice J1-J2 flows, J1 = 1, J2/J1 uniform in [0, 1], lattice range uniform in
{3, 5, 7}, frequency count uniform in {32, 48, 64} on an exponential grid in [0.005, 50],
cutoff 50 -> 0.05 x 0.98.

Serving: requests drawn uniformly over the square, cubic and pyrochlore J1-J2 models, J1 = 1,
J2 uniform in [-0.5, 0.5], range uniform in 3..7, frequency count uniform in {32, 48, 64}
(grid [0.005, 50]), cutoff 50 -> 0.05 x 0.98, arriving as an open-loop Poisson stream.

Draws come from numpy's MT19937 generator with the fixed seed below, in a fixed order per
request, so a workload is the same on every machine.
"""
from __future__ import annotations

import numpy as np

from .serve import FlowSpec

SEED = 20261203

_MODELS = {"square": "square-j1j2heisenberg", "cubic": "cubic-j1j2heisenberg", "pyrochlore": "pyrochlore-j1j2heisenberg"}


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.MT19937(seed))


def _spec(lattice: str, rng_: int, j2: float, n: int) -> FlowSpec:
    return FlowSpec(lattice, int(rng_), _MODELS[lattice], (("j1", "1.0"), ("j2", f"{j2:.6f}")), int(n),
                    0.005, 50.0, 50.0, 0.05, 0.98)


def scan_specs(n: int = 128, seed: int = SEED) -> list[FlowSpec]:
    g = _rng(seed)
    out = []
    for _ in range(n):
        j2 = g.uniform(0.0, 1.0)
        r = g.choice([3, 5, 7])
        nf = g.choice([32, 48, 64])
        out.append(_spec("square", r, j2, nf))
    return out


def serve_specs(n: int, seed: int = SEED + 1) -> list[FlowSpec]:
    g = _rng(seed)
    lattices = ["square", "cubic", "pyrochlore"]
    out = []
    for _ in range(n):
        lat = lattices[int(g.integers(0, 3))]
        j2 = g.uniform(-0.5, 0.5)
        r = int(g.integers(3, 8))
        nf = [32, 48, 64][int(g.integers(0, 3))]
        out.append(_spec(lat, r, j2, nf))
    return out


def poisson_arrivals(n: int, rate: float, seed: int = SEED + 2) -> np.ndarray:
    """Arrival offsets (seconds) of n requests at `rate` per second; all at 0 for rate = inf."""
    if not np.isfinite(rate):
        return np.zeros(n)
    g = _rng(seed)
    return np.cumsum(g.exponential(1.0 / rate, size=n))
