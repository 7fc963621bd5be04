"""Batched SU(2) flows through the C ABI (spn_batch_*): many flows on one GPU advanced
together, one launch per kernel per step for all of them, with flows joining and leaving
between steps (continuous batching).

Each flow follows the reference's per-flow cycle (SpinParser::runCore, src/SpinParser.cpp:126-187):
flow and measurement at every cutoff, divergence check, Euler step, final measurement at the
last cutoff.  ``Su2Batch.result`` returns the same arrays as ``driver.run_flow`` on a single
``Su2Flow``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._capi import check, load_library
from .core import LatticeTables, _ptr, make_desc

PHASE_FLOWING, PHASE_FINAL, PHASE_DONE = 0, 1, 2
FLOW_DIVERGED, FLOW_NODE_OVERFLOW = 0x1, 0x2


@dataclass
class BatchResult:
    cutoffs: np.ndarray   # [n] cutoffs measured
    zz: np.ndarray        # [n, n_corr]
    dd: np.ndarray        # [n, n_corr]
    chi_zz: np.ndarray    # [n, Nl]
    chi_dd: np.ndarray    # [n, Nl]
    diverged: bool


class Su2Batch:
    def __init__(self, device: int = 0, nodes_per_iteration: int = 1, use_graph: bool = True):
        lib = load_library()
        self._lib = lib
        self.device = device
        h = C.c_void_p()
        check(lib.spn_batch_create(device, C.byref(h)))
        self._h = h
        check(lib.spn_batch_set_variant(h, nodes_per_iteration, int(use_graph)))
        self._flows = {}

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.spn_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_variant(self, nodes_per_iteration: int = 1, use_graph: bool = True) -> None:
        """Kernel variant and graph replay; results do not change."""
        check(self._lib.spn_batch_set_variant(self._h, nodes_per_iteration, int(use_graph)))

    def set_grouping(self, min_group: int = 2, cap_divisor: int = 1) -> None:
        """Cross-flow sharing of node supports in the vertex flow: groups of at least
        `min_group` flows with the same mesh, lattice tables and cutoff list at the same cutoff
        (0 = off), in subgroups of at most the kernel's flows per block / cap_divisor.  Results
        do not change."""
        check(self._lib.spn_batch_set_grouping(self._h, int(min_group), int(cap_divisor)))

    def autotune(self, reps: int = 2) -> dict:
        """Times the vertex flow of the current flows under each candidate configuration
        (nodes per iteration x cross-flow sharing) and keeps the fastest; no state changes."""
        a, m, c, t = C.c_int(), C.c_int(), C.c_int(), C.c_float()
        check(self._lib.spn_batch_autotune(self._h, int(reps), C.byref(a), C.byref(m), C.byref(c), C.byref(t)))
        return {"nodes_per_iteration": a.value, "min_group": m.value, "cap_divisor": c.value, "vertex_ms": t.value}

    def set_paused(self, flow_id: int, paused: bool) -> None:
        """Holds a flow out of the following steps (its state and results stay as they are)."""
        check(self._lib.spn_batch_set_paused(self._h, flow_id, int(bool(paused))))

    def grouped_flows(self) -> int:
        """Flows the current plan evaluates with the grouped kernel."""
        n = C.c_int()
        check(self._lib.spn_batch_grouped_flows(self._h, C.byref(n)))
        return n.value

    @staticmethod
    def footprint(tables: LatticeTables, freq, n_cutoffs: int) -> int:
        """Device bytes a flow occupies in a batch (the admission measure)."""
        lib = load_library()
        d, keep = make_desc(tables, freq)
        out = C.c_longlong()
        check(lib.spn_batch_footprint(C.byref(d), int(n_cutoffs), C.byref(out)))
        return out.value

    def add(self, tables: LatticeTables, freq, cutoffs, state=None, spin_length: float = 0.5, flags: int = 0,
            normalization: float | None = None) -> int:
        """Admits a flow; `state` = (v2, v4ss, v4dd) at cutoffs[0], default the model's
        initial condition.  Returns the flow id."""
        freq = np.ascontiguousarray(freq, np.float32)
        cut = np.ascontiguousarray(cutoffs, np.float32)
        if state is None:
            state = tables.initial_state(len(freq), normalization if normalization is not None else 2.0 * spin_length)
        v2, ss, dd = (np.ascontiguousarray(x, np.float32) for x in state)
        d, keep = make_desc(tables, freq, spin_length, self.device, flags)
        fid = C.c_int()
        check(self._lib.spn_batch_add(self._h, C.byref(d), len(cut), _ptr(cut, C.c_float), _ptr(v2, C.c_float),
                                      _ptr(ss, C.c_float), _ptr(dd, C.c_float), C.byref(fid)))
        n = len(freq)
        self._flows[fid.value] = (len(cut), d.n_corr, tables.n_sites, n, n * n * (n + 1) // 2)
        return fid.value

    def step(self) -> int:
        """Advances every unfinished flow by one step; returns the flows still active."""
        n = C.c_int()
        check(self._lib.spn_batch_step(self._h, C.byref(n)))
        return n.value

    def run(self, max_steps: int | None = None) -> int:
        """Steps until every flow is done (or max_steps); returns the steps taken."""
        k = 0
        while max_steps is None or k < max_steps:
            k += 1
            if self.step() == 0:
                break
        self.synchronize()
        return k

    def synchronize(self) -> None:
        check(self._lib.spn_batch_synchronize(self._h))

    def poll(self, flow_id: int):
        """(phase, cutoff index, flags) as the host last saw them."""
        p, s, f = C.c_int(), C.c_int(), C.c_int()
        check(self._lib.spn_batch_poll(self._h, flow_id, C.byref(p), C.byref(s), C.byref(f)))
        return p.value, s.value, f.value

    def result(self, flow_id: int) -> BatchResult:
        n_cut, n_corr, nl, _, _ = self._flows[flow_id]
        cut = np.empty(n_cut, np.float32)
        zz = np.empty((n_cut, n_corr), np.float32)
        dd = np.empty((n_cut, n_corr), np.float32)
        cz = np.empty((n_cut, nl), np.float32)
        cd = np.empty((n_cut, nl), np.float32)
        m = C.c_int()
        fp = C.POINTER(C.c_float)
        check(self._lib.spn_batch_get_result(self._h, flow_id, C.byref(m), cut.ctypes.data_as(fp), zz.ctypes.data_as(fp),
                                             dd.ctypes.data_as(fp), cz.ctypes.data_as(fp), cd.ctypes.data_as(fp)))
        k = m.value
        _, _, flags = self.poll(flow_id)
        return BatchResult(cut[:k], zz[:k], dd[:k], cz[:k], cd[:k], bool(flags & FLOW_DIVERGED))

    def state(self, flow_id: int):
        """(cutoff, v2, v4ss, v4dd) of a flow now."""
        _, _, nl, n, fn = self._flows[flow_id]
        v2 = np.empty(n, np.float32)
        ss = np.empty(fn * nl, np.float32)
        dd = np.empty(fn * nl, np.float32)
        c = C.c_float()
        fp = C.POINTER(C.c_float)
        check(self._lib.spn_batch_get_state(self._h, flow_id, C.byref(c), v2.ctypes.data_as(fp), ss.ctypes.data_as(fp),
                                            dd.ctypes.data_as(fp)))
        return float(c.value), v2, ss, dd

    def remove(self, flow_id: int) -> None:
        check(self._lib.spn_batch_remove(self._h, flow_id))
        self._flows.pop(flow_id, None)

    def stats(self) -> dict:
        s, g, n = C.c_longlong(), C.c_longlong(), C.c_int()
        check(self._lib.spn_batch_stats(self._h, C.byref(s), C.byref(g), C.byref(n)))
        return {"steps": s.value, "graph_builds": g.value, "flows": n.value}
