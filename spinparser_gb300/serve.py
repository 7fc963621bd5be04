"""Serving SU(2) flows: continuous batching over one GPU (``Su2Batch``).

Requests (``FlowSpec``: lattice, range, model, couplings, frequency grid, cutoff list) are
queued as they arrive.  Between batch steps the server admits queued requests -- in arrival
order ("fifo") or smallest expected work first ("sjf": the flow's nominal work per step times
its number of steps) -- while their device footprint fits the memory budget (and, optionally,
a flow-count limit).  Under "srpt" every request that fits is admitted in arrival order, and
before each step only the k resident flows with the least remaining work run (the others are
paused, keeping their state): shortest-remaining-work-first with preemption between steps;
every admitted flow keeps its vertex and self-energy state resident on the device until it
finishes, and all resident flows advance together, one cutoff step per batch step.  Finished
flows are retired at once (results copied out, memory released) so that waiting requests take
their place.  Each ticket records its arrival, admission and completion time; the time to
result is completion minus arrival.

A flow's results do not depend on the company it keeps in the batch (the batch engine
evaluates every flow with the single-flow device code), so serving changes when a result
arrives, never what it is.
"""
from __future__ import annotations

import ctypes as C
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from ._capi import check, load_library
from .batch import FLOW_DIVERGED, PHASE_DONE, BatchResult, Su2Batch
from .core import Lattice, cutoff_exponential, frequency_exponential


@dataclass(frozen=True)
class FlowSpec:
    """One flow as a task file describes it (exponential frequency and cutoff grids)."""
    lattice: str
    range: int
    model: str
    params: tuple          # ((name, value), ...) coupling parameters
    n_freq: int
    fmin: float
    fmax: float
    cmax: float
    cmin: float
    cstep: float
    flags: int = 0

    def build(self):
        lat = Lattice(self.lattice, self.range, self.model, dict(self.params))
        tab = lat.tables()
        return tab, frequency_exponential(self.fmin, self.fmax, self.n_freq), cutoff_exponential(self.cmax, self.cmin, self.cstep)


@dataclass
class Ticket:
    id: int
    spec: FlowSpec
    t_arrival: float
    t_admit: float | None = None
    t_done: float | None = None
    flow_id: int | None = None
    footprint: int = 0
    work: float = 0.0  # expected work of the whole flow (nominal flops), for "sjf" admission
    result: BatchResult | None = None
    _built: tuple | None = field(default=None, repr=False)

    @property
    def time_to_result(self) -> float | None:
        return None if self.t_done is None else self.t_done - self.t_arrival


def device_memory(device: int = 0):
    """(free, total) device bytes."""
    lib = load_library()
    f, t = C.c_longlong(), C.c_longlong()
    check(lib.spn_device_memory(device, C.byref(f), C.byref(t)))
    return f.value, t.value


def expected_work(tab, freq, cut) -> float:
    """Nominal work of a flow: F_N (2N+8)(3*100*Nl + 4*sum O) flops per step times its steps."""
    n = len(freq)
    fn = n * n * (n + 1) // 2
    return float(fn) * (2 * n + 8) * (300.0 * tab.n_sites + 4.0 * tab.n_overlap) * max(len(cut) - 1, 1)


def prepare(t: Ticket) -> None:
    """Build a queued request's tables once; fills its device footprint and expected work."""
    if t._built is None:
        t._built = t.spec.build()
        tab, freq, cut = t._built
        t.footprint = Su2Batch.footprint(tab, freq, len(cut))
        t.work = expected_work(tab, freq, cut)


def next_ticket(queue, policy: str, now: float | None = None, max_wait: float | None = None) -> Ticket:
    """The request a server admits next: the oldest ("fifo") or the one with the least expected
    work, ties to the oldest ("sjf").  Under "sjf" a large request could wait for ever while
    smaller ones keep arriving; with `max_wait` set, the oldest request goes first once it has
    waited longer than that (seconds since its arrival at `now`)."""
    if policy == "sjf":
        oldest = min(queue, key=lambda q: (q.t_arrival, q.id))
        if max_wait is not None and now is not None and now - oldest.t_arrival > max_wait:
            prepare(oldest)
            return oldest
        for q in queue:
            prepare(q)
        return min(queue, key=lambda q: (q.work, q.id))
    prepare(queue[0])
    return queue[0]


class FlowServer:
    def __init__(self, device: int = 0, memory_budget: int | None = None, max_flows: int | None = None,
                 nodes_per_iteration: int = 1, use_graph: bool = True, clock=time.perf_counter, policy: str = "fifo",
                 max_wait: float | None = None, autotune: bool = False, autotune_interval: int = 50,
                 keep_oldest: bool = False):
        if policy not in ("fifo", "sjf", "srpt"):
            raise ValueError("policy must be 'fifo', 'sjf' or 'srpt'")
        self.policy = policy
        self.max_wait = max_wait
        # srpt: flows that run at each step (the rest are paused); max_flows keeps its meaning
        # of a residency limit for the other policies
        self.running = max(1, int(max_flows)) if (policy == "srpt" and max_flows) else 1
        if policy == "srpt":
            max_flows = None
        self._paused: set[int] = set()
        # srpt: the oldest resident request runs at every step as well, so that the request the
        # policy would defer longest keeps making progress (bounds the tail of time to result)
        self.keep_oldest = keep_oldest
        # batch autotuner: run once a set of running flows has stepped together for
        # autotune_interval steps (the first steps of a flow, at large cutoffs, have few
        # loop-frequency nodes and do not show which configuration wins later)
        self.autotune = autotune
        self.autotune_interval = autotune_interval
        self._tuned_set: frozenset | None = None
        self._seen_set: frozenset | None = None
        self._set_since = 0
        self.tunings: list[dict] = []
        self.batch = Su2Batch(device, nodes_per_iteration, use_graph)
        if memory_budget is None:
            free, _ = device_memory(device)
            memory_budget = int(0.8 * free)
        self.budget = memory_budget
        self.max_flows = max_flows
        self.clock = clock
        self.queue: deque[Ticket] = deque()
        self.active: dict[int, Ticket] = {}   # flow id -> ticket
        self.finished: list[Ticket] = []
        self.used = 0
        self._next = 0
        self.steps = 0

    def submit(self, spec: FlowSpec, t_arrival: float | None = None) -> Ticket:
        t = Ticket(self._next, spec, self.clock() if t_arrival is None else t_arrival)
        self._next += 1
        self.queue.append(t)
        return t

    def _admit(self) -> None:
        while self.queue:
            if self.max_flows is not None and len(self.active) >= self.max_flows:
                return
            t = next_ticket(self.queue, "fifo" if self.policy == "srpt" else self.policy, self.clock(), self.max_wait)
            if self.active and self.used + t.footprint > self.budget:
                return
            tab, freq, cut = t._built
            # the request leaves the queue only once the batch holds it: if add() raises (out
            # of device memory, say), it stays queued and the error reaches the caller
            t.flow_id = self.batch.add(tab, freq, cut, flags=t.spec.flags)
            self.queue.remove(t)
            t.t_admit = self.clock()
            self.used += t.footprint
            self.active[t.flow_id] = t

    def _retire(self) -> None:
        for fid in list(self.active):
            phase, _, _ = self.batch.poll(fid)
            if phase != PHASE_DONE:
                continue
            t = self.active.pop(fid)
            self._paused.discard(fid)
            t.result = self.batch.result(fid)
            t.t_done = self.clock()
            self.batch.remove(fid)
            self.used -= t.footprint
            t._built = None
            self.finished.append(t)

    def _choose_running(self) -> None:
        """srpt: the `running` resident flows with the least remaining work take the next step
        (ties to the older request), and with keep_oldest also the oldest resident request;
        every other resident flow is paused."""
        rem = []
        for fid, t in self.active.items():
            _, step, _ = self.batch.poll(fid)
            n_cut = len(t._built[2])
            rem.append((t.work * max(n_cut - 1 - step, 0) / max(n_cut - 1, 1), t.id, fid))
        rem.sort()
        run = {fid for _, _, fid in rem[:self.running]}
        if self.keep_oldest and self.active:
            run.add(min(self.active, key=lambda f: (self.active[f].t_arrival, self.active[f].id)))
        for fid in self.active:
            want = fid not in run
            if want != (fid in self._paused):
                self.batch.set_paused(fid, want)
                if want:
                    self._paused.add(fid)
                else:
                    self._paused.discard(fid)

    def pump(self) -> int:
        """Admits what fits, advances the resident flows by one step (under "srpt" only the
        ones with the least remaining work) and retires finished flows.  Returns the number of
        flows resident or queued."""
        self._admit()
        if self.active:
            if self.policy == "srpt":
                self._choose_running()
            if self.autotune:
                running = frozenset(f for f in self.active if f not in self._paused)
                if running != self._seen_set:
                    self._seen_set, self._set_since = running, self.steps
                if running != self._tuned_set and self.steps - self._set_since >= self.autotune_interval:
                    self.tunings.append({"step": self.steps, "flows": len(running), **self.batch.autotune(1)})
                    self._tuned_set = running
            self.batch.step()
            self.steps += 1
            self._retire()
        return len(self.active) + len(self.queue)

    def drain(self) -> None:
        """Runs until every submitted request has its result."""
        while self.pump():
            pass

    def close(self) -> None:
        self.batch.close()


def time_to_result_stats(tickets) -> dict:
    ttr = np.array([t.time_to_result for t in tickets if t.time_to_result is not None])
    if ttr.size == 0:
        return {"n": 0}
    return {"n": int(ttr.size), "p50_s": float(np.percentile(ttr, 50)), "p99_s": float(np.percentile(ttr, 99)),
            "mean_s": float(ttr.mean()), "max_s": float(ttr.max())}


def diverged(t: Ticket) -> bool:
    return t.result is not None and t.result.diverged
