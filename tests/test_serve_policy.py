"""Admission order of the flow server (host logic, no GPU): arrival order for "fifo", least
expected work first for "sjf", ties to the oldest request."""
import pytest

from spinparser_gb300.serve import FlowSpec, Ticket, expected_work, next_ticket


def spec(rng, n):
    return FlowSpec("square", rng, "square-j1j2heisenberg", (("j1", "1.0"), ("j2", "0.3")), n, 0.005, 50.0,
                    50.0, 0.5, 0.9)


def queue(*specs):
    return [Ticket(i, s, float(i)) for i, s in enumerate(specs)]


def test_fifo_takes_the_oldest():
    q = queue(spec(5, 16), spec(3, 8))
    assert next_ticket(q, "fifo") is q[0]
    assert q[0].footprint > 0 and q[0].work > 0
    assert q[1]._built is None  # fifo builds only the head


def test_sjf_takes_the_least_work_and_ties_to_the_oldest():
    q = queue(spec(5, 16), spec(3, 16), spec(3, 8), spec(3, 8))
    t = next_ticket(q, "sjf")
    assert t is q[2]
    works = [x.work for x in q]
    assert works[2] == works[3] < works[1] < works[0]
    q.remove(t)
    assert next_ticket(q, "sjf").id == 3  # the remaining (3, 8) request


def test_expected_work_scales_with_the_steps():
    q = queue(spec(3, 8))
    next_ticket(q, "fifo")
    tab, freq, cut = q[0]._built
    assert expected_work(tab, freq, cut[:11]) == pytest.approx(q[0].work * 10 / (len(cut) - 1))


def test_unknown_policy_is_rejected():
    from spinparser_gb300.serve import FlowServer
    with pytest.raises(ValueError):
        FlowServer(policy="lifo")


def test_sjf_admits_the_oldest_once_it_waited_too_long():
    q = queue(spec(5, 16), spec(3, 8))  # arrivals at t = 0 (large) and t = 1 (small)
    assert next_ticket(q, "sjf", now=5.0, max_wait=10.0) is q[1]
    assert next_ticket(q, "sjf", now=12.0, max_wait=10.0) is q[0]
    assert next_ticket(q, "sjf", now=12.0) is q[1]  # no bound: least work first


class _FailingBatch:
    def add(self, *a, **k):
        raise MemoryError("device memory exhausted")


def test_request_stays_queued_when_the_batch_cannot_take_it():
    from collections import deque

    from spinparser_gb300.serve import FlowServer

    srv = FlowServer.__new__(FlowServer)  # host logic only: no device batch
    srv.policy, srv.max_wait, srv.max_flows, srv.budget, srv.used = "fifo", None, None, 1 << 40, 0
    srv.clock = lambda: 0.0
    srv.batch = _FailingBatch()
    srv.queue, srv.active = deque(queue(spec(3, 8))), {}
    with pytest.raises(MemoryError):
        srv._admit()
    assert len(srv.queue) == 1 and not srv.active


class _FakeBatch:
    """poll() answers from a step table; set_paused() records the flows held out."""

    def __init__(self, steps):
        self.steps, self.paused = steps, set()

    def poll(self, fid):
        return 0, self.steps[fid], 0

    def set_paused(self, fid, paused):
        (self.paused.add if paused else self.paused.discard)(fid)


def test_srpt_runs_the_flows_with_least_remaining_work():
    from spinparser_gb300.serve import FlowServer, prepare

    srv = FlowServer.__new__(FlowServer)  # host logic only: no device batch
    srv.policy, srv.running, srv._paused, srv.keep_oldest = "srpt", 1, set(), False
    big, small = Ticket(0, spec(5, 16), 0.0), Ticket(1, spec(3, 8), 1.0)
    for t in (big, small):
        prepare(t)
    n_cut = len(big._built[2])
    srv.active = {10: big, 11: small}
    srv.batch = _FakeBatch({10: 0, 11: 0})
    srv._choose_running()
    assert srv.batch.paused == {10}  # the small request runs first
    srv.batch.steps = {10: n_cut - 2, 11: 0}  # the big one is almost done: least remaining work
    srv._choose_running()
    assert srv.batch.paused == {11}
    srv.running = 2
    srv._choose_running()
    assert srv.batch.paused == set()


def test_srpt_keeps_the_oldest_request_running():
    from spinparser_gb300.serve import FlowServer, prepare

    srv = FlowServer.__new__(FlowServer)
    srv.policy, srv.running, srv._paused, srv.keep_oldest = "srpt", 1, set(), True
    big, small = Ticket(0, spec(5, 16), 0.0), Ticket(1, spec(3, 8), 1.0)
    for t in (big, small):
        prepare(t)
    srv.active = {10: big, 11: small}
    srv.batch = _FakeBatch({10: 0, 11: 0})
    srv._choose_running()
    assert srv.batch.paused == set()  # the least remaining work and the oldest request both run
