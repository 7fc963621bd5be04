"""Replica-only multi-GPU logic, exercised with two gloo ranks on the CPU: the work split of
independent flows and the whole-job timing (units summed, slowest rank's time).  Each rank
runs a small flow with the CPU oracle standing in for its GPU, so the test needs no device."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from spinparser_gb300 import replicas


def test_shard_partitions_flows():
    parts = [replicas.shard(10, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == list(range(10))
    assert all(len(p) in (3, 4) for p in parts)
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def test_aggregate_without_process_group_is_local():
    t = replicas.aggregate(12, 3.0)
    assert (t.units, t.seconds, t.world) == (12.0, 3.0, 1)
    assert t.throughput == 4.0


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import spinparser_gb300 as spn
    from oracle import Oracle

    tab = spn.Lattice("square", 2, "square-heisenberg", {"j": "1.0"}).tables()
    freq = spn.frequency_exponential(0.05, 10.0, 6)
    cut = spn.cutoff_exponential(10.0, 1.0, 0.8)
    mine = replicas.shard(5, rank, world)  # five independent flows (J scan)
    chis = {}
    base = np.abs(tab.interaction_J)
    for i in mine:
        tab.interaction_J = base * (0.5 + 0.25 * i)
        n, cs, _, _ = Oracle(tab, freq).flow(cut, *tab.initial_state(len(freq)))
        chis[i] = cs[n - 1].tolist()
    local_seconds = 1.0 + rank  # rank 1 is the slow one
    job = replicas.aggregate(len(mine), local_seconds)
    out[rank] = {"units": job.units, "seconds": job.seconds, "world": job.world, "chis": chis}
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_split_flows_and_time_by_slowest_rank():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=240)
        assert all(p.exitcode == 0 for p in procs)
        res = dict(out)
    for r in (0, 1):
        assert res[r]["units"] == 5 and res[r]["seconds"] == 2.0 and res[r]["world"] == 2
    flows = {**res[0]["chis"], **res[1]["chis"]}
    assert sorted(flows) == [0, 1, 2, 3, 4]
    # a flow's result does not depend on which rank ran it: rerun flow 3 locally
    import spinparser_gb300 as spn
    from oracle import Oracle

    tab = spn.Lattice("square", 2, "square-heisenberg", {"j": "1.0"}).tables()
    freq = spn.frequency_exponential(0.05, 10.0, 6)
    cut = spn.cutoff_exponential(10.0, 1.0, 0.8)
    tab.interaction_J = np.abs(tab.interaction_J) * (0.5 + 0.25 * 3)
    n, cs, _, _ = Oracle(tab, freq).flow(cut, *tab.initial_state(len(freq)))
    assert np.array_equal(np.array(flows[3], np.float32), cs[n - 1])


def _scan_rank(rank, world, port, out):
    """A rank of the sharded scan driver: flows dealt by replicas.run_sharded, the CPU oracle
    standing in for the rank's GPU batch."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import time

    import spinparser_gb300 as spn
    from oracle import Oracle

    freq = spn.frequency_exponential(0.05, 10.0, 6)
    cut = spn.cutoff_exponential(10.0, 1.0, 0.8)
    specs = [(2 + (i % 2), 0.1 * i) for i in range(7)]  # (range, J2) of seven flows

    def solve(local):
        t0 = time.perf_counter()
        res = []
        for rng_, j2 in local:
            tab = spn.Lattice("square", rng_, "square-j1j2heisenberg", {"j1": "1.0", "j2": str(j2)}).tables()
            n, cs, _, _ = Oracle(tab, freq).flow(cut, *tab.initial_state(len(freq)))
            res.append(cs[n - 1].tolist())
        return res, (time.perf_counter() - t0) + 5.0 * rank  # rank 1 is made the slow one

    job, results, mine = replicas.run_sharded(specs, solve)
    out[rank] = {"units": job.units, "seconds": job.seconds, "world": job.world, "mine": mine, "results": results}
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_scan_driver_on_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_scan_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=240)
        assert all(p.exitcode == 0 for p in procs)
        res = dict(out)
    assert res[0]["mine"] == [0, 2, 4, 6] and res[1]["mine"] == [1, 3, 5]
    for r in (0, 1):
        assert res[r]["units"] == 7 and res[r]["world"] == 2
        assert res[r]["seconds"] >= 5.0  # the slowest rank's time
    assert res[0]["results"] == res[1]["results"]  # every rank holds every flow's result
    import spinparser_gb300 as spn
    from oracle import Oracle

    freq = spn.frequency_exponential(0.05, 10.0, 6)
    cut = spn.cutoff_exponential(10.0, 1.0, 0.8)
    for i in (3, 6):  # a flow's result does not depend on the rank that ran it
        tab = spn.Lattice("square", 2 + (i % 2), "square-j1j2heisenberg", {"j1": "1.0", "j2": str(0.1 * i)}).tables()
        n, cs, _, _ = Oracle(tab, freq).flow(cut, *tab.initial_state(len(freq)))
        assert np.array_equal(np.array(res[0]["results"][i], np.float32), cs[n - 1])
