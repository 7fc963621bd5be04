#!/usr/bin/env python3
"""Benchmark of the GB300 SU(2) pf-FRG flow core: cutoff steps per second of one flow.

Workload (default): SU(2) J1-J2 Heisenberg model on the simple cubic lattice, J1 = 1,
J2 = 0.25, lattice range 6 (23 symmetry-reduced site pairs, 4095 RPA pairs), 64 positive
Matsubara frequencies exponentially spaced in [0.005, 100], cutoff 100 -> 0.05 x 0.98
(377 cutoff values).  A step is one cutoff step as SpinParser's loop runs it: flow
right-hand side (self-energy flow + vertex flow), correlation measurement, explicit Euler
update.  The state is the model's initial condition advanced by the flow itself.

The work of a step grows as the cutoff decreases (more loop-frequency nodes lie above it),
so the K timed steps are spread evenly over the whole cutoff list: before each timed step
the flow's cutoff is moved to the next sampled value (untimed, as is an L2 flush), then one
genuine 0.98 step is taken.  The complete flow is also timed once ("full_flow").

JSON line (rank 0):
  value     steps/s with the state resident in HBM; device time from CUDA events on the
            flow's stream; L2 flushed (256 MB write) before every timed step
  e2e       steps/s through the C ABI with host buffers: every step uploads the state from
            pinned host memory, runs the step, reads the state and the correlations back
  roofline  the vertex-flow kernel: algorithmic FP32 work per launch
            F_RHS = F_N (2N+8) (3*100*Nl + 4*sum O) over its CUDA-event launch time, against
            the FP32 FMA throughput measured in-run on the same GPU; "evaluated" uses the
            node counts the step actually used instead of 2N+8; "gather": the kernel's slab
            gathers (16 segments of Nl pairs per evaluated node) per second against a pure
            gather kernel timed in-run on the same GPU (spn_measure_gather_peak)
  cpu_baseline  the CPU port of the reference's SU(2) core (the oracle's sources built with the
            reference's flags, -O3 -fopenmp) on all of this host's cores: three complete
            cutoff steps (full RHS over every triple, measurement, Euler) at cutoffs spread
            over the flow, from the GPU flow's final state; nproc and CPU model recorded

--impl reference times that CPU core alone (the reference's own C++ build needs Boost and
HDF5, absent here): every timed step one complete cutoff step at the cutoffs the GPU arm
times, so steps x ms_per_step is CPU time actually spent.  --gpus N > 1: replicas only
(independent flows, no collective).

Other workloads (--workload): pyrochlore-r5-n64, square-r3-n32, the serving mix's largest
classes pyrochlore-j1j2-r6-n64 / -r7-n64 and the reference README's readme-square-r4-n32 (the
same line for other shapes; --impl reference --cpu-full-flow times a whole CPU flow);
scan-square-j1j2-128 and serve-mixed (batched and served flows against sequential plain solves,
dealt over ranks under torchrun; --flows, --rates, --policy fifo|sjf[@k]|srpt[@k]|srpt+old[@k],
--grouping auto|on|off; --impl reference: the CPU port's flows/s; --profile-window START,COUNT:
batch steps inside an NVTX range for ncu); precision-* (FP32 forms against the FP64 GPU flow);
xyz-honeycomb-kitaev-r9-n48 and tri-honeycomb-kitaev-gamma-r9-n32 (whole flows of the XYZ and
TRI cores against their oracles; --flow-cutoffs M for short runs).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "cubic-j1j2-r6-n64": dict(lattice="cubic", range=6, model="cubic-j1j2heisenberg", params={"j1": "1.0", "j2": "0.25"},
                              n_freq=64, fmin=0.005, fmax=100.0, cmax=100.0, cmin=0.05, cstep=0.98),
    "square-r3-n32": dict(lattice="square", range=3, model="square-heisenberg", params={"j": "1.0"},
                          n_freq=32, fmin=0.005, fmax=50.0, cmax=50.0, cmin=0.05, cstep=0.98),
    "pyrochlore-r5-n64": dict(lattice="pyrochlore", range=5, model="pyrochlore-heisenberg", params={"j": "1.0"},
                              n_freq=64, fmin=0.002, fmax=100.0, cmax=100.0, cmin=0.01, cstep=0.99),
    # the largest request classes of the serving mix: pyrochlore range 6 (48 sites) and range 7
    # (70 sites), both on the CTA-per-triple kernel, J1-J2 with J2 = 0.25
    "pyrochlore-j1j2-r6-n64": dict(lattice="pyrochlore", range=6, model="pyrochlore-j1j2heisenberg",
                                   params={"j1": "1.0", "j2": "0.25"}, n_freq=64, fmin=0.005, fmax=50.0, cmax=50.0,
                                   cmin=0.05, cstep=0.98),
    "pyrochlore-j1j2-r7-n64": dict(lattice="pyrochlore", range=7, model="pyrochlore-j1j2heisenberg",
                                   params={"j1": "1.0", "j2": "0.25"}, n_freq=64, fmin=0.005, fmax=50.0, cmax=50.0,
                                   cmin=0.05, cstep=0.98),
    # the reference README's quick-start task (square r4, N = 32, cutoff 50 -> 0.1 x 0.95): the
    # sanity check of the CPU timings against the one figure the reference publishes
    "readme-square-r4-n32": dict(lattice="square", range=4, model="square-heisenberg", params={"j": "1.0"},
                                 n_freq=32, fmin=0.005, fmax=50.0, cmax=50.0, cmin=0.1, cstep=0.95),
}
DEFAULT_WORKLOAD = "cubic-j1j2-r6-n64"
# multi-flow workloads (spinparser_gb300/workloads.py): the seeded scan and the serving stream
MULTI_WORKLOADS = ("scan-square-j1j2-128", "serve-mixed")
# precision study: the single-flow workload run to the end in FP32 forms and in FP64 on the GPU
PRECISION_WORKLOADS = {"precision-cubic-j1j2-r6-n64": "cubic-j1j2-r6-n64",
                       "precision-pyrochlore-r5-n64": "pyrochlore-r5-n64"}
# the XYZ core (models with diagonal couplings): a Heisenberg-Kitaev flow
XYZ_WORKLOADS = {
    "xyz-honeycomb-kitaev-r9-n48": dict(lattice="honeycomb", range=9, model="honeycomb-kitaev",
                                        params={"j": "0.1", "k": "-1.0"}, n_freq=48, fmin=0.005, fmax=50.0,
                                        cmax=50.0, cmin=0.05, cstep=0.98),
}
# the TRI core (time-reversal-invariant models with off-diagonal couplings): a
# Heisenberg-Kitaev-Gamma flow
TRI_WORKLOADS = {
    "tri-honeycomb-kitaev-gamma-r9-n32": dict(lattice="honeycomb", range=9, model="honeycomb-kitaev-gamma",
                                              params={"j": "0.2", "k": "1.0", "g": "-0.1"}, n_freq=32, fmin=0.005,
                                              fmax=50.0, cmax=50.0, cmin=0.05, cstep=0.98),
}
METRIC = "cutoff steps/s per flow"
PRECISION_FORMS = {
    "fp64-self-energy": "FP32 vertex state and flow with Kahan-compensated loop-frequency sums; FP64 self-energy state, "
                        "flow and Euler update, FP64 quadrature weights and FP64 measurement accumulation "
                        "(SPN_SU2_FP64_SELF_ENERGY)",
    "plain": "FP32 vertex and self-energy state (the reference's types) with Kahan-compensated loop-frequency sums; "
             "FP64 quadrature weights and FP64 measurement accumulation",
}
KERNELS_PER_STEP = 7  # self-energy, node tables, vertex flow, 2 x correlation, 2 x Euler (state, self-energy)


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + list(MULTI_WORKLOADS) + list(PRECISION_WORKLOADS) +
                    list(XYZ_WORKLOADS) + list(TRI_WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--flows", type=int, default=None, help="multi-flow workloads: number of flows / requests")
    ap.add_argument("--rates", type=str, default="0.5,1,2,4,inf",
                    help="serve-mixed: arrival rates as multiples of the sequential plain-GPU capacity")
    ap.add_argument("--policy", type=str, default="fifo",
                    help="serve-mixed: server arms to run at every rate, comma separated: fifo or sjf, optionally @k "
                         "for a k-flow residency limit, srpt@k (k flows with the least remaining work run at each "
                         "step) or srpt+old@k (those and the oldest request), e.g. fifo,sjf@2,srpt@1,srpt+old@1")
    ap.add_argument("--grouping", choices=["auto", "on", "off"], default="auto",
                    help="scan/serve: batch configuration chosen by the batch autotuner (auto), cross-flow sharing "
                         "for every group of >= 2 flows (on), or the per-flow kernel without sharing (off)")
    ap.add_argument("--profile-window", type=str, default=None,
                    help="scan/serve: START,COUNT -- run the batch alone (no plain arm, no graph replay) for START "
                         "steps, then COUNT steps inside an NVTX range 'batch_steps' (for ncu --nvtx-include), "
                         "print their time and exit")
    ap.add_argument("--flow-cutoffs", type=int, default=None,
                    help="XYZ/TRI workloads: run only the first M cutoffs of the flow (short runs for profiling)")
    ap.add_argument("--precision", choices=["fp64-self-energy", "plain"], default="fp64-self-energy",
                    help="single-flow workloads: the precision form timed (default: FP32 vertex with Kahan sums, FP64 "
                         "self-energy, quadrature weights and measurement; plain: FP32 self-energy state)")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-full-flow", action="store_true")
    ap.add_argument("--cpu-full-flow", action="store_true",
                    help="--impl reference: time the whole flow (every cutoff: RHS, measurement, Euler) on the "
                         "host cores instead of sampled steps")
    return ap.parse_args()


def setup(wl):
    import spinparser_gb300 as spn

    lat = spn.Lattice(wl["lattice"], wl["range"], wl["model"], wl["params"])
    tab = lat.tables()
    freq = spn.frequency_exponential(wl["fmin"], wl["fmax"], wl["n_freq"])
    cut = spn.cutoff_exponential(wl["cmax"], wl["cmin"], wl["cstep"])
    return tab, freq, cut


def sampled_steps(n_cut: int, first: int, k: int) -> list[int]:
    """k cutoff indices spread evenly over [first, n_cut - 2]."""
    return [int(round(x)) for x in np.linspace(first, n_cut - 2, k)]


def flops_nominal(tab, n):
    fn = n * n * (n + 1) // 2
    return float(fn) * (2 * n + 8) * (3 * 100 * tab.n_sites + 4 * tab.n_overlap)


def gathers_evaluated(n, counts):
    """Slab-segment gathers of the vertex flow for the node counts of a step: four access
    buffers of four interpolation supports per node, each support one segment of Nl pairs."""
    c = np.asarray(counts, np.float64)
    tot = 0.0
    for s in range(n):
        for u in range(s + 1):
            tot += n * (c[s] + c[u]) + float(np.sum(c))
    return 16.0 * tot


def flops_evaluated(tab, n, counts):
    """Same per-node costs, with the node counts the step actually used."""
    c = np.asarray(counts, np.float64)
    tot = 0.0
    for s in range(n):
        for u in range(s + 1):
            base = c[s] + c[u]
            tot += n * base * 100 * tab.n_sites + float(np.sum(c)) * (100 * tab.n_sites + 4 * tab.n_overlap)
    return tot


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) >= 9:
                    rows.append(p)
        os.unlink(self.file.name)
        if not rows:
            return None

        def num(x):
            try:
                return float(x)
            except ValueError:
                return float("nan")

        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.nanmedian([num(r[1]) for r in rows])),
                "sm_max_mhz": float(np.nanmax([num(r[2]) for r in rows])), "reasons": reasons,
                "samples": len(rows), "power_w_max": float(np.nanmax([num(r[3]) for r in rows]))}


def cpu_info() -> dict:
    """Host cores and CPU model of the machine the CPU numbers come from."""
    model = None
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"nproc": os.cpu_count() or 1, "cpu_model": model or platform.machine()}


CPU_BUILD = "oracle sources at the reference's flags: g++ -O3 -fopenmp (default FP contraction)"


class CpuStep:
    """One cutoff step of the CPU core, as the reference's loop runs it: the complete flow
    right-hand side (self-energy flow, then the vertex flow of every triple, OpenMP over
    triples on all host cores), the correlation measurement and the explicit Euler update,
    with the oracle built at the reference's optimisation flags."""

    def __init__(self, tab, freq, state):
        from oracle import Oracle

        self.orc = Oracle(tab, freq, timing=True)
        self.threads = os.cpu_count() or 1
        self.v2, self.ss, self.dd = (np.array(x, np.float32).reshape(-1) for x in state)
        self.flush = np.empty(64 * 1024 * 1024, np.float32)  # 256 MB, larger than the host caches

    def flush_caches(self, i):
        self.flush.fill(float(i))

    def run(self, cutoff, new_cutoff):
        o = self.orc
        dv2, dss, ddd = o.rhs(cutoff, self.v2, self.ss, self.dd, threads=self.threads)
        o.correlation(cutoff, self.v2, self.ss, self.dd)
        o.euler(cutoff, new_cutoff, self.v2, dv2)
        o.euler(cutoff, new_cutoff, self.ss, dss)
        o.euler(cutoff, new_cutoff, self.dd, ddd)

    def warm(self, cutoff):
        """An untimed warm-up: the self-energy flow and a 1 % triple sample (threads started,
        pages touched)."""
        o = self.orc
        dv2 = o.self_energy(cutoff, self.v2, self.ss, self.dd)
        sample = np.arange(0, o.fn, 100, dtype=np.int32)
        o.vertex_sample(cutoff, self.v2, dv2, self.ss, self.dd, sample, self.threads)


def cpu_baseline(tab, freq, cut, state, n_steps=3):
    """The CPU core on all host cores: n_steps complete cutoff steps (full RHS, measurement,
    Euler) at cutoffs spread evenly over the list, from the given state."""
    step = CpuStep(tab, freq, state)
    # the midpoints of n_steps equal parts of the list (the work of a step grows as the
    # cutoff falls, so the mean over them follows the whole flow's mean)
    idx = [min(len(cut) - 2, int((i + 0.5) * (len(cut) - 1) / n_steps)) for i in range(n_steps)]
    step.warm(float(cut[idx[0]]))
    secs = []
    for i, k in enumerate(idx):
        step.flush_caches(i)
        t0 = time.perf_counter()
        step.run(float(cut[k]), float(cut[k + 1]))
        secs.append(time.perf_counter() - t0)
    t_step = float(np.mean(secs))
    info = cpu_info()
    return {"value": 1.0 / t_step, "unit": "steps/s", "cores": step.threads, "kind": "port", **info,
            "build": CPU_BUILD,
            "sample": f"{n_steps} complete cutoff steps (every one of {step.orc.fn} triples, measurement, Euler) at "
                      f"cutoffs {[round(float(cut[k]), 4) for k in idx]}; {sum(secs):.1f} s on {step.threads} threads; "
                      f"mean {t_step:.2f} s per step"}


def workload_config(args, wl, tab, cut, n, world=1):
    """The workload as both arms print it."""
    fn = n * n * (n + 1) // 2
    return {"workload": args.workload, "lattice": wl["lattice"], "range": wl["range"], "model": wl["model"],
            "params": wl["params"], "n_freq": n, "freq_range": [wl["fmin"], wl["fmax"]],
            "cutoff": [wl["cmax"], wl["cmin"], wl["cstep"]], "n_cutoffs": len(cut), "n_sites": tab.n_sites,
            "n_overlap": tab.n_overlap, "n_triples": fn, "parallelism": f"replicas x{world}",
            "timed_steps": "spread evenly over the cutoff list",
            "l2": "flushed (256 MB write) before every timed step"}


def run_reference(args, wl):
    """--impl reference: the reference's SU(2) core on the host cores (the oracle port built with
    the reference's flags), rank 0 only.  Every timed step is one complete cutoff step (full
    RHS over all triples, measurement, Euler) at the cutoffs the GPU arm times; the state is
    the model's initial condition, advanced by these steps (the work of a step depends on the
    cutoff, not on the state's values)."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    tab, freq, cut = setup(wl)
    n = len(freq)
    if args.cpu_full_flow:
        run_reference_flow(args, wl, tab, freq, cut)
        return
    step = CpuStep(tab, freq, tab.initial_state(n))
    schedule = sampled_steps(len(cut), args.warmup, args.steps)
    for _ in range(args.warmup):
        step.warm(float(cut[schedule[0]]))
    secs = []
    wall0 = time.perf_counter()
    for i, k in enumerate(schedule):
        step.flush_caches(i)
        t0 = time.perf_counter()
        step.run(float(cut[k]), float(cut[k + 1]))
        secs.append(time.perf_counter() - t0)
    wall = time.perf_counter() - wall0
    total = float(np.sum(secs))
    value = len(schedule) / total
    info = cpu_info()
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": len(schedule), "warmup": args.warmup, "ms_per_step": 1e3 * total / len(schedule),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (model initial condition, advanced by the timed steps)",
            "config": workload_config(args, wl, tab, cut, n),
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": step.threads, "kind": "port", **info,
                             "build": CPU_BUILD,
                             "sample": f"{len(schedule)} complete cutoff steps (full RHS over all {step.orc.fn} triples, "
                                       f"measurement, Euler) at the GPU arm's cutoffs; warm-up steps: self-energy + "
                                       f"1 % triple sample, untimed"},
            "lattice_tables": "built by the repository's lattice factory (input, pinned by the hyperkagome golden)",
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))


def run_reference_flow(args, wl, tab, freq, cut):
    """The whole flow of the workload on the host cores, as the reference's loop runs it
    (measurement at every cutoff, RHS, Euler), with the oracle built at the reference's flags;
    wall time of the complete flow."""
    from oracle import Oracle

    orc = Oracle(tab, freq, timing=True)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    n_meas, _, _, _ = orc.flow(cut, *tab.initial_state(len(freq)), threads=threads)
    secs = time.perf_counter() - t0
    steps = n_meas - 1
    info = cpu_info()
    line = {"impl": "reference", "metric": METRIC, "value": steps / secs, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": 0, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (model initial condition, advanced by the flow)",
            "config": workload_config(args, wl, tab, cut, len(freq)),
            "cpu_baseline": {"value": steps / secs, "unit": "steps/s", "cores": threads, "kind": "port", **info,
                             "build": CPU_BUILD,
                             "sample": f"the whole flow: {len(cut)} cutoffs, {steps} RHS evaluations, measurement at "
                                       f"every cutoff; {secs:.2f} s wall"},
            "full_flow_seconds": secs,
            "e2e": {"value": steps / secs, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _plain_solve(spec):
    """One request solved alone on the plain single-flow path (tables, flow, full cutoff loop)."""
    import spinparser_gb300 as spn
    from spinparser_gb300.driver import run_flow

    tab, freq, cut = spec.build()
    flow = spn.Su2Flow(tab, freq, flags=spec.flags)
    meas, zz, dd, cz, cd, div = run_flow(flow, cut, tab.initial_state(len(freq)))
    flow.close()
    return meas, zz, dd, div


def _cpu_flow_seconds(specs, steps_per_class):
    """CPU time of whole flows, per distinct (lattice, range, model, N): the mean time of
    complete CPU steps at cutoffs spread over the flow, times the flow's steps."""
    classes = {}
    for sp in specs:
        classes.setdefault((sp.lattice, sp.range, sp.model, sp.n_freq), []).append(sp)
    total, samples, b = 0.0, [], None
    for (lat, rng_, model, n), members in classes.items():
        sp = members[0]
        tab, freq, cut = sp.build()
        b = cpu_baseline(tab, freq, cut, tab.initial_state(len(freq)), steps_per_class)
        t_step = 1.0 / b["value"]
        total += t_step * (len(cut) - 1) * len(members)
        samples.append(f"{lat} r{rng_} N{n}: {t_step:.3f} s/step x {len(members)}")
    return total, samples, b


def run_batch_window(args):
    """The batch of the scan or serving workload's flows (all admitted at once), steps START ..
    START + COUNT - 1 inside an NVTX range 'batch_steps'; no graph replay, so every kernel is a
    plain launch that a profiler sees by name."""
    import torch

    from spinparser_gb300 import workloads
    from spinparser_gb300.batch import Su2Batch

    start, count = (int(x) for x in args.profile_window.split(","))
    scan = args.workload.startswith("scan")
    n = args.flows or (128 if scan else 24)
    specs = workloads.scan_specs(n) if scan else workloads.serve_specs(n)
    torch.cuda.set_device(0)
    b = Su2Batch(use_graph=False)
    for sp in specs:
        tab, freq, cut = sp.build()
        b.add(tab, freq, cut, flags=sp.flags)
    tune = None
    if args.grouping == "off":
        b.set_grouping(0)
    elif args.grouping == "on":
        b.set_grouping(2)
    else:
        tune = b.autotune(1)
    for _ in range(start):
        b.step()
    b.synchronize()
    torch.cuda.nvtx.range_push("batch_steps")
    t0 = time.perf_counter()
    for _ in range(count):
        b.step()
    b.synchronize()
    secs = time.perf_counter() - t0
    torch.cuda.nvtx.range_pop()
    print(json.dumps({"workload": args.workload, "flows": n, "grouping": args.grouping, "autotune": tune,
                      "grouped_flows": b.grouped_flows(), "window": [start, count], "seconds": secs,
                      "ms_per_step": 1e3 * secs / max(count, 1)}))
    b.close()


def run_multi_reference(args):
    """--impl reference for the scan and serving workloads: the CPU port's flows/s, rank 0 only.
    Per (lattice, range, model, N) class of the seeded flows, the mean time of complete CPU
    steps (full RHS, measurement, Euler) at cutoffs spread over the flow, times the flow's steps
    and the class's flows (extrapolated to whole flows)."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from spinparser_gb300 import workloads

    scan = args.workload.startswith("scan")
    n = args.flows or (128 if scan else 24)
    specs = workloads.scan_specs(n) if scan else workloads.serve_specs(n)
    t0 = time.perf_counter()
    cpu_s, samples, b = _cpu_flow_seconds(specs, 2 if scan else 1)
    wall = time.perf_counter() - t0
    value = n / cpu_s
    line = {"impl": "reference", "metric": "scan flows/s" if scan else "served flows/s", "value": value,
            "unit": "flows/s", "n_gpus": args.gpus, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": args.workload, "flows": n, "seed": workloads.SEED},
            "cpu_baseline": {"value": value, "unit": "flows/s", "cores": b["cores"], "kind": "port", "nproc": b["nproc"],
                             "cpu_model": b["cpu_model"], "build": CPU_BUILD,
                             "sample": "per (lattice, range, N): mean time of %d complete CPU steps spread over the "
                                       "flow, x its steps (extrapolated); " % (2 if scan else 1) + "; ".join(samples)},
            "cpu_seconds_for_all_flows": cpu_s,
            "e2e": {"value": value, "unit": "flows/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": wall}
    print(json.dumps(line))


def _by_class(specs, secs):
    """Total seconds and flow count per (lattice, range, N) class."""
    out = {}
    for sp, t in zip(specs, secs):
        k = f"{sp.lattice} r{sp.range} N{sp.n_freq}"
        tot, cnt = out.get(k, (0.0, 0))
        out[k] = (tot + float(t), cnt + 1)
    return {k: {"seconds": round(v[0], 4), "flows": v[1]} for k, v in sorted(out.items())}


def _check_same(a, b):
    """Largest absolute difference of two flows' correlations (0.0 = bit-identical)."""
    am, azz, add_, _ = a
    if len(am) != len(b.cutoffs) or not np.array_equal(am, b.cutoffs):
        return float("inf")
    return float(max(np.nanmax(np.abs(azz.reshape(b.zz.shape) - b.zz)), np.nanmax(np.abs(add_.reshape(b.dd.shape) - b.dd))))


def _serve_local(items, arrivals, policy, plain, grouping="auto"):
    """One rank's server over its dealt requests: (index, spec) items arriving at their offsets
    of the global stream.  Returns per item (time to result, largest difference from the same
    flow solved alone) and the rank's makespan."""
    from spinparser_gb300.serve import FlowServer

    name, _, slots = policy.partition("@")
    keep_oldest = name.endswith("+old")
    name = name[:-len("+old")] if keep_oldest else name
    # the scan (every flow admitted at once) is tuned once its flows have stepped together; a
    # request stream's running set changes too often for tuning to pay
    srv = FlowServer(policy=name, max_flows=int(slots) if slots else None, keep_oldest=keep_oldest,
                     autotune=(grouping == "auto" and not np.any(arrivals)))
    if grouping == "off":
        srv.batch.set_grouping(0)
    elif grouping == "on":
        srv.batch.set_grouping(2)
    order = sorted(range(len(items)), key=lambda j: arrivals[items[j][0]])
    t0 = time.perf_counter()
    tickets, k = {}, 0
    while True:
        now = time.perf_counter() - t0
        while k < len(order) and arrivals[items[order[k]][0]] <= now:
            j = order[k]
            tickets[j] = srv.submit(items[j][1], t_arrival=t0 + arrivals[items[j][0]])
            k += 1
        if srv.pump() == 0:
            if k >= len(order):
                break
            time.sleep(min(0.01, max(0.0, arrivals[items[order[k]][0]] - (time.perf_counter() - t0))))
    makespan = time.perf_counter() - t0
    steps = (srv.steps, srv.tunings[:4])
    srv.close()
    out = [(tickets[j].time_to_result, _check_same(plain[items[j][0]], tickets[j].result)) for j in range(len(items))]
    return out, makespan, steps


def run_multi(args):
    """Multi-flow workloads: batched / served flows against sequential plain-GPU solves.  Under
    torchrun the flows are dealt round-robin over the ranks (replicas.run_sharded), each rank
    runs its own plain solves and its own batch or server, and flows/s is all flows over the
    slowest rank's time (weak scaling: per-rank work is the dealt share)."""
    import torch

    from spinparser_gb300 import replicas, workloads
    from spinparser_gb300.serve import time_to_result_stats

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    scan = args.workload.startswith("scan")
    n = args.flows or (128 if scan else 24)
    specs = workloads.scan_specs(n) if scan else workloads.serve_specs(n)
    items = list(enumerate(specs))
    # warm-up (untimed): kernels loaded, caches warm, allocator primed
    warm = [workloads.FlowSpec("square", 3, "square-j1j2heisenberg", (("j1", "1.0"), ("j2", "0.3")), 16,
                               0.005, 50.0, 50.0, 5.0, 0.9)] * 3
    for sp in warm:
        _plain_solve(sp)
    from spinparser_gb300.serve import FlowServer

    srv = FlowServer()
    for sp in warm:
        srv.submit(sp)
    srv.drain()
    srv.close()

    sampler = ClockSampler(local)
    sampler.start()
    plain = {}

    # sequential plain-GPU solves of each rank's share (FIFO, all present at t = 0)
    def plain_solve(local_items):
        t0 = time.perf_counter()
        res = []
        for i, sp in local_items:
            ts = time.perf_counter()
            plain[i] = _plain_solve(sp)
            res.append(time.perf_counter() - ts)
        return res, time.perf_counter() - t0

    if dist:
        dist.barrier()
    job_plain, service_all, mine = replicas.run_sharded(items, plain_solve)
    service = np.array(service_all)
    arms = {}
    rates = [float("inf")] if scan else [float(x) * world / service.mean() for x in args.rates.split(",")]
    max_diff = 0.0
    policies = ["fifo"] if scan else args.policy.split(",")
    for rate in rates:
        arrivals = workloads.poisson_arrivals(n, rate)
        served = {}
        for policy in policies:
            stats = {}

            def served_solve(local_items):
                out, makespan, steps = _serve_local(local_items, arrivals, policy, plain, args.grouping)
                stats["steps"] = steps
                return out, makespan

            if dist:
                dist.barrier()
            job, res, _ = replicas.run_sharded(items, served_solve)
            max_diff = max(max_diff, max(r[1] for r in res))
            ttr = np.array([r[0] for r in res])
            served[policy] = {"flows_per_s": job.throughput, "makespan_s": job.seconds, "steps_rank0": stats["steps"][0],
                              "autotune_rank0": stats["steps"][1],
                              "n": n, "p50_s": float(np.percentile(ttr, 50)), "p99_s": float(np.percentile(ttr, 99)),
                              "mean_s": float(ttr.mean()), "max_s": float(ttr.max())}
        # the same arrivals served by each rank's sequential plain path (FIFO queue of its
        # service times over its share of the stream)
        plain_ttr, free_at = [], {}
        for k in range(n):
            r_ = k % world
            start = max(free_at.get(r_, 0.0), arrivals[k])
            free_at[r_] = start + service[k]
            plain_ttr.append(free_at[r_] - arrivals[k])
        span = max(free_at.values())
        arms["inf" if not np.isfinite(rate) else f"{rate:.4g}"] = {
            "arrival_rate_per_s": None if not np.isfinite(rate) else rate,
            "batched": served[policies[0]],
            **({"batched_by_policy": served} if len(policies) > 1 else {}),
            "plain_gpu_fifo": {"flows_per_s": n / max(span, 1e-9), "makespan_s": span,
                               "p50_s": float(np.percentile(plain_ttr, 50)), "p99_s": float(np.percentile(plain_ttr, 99))},
        }
    clocks = sampler.stop()
    if dist:
        dist.barrier()
    if rank != 0:
        dist.destroy_process_group()
        return
    cpu_s, cpu_samples, cpu_b = (_cpu_flow_seconds(specs, 2 if scan else 1) if not args.no_cpu_baseline and world == 1
                                 else (None, [], None))
    top = arms[list(arms)[-1]]
    line = {
        "metric": "scan flows/s" if scan else "served flows/s",
        "value": top["batched"]["flows_per_s"], "unit": "flows/s", "n_gpus": world,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": {"workload": args.workload, "flows": n, "seed": workloads.SEED, "grouping": args.grouping,
                   "parallelism": f"replicas x{world} (flows dealt round-robin)",
                   "draws": "square J1-J2, J2 U[0,1], range U{3,5,7}, N U{32,48,64}, grid [0.005,50], cutoff 50->0.05 x0.98"
                   if scan else "square/cubic/pyrochlore J1-J2, J2 U[-0.5,0.5], range U{3..7}, N U{32,48,64}, "
                                "grid [0.005,50], cutoff 50->0.05 x0.98, Poisson arrivals"},
        "plain_gpu_sequential": {"flows_per_s": job_plain.throughput, "seconds": job_plain.seconds,
                                 "service_s_mean": float(service.mean()), "service_s_max": float(service.max()),
                                 "seconds_by_class": _by_class(specs, service)},
        "speedup_vs_plain": top["batched"]["flows_per_s"] / job_plain.throughput,
        "arms": arms,
        "max_abs_diff_vs_plain": max_diff,
        "cpu_baseline": None if cpu_s is None else {
            "value": n / cpu_s, "unit": "flows/s", "cores": cpu_b["cores"], "kind": "port", "nproc": cpu_b["nproc"],
            "cpu_model": cpu_b["cpu_model"], "build": CPU_BUILD,
            "sample": "per (lattice, range, N): mean time of %d complete CPU steps spread over the flow, x its steps "
                      "(extrapolated); " % (2 if scan else 1) + "; ".join(cpu_samples)},
        "clocks": clocks,
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def _flow_history(flow, cut, fp64):
    """Runs a flow over the whole cutoff list as the task driver does (measure, then step) and
    returns (chi_zz[k, Nl], zz[k, n_corr], seconds, steps measured); stops at a divergence."""
    import spinparser_gb300 as spn  # noqa: F401

    chi = np.full((len(cut), flow.nl), np.nan)
    zz = np.full((len(cut), flow.n_corr), np.nan)
    t0 = time.perf_counter()
    k = 0
    for k in range(len(cut)):
        if fp64:
            z, _, c, _ = flow.measure_correlation_f64()
        else:
            z, _, c, _ = flow.measure_correlation()
        chi[k], zz[k] = c, z
        if k + 1 == len(cut):
            break
        flow.compute_step()
        flow.finalize_step(float(cut[k + 1]))
        if flow.is_diverged():
            break
    flow.synchronize()
    return chi, zz, time.perf_counter() - t0, k + 1


def run_precision(args):
    """Error of the FP32 flows against the FP64 flow of the same task, both on the GPU.

    Three flows from the same initial condition over the whole cutoff list, each measured at
    every cutoff: the FP64 flow (SPN_SU2_FP64: every operation in double), the precision form
    (FP32 vertex with Kahan-compensated loop-frequency sums, FP64 self-energy state, quadrature
    weights and measurement accumulation: SPN_SU2_FP64_SELF_ENERGY) and the plain FP32 flow.
    The error at cutoff k is normwise, max_rid |chi32 - chi64| / max_rid |chi64| of the static
    spin susceptibility (and the same for the correlation entries zz)."""
    import torch

    import spinparser_gb300 as spn

    torch.cuda.set_device(0)
    name = PRECISION_WORKLOADS[args.workload]
    wl = WORKLOADS[name]
    tab, freq, cut = setup(wl)
    init = tab.initial_state(len(freq))
    sampler = ClockSampler(0)
    sampler.start()
    arms = {}
    for label, flags in (("fp64", spn.FP64), ("fp32_fp64_self_energy", spn.FP64_SELF_ENERGY), ("fp32_plain", 0)):
        flow = spn.Su2Flow(tab, freq, flags=flags)
        flow.set_state(float(cut[0]), *init)
        if flags != spn.FP64:
            flow.autotune()
        arms[label] = _flow_history(flow, cut, flags == spn.FP64)
        flow.close()
    clocks = sampler.stop()
    chi64, zz64, t64, n64 = arms["fp64"]

    def err(a, b):
        return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))

    report = {}
    for label in ("fp32_fp64_self_energy", "fp32_plain"):
        chi, zz, secs, nk = arms[label]
        n = min(nk, n64)
        e_chi = np.array([err(chi[k], chi64[k]) for k in range(n)])
        e_zz = np.array([err(zz[k], zz64[k]) for k in range(n)])
        idx = sorted(set(np.linspace(0, n - 1, 12).astype(int).tolist()))
        report[label] = {
            "final_rel_err_chi": float(e_chi[n - 1]), "final_rel_err_zz": float(e_zz[n - 1]),
            "max_rel_err_chi": float(e_chi.max()), "max_rel_err_zz": float(e_zz.max()),
            "growth": [{"step": k, "cutoff": float(cut[k]), "rel_err_chi": float(e_chi[k]),
                        "rel_err_zz": float(e_zz[k])} for k in idx],
            "steps_measured": nk, "flow_seconds": secs, "steps_per_s": (nk - 1) / secs,
        }
    main_arm = report["fp32_fp64_self_energy"]
    line = {
        "metric": "final correlation rel. error vs FP64 GPU flow", "value": main_arm["final_rel_err_chi"],
        "unit": "relative", "n_gpus": 1, "higher_is_better": False, "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (model initial condition, advanced by the flow)", "tolerance": 1e-4,
        "within_tolerance": bool(main_arm["final_rel_err_chi"] <= 1e-4 and main_arm["final_rel_err_zz"] <= 1e-4),
        "config": {"workload": args.workload, "lattice": wl["lattice"], "range": wl["range"], "model": wl["model"],
                   "params": wl["params"], "n_freq": len(freq), "freq_range": [wl["fmin"], wl["fmax"]],
                   "cutoff": [wl["cmax"], wl["cmin"], wl["cstep"]], "n_cutoffs": len(cut), "n_sites": tab.n_sites},
        "fp64_flow": {"steps_measured": n64, "flow_seconds": t64, "steps_per_s": (n64 - 1) / t64},
        "arms": report,
        "clocks": clocks,
    }
    print(json.dumps(line))


def run_xyz(args):
    """The XYZ or TRI core: one whole flow on the GPU (device-resident state, measurement at
    every cutoff, as the driver runs it), against the core's oracle on the host cores (two
    right-hand sides at cutoffs a third and two thirds into the flow)."""
    import torch

    import spinparser_gb300 as spn

    torch.cuda.set_device(0)
    tri = args.workload in TRI_WORKLOADS
    wl = (TRI_WORKLOADS if tri else XYZ_WORKLOADS)[args.workload]
    lat = spn.Lattice(wl["lattice"], wl["range"], wl["model"], wl["params"])
    tab, st = lat.tables(), lat.spin_tables()
    freq = spn.frequency_exponential(wl["fmin"], wl["fmax"], wl["n_freq"])
    cut = spn.cutoff_exponential(wl["cmax"], wl["cmin"], wl["cstep"])
    n_cut = len(cut)
    if args.flow_cutoffs:
        cut = cut[:max(args.flow_cutoffs, 2)]
    if tri:
        init = spn.tri_initial_state(lat, len(freq))
        flow = spn.TriFlow(tab, st, freq)
    else:
        init = spn.xyz_initial_state(lat, len(freq))
        flow = spn.XyzFlow(tab, st, freq)
    warm = max(args.warmup, 3)
    flow.run(cut[:warm + 1], *init)  # untimed warm-up
    sampler = ClockSampler(0)
    sampler.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    measured, corr, diverged = flow.run(cut, *init)
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    clocks = sampler.stop()
    steps = len(measured) - 1
    line = {
        "metric": "cutoff steps/s per flow (%s core)" % ("TRI" if tri else "XYZ"), "value": steps / secs,
        "unit": "steps/s", "n_gpus": 1,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * secs / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (model initial condition, advanced by the flow)",
        "config": {"workload": args.workload, **{k: wl[k] for k in ("lattice", "range", "model", "params", "n_freq")},
                   "cutoff": [wl["cmax"], wl["cmin"], wl["cstep"]], "n_cutoffs": n_cut, "n_sites": tab.n_sites,
                   "n_overlap": tab.n_overlap,
                   "timed": ("the first %d cutoffs" % len(cut) if args.flow_cutoffs else "the whole flow") +
                            ", measurement at every cutoff"},
        "diverged": diverged, "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        from oracle import TriOracle, XyzOracle

        orc = (TriOracle if tri else XyzOracle)(tab, st, freq)
        _, v2, v4 = flow.get_state()
        threads = os.cpu_count() or 1
        samples = []
        for frac in (1 / 3, 2 / 3):
            c = float(cut[int(frac * (len(cut) - 1))])
            t1 = time.perf_counter()
            orc.rhs(c, v2, v4, threads=threads)
            samples.append(time.perf_counter() - t1)
        per_step = float(np.mean(samples))
        line["cpu_baseline"] = {"value": 1.0 / per_step, "unit": "steps/s", "cores": threads, "kind": "port",
                                "sample": "two full right-hand sides of the %s oracle at the final state, cutoffs a "
                                          % ("TRI" if tri else "XYZ") +
                                          "third and two thirds into the list; %.2f s per step" % per_step}
    print(json.dumps(line))
    flow.close()


def main():
    args = parse_args()
    if args.workload in XYZ_WORKLOADS or args.workload in TRI_WORKLOADS:
        run_xyz(args)
        return
    if args.workload in MULTI_WORKLOADS:
        if args.profile_window:
            run_batch_window(args)
        elif args.impl == "reference":
            run_multi_reference(args)
        else:
            run_multi(args)
        return
    if args.workload in PRECISION_WORKLOADS:
        run_precision(args)
        return
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
        return
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")

    import torch

    import spinparser_gb300 as spn

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    tab, freq, cut = setup(wl)
    n = len(freq)
    if args.warmup + 2 > len(cut):
        raise SystemExit("not enough cutoff values")
    flags = spn.FP64_SELF_ENERGY if args.precision == "fp64-self-energy" else 0
    flow = spn.Su2Flow(tab, freq, device=local, flags=flags)
    stream = torch.cuda.Stream(device=local)
    flow.set_stream(stream.cuda_stream)
    flow.set_state(float(cut[0]), *tab.initial_state(n))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2

    def step(k):
        flow.compute_step()
        flow.launch_correlation()
        flow.finalize_step(float(cut[k + 1]))

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    if flow.is_diverged():
        raise SystemExit("flow diverged during warm-up")
    # pick the vertex-flow kernel variant on a mid-flow cutoff (work grows as the cutoff falls)
    c_keep = flow.get_state()[0]
    flow.set_cutoff(float(cut[len(cut) // 2]))
    variant = flow.autotune(3)
    flow.set_cutoff(c_keep)

    schedule = sampled_steps(len(cut), args.warmup, args.steps)
    starts = [torch.cuda.Event(enable_timing=True) for _ in schedule]
    ends = [torch.cuda.Event(enable_timing=True) for _ in schedule]
    counts_sum = np.zeros(n, np.float64)
    sampler = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    flow.set_profiling(True)
    sampler.start()
    wall0 = time.perf_counter()
    flops_eval = 0.0
    gathers_eval = 0.0
    for i, k in enumerate(schedule):
        flow.set_cutoff(float(cut[k]))
        with torch.cuda.stream(stream):
            flush.fill_(float(i))
        starts[i].record(stream)
        step(k)
        ends[i].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    clocks = sampler.stop()
    if dist:
        dist.barrier()
    total_ms = float(np.sum([s.elapsed_time(e) for s, e in zip(starts, ends)]))
    prof = flow.profile()
    diverged = flow.is_diverged()
    flow.set_profiling(False)
    # evaluated work of the sampled steps (node counts depend only on the cutoff)
    for k in schedule:
        flow.set_cutoff(float(cut[k]))
        flow.compute_step()
        flops_eval += flops_evaluated(tab, n, flow.node_counts())
        gathers_eval += gathers_evaluated(n, flow.node_counts())
    # replicas: every rank ran its own flow; units summed, slowest rank's time
    from spinparser_gb300 import replicas

    job = replicas.aggregate(len(schedule), total_ms * 1e-3)
    total_ms = job.seconds * 1e3

    # end to end through the C ABI with pinned host buffers
    fn_nl = flow.fn * flow.nl
    pin = lambda m: torch.empty(m, dtype=torch.float32, pin_memory=True).numpy()  # noqa: E731
    h_v2, h_ss, h_dd = pin(n), pin(fn_nl), pin(fn_nl)
    h_zz, h_dc = pin(flow.n_corr), pin(flow.n_corr)
    flow.get_state(h_v2, h_ss, h_dd)
    e2e_sched = sampled_steps(len(cut), args.warmup, args.e2e_steps)
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for k in e2e_sched:
        flow.set_state(float(cut[k]), h_v2, h_ss, h_dd)
        flow.compute_step()
        flow.launch_correlation()
        flow.get_correlation(h_zz, h_dc)
        flow.finalize_step(float(cut[k + 1]))
        flow.get_state(h_v2, h_ss, h_dd)
    e2e_s = time.perf_counter() - e0
    state_bytes = 4 * (n + 2 * fn_nl)

    # the complete flow, device resident (time to result of one flow)
    full = None
    if not args.no_full_flow:
        flow.set_state(float(cut[0]), *tab.initial_state(n))
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        f0.record(stream)
        for k in range(len(cut) - 1):
            step(k)
        flow.launch_correlation()
        f1.record(stream)
        torch.cuda.synchronize()
        fs = f0.elapsed_time(f1) * 1e-3
        full = {"steps": len(cut) - 1, "seconds": fs, "steps_per_s": (len(cut) - 1) / fs,
                "diverged": flow.is_diverged()}

    fp32_peak, clk = spn.measure_fp32_peak(local)
    gather = None
    if tab.n_sites <= 32:
        # the slab gathers against a pure gather kernel: state-sized (L2-resident) and
        # L1-resident working sets; the larger rate is the denominator
        g_l2 = spn.measure_gather_peak(tab.n_sites, flow.fn, local)
        g_l1 = spn.measure_gather_peak(tab.n_sites, 512, local)
        g_ach = gathers_eval / (prof["vertex_ms"] * 1e-3)
        gather = {"kernel": "su2_vertex_flow_kernel", "achieved": g_ach / 1e9, "peak": max(g_l1, g_l2) / 1e9,
                  "unit": "G segments/s", "frac": g_ach / max(g_l1, g_l2), "peak_l2_resident": g_l2 / 1e9,
                  "peak_l1_resident": g_l1 / 1e9,
                  "segment": f"{tab.n_sites} float2 pairs (one interpolation support of one access buffer)",
                  "peak_source": "measured in-run: pure gather kernel on this GPU (spn_measure_gather_peak)"}
    avg_vertex_ms = prof["vertex_ms"] / max(1, prof["vertex_launches"])
    nominal = flops_nominal(tab, n)
    achieved = nominal / (avg_vertex_ms * 1e-3) / 1e12
    achieved_eval = flops_eval / (prof["vertex_ms"] * 1e-3) / 1e12
    # the dominant kernel: a warp per triple up to 32 sites, a CTA per triple above
    kernel = "su2_vertex_flow_kernel" if tab.n_sites <= 32 else "su2_vertex_big_kernel"
    traffic = None
    prof_file = os.path.join(ROOT, "profiles", f"{kernel.replace('su2_', '').replace('_kernel', '')}_{args.workload}.json")
    if os.path.exists(prof_file):
        traffic = json.load(open(prof_file)).get("dram_bytes_per_launch")

    if rank != 0:
        flow.close()
        if dist:
            dist.destroy_process_group()
        return
    value = job.throughput
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": len(schedule),
        "warmup": args.warmup, "ms_per_step": total_ms / len(schedule), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (model initial condition, advanced by the flow)",
        "config": workload_config(args, wl, tab, cut, n, world),
        "e2e": {"value": len(e2e_sched) / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes + 8 * flow.n_corr},
        "roofline": {"bound": "fp32", "kernel": kernel, "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": traffic,
                     "algorithmic_flops_per_launch": nominal, "avg_launch_ms": avg_vertex_ms,
                     "achieved_evaluated": achieved_eval, "frac_evaluated": achieved_eval / fp32_peak,
                     "peak_source": "measured in-run: pure-FFMA kernel on this GPU (MEASURED_PEAKS.json has no "
                                    "FP32 CUDA-core figure)", "fp32_clock_ghz_implied": clk,
                     "gather": gather},
        "precision_form": PRECISION_FORMS[args.precision],
        "vertex_variant": dict(variant, kernel=kernel),
        "gpu_launches": KERNELS_PER_STEP * len(schedule),
        "clocks": clocks,
        "full_flow": full,
        "diverged": diverged,
        "wall_s": wall,
    }
    if not args.no_cpu_baseline and world == 1:
        c, v2, ss, dd = flow.get_state()
        line["cpu_baseline"] = cpu_baseline(tab, freq, cut, (v2, ss, dd), 3)
    print(json.dumps(line))
    flow.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
