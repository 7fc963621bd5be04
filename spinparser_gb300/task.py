"""Task files, checkpoints and observable files through the C ABI.

``run_task`` is SpinParser's ``run`` for one SU(2) task file (src/SpinParser.cpp:53-210):
the library parses the task, builds the lattice, runs the flow on the GPU and writes the
.obs / .checkpoint / .data / .ldf files beside the task file, with the calculation status
recorded in the task file so that a second call resumes or post-processes.  The checkpoint
and observable helpers expose the same file writers for callers that drive a flow
themselves (``Su2Flow``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._capi import RunOptions, RunResult, check, load_library
from .core import RES_DIR, FP64_SELF_ENERGY, Lattice

STATUS_NAMES = ("new", "running", "postprocessing", "finished")


@dataclass
class RunSummary:
    status: str          # calculation status recorded in the task file afterwards
    steps: int           # flow steps computed in this call
    measurements: int    # correlation measurements evaluated on the device
    diverged: bool
    flow_seconds: float  # wall time of the cutoff loop


def run_task(task_path: str, *, resource_path: str | None = None, checkpoint_time: int = 3600,
             force_restart: bool = False, defer: bool = False, debug_lattice: bool = False, verbose: int = 0,
             device: int = 0, fp64_self_energy: bool = False, autotune: bool = True) -> RunSummary:
    """Runs a task file; the keyword arguments are the reference's command-line options
    (--resourcePath, --checkpointTime, --forceRestart, --defer, --debugLattice, --verbose)
    plus the device, the FP64 self-energy mode and the kernel-variant autotuning."""
    lib = load_library()
    o = RunOptions()
    check(lib.spn_run_options_default(C.byref(o)))
    o.resource_path = (resource_path or RES_DIR).encode()
    o.checkpoint_time = int(checkpoint_time)
    o.force_restart = int(force_restart)
    o.defer = int(defer)
    o.debug_lattice = int(debug_lattice)
    o.verbose = int(verbose)
    o.device = int(device)
    o.flags = FP64_SELF_ENERGY if fp64_self_energy else 0
    o.autotune = int(autotune)
    r = RunResult()
    check(lib.spn_run_task(str(task_path).encode(), C.byref(o), C.byref(r)))
    return RunSummary(STATUS_NAMES[r.status], r.steps, r.measurements, bool(r.diverged), r.flow_seconds)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def write_checkpoint(path: str, cutoff: float, v2, v4ss, v4dd, append: bool = False) -> int:
    """Writes one checkpoint group; returns its id, or -1 if the file already holds a
    checkpoint at this cutoff (SU2EffectiveAction::writeCheckpoint)."""
    lib = load_library()
    v2, ss, dd = _f32(v2), _f32(v4ss), _f32(v4dd)
    if ss.size != dd.size:
        raise ValueError("v4ss and v4dd differ in size")
    fp = C.POINTER(C.c_float)
    out = C.c_int()
    check(lib.spn_su2_write_checkpoint(str(path).encode(), int(append), float(cutoff), v2.size, v2.ctypes.data_as(fp),
                                       ss.size, ss.ctypes.data_as(fp), dd.ctypes.data_as(fp), C.byref(out)))
    return out.value


def read_checkpoint(path: str, n_v2: int, n_v4: int, checkpoint_id: int = -1):
    """Reads checkpoint `checkpoint_id` (the last one for -1).  Returns (cutoff, v2, v4ss,
    v4dd), or None if it does not exist (SU2EffectiveAction::readCheckpoint)."""
    lib = load_library()
    v2 = np.empty(n_v2, np.float32)
    ss = np.empty(n_v4, np.float32)
    dd = np.empty(n_v4, np.float32)
    fp = C.POINTER(C.c_float)
    cut = C.c_float()
    found = C.c_int()
    check(lib.spn_su2_read_checkpoint(str(path).encode(), int(checkpoint_id), C.byref(cut), n_v2, v2.ctypes.data_as(fp),
                                      n_v4, ss.ctypes.data_as(fp), dd.ctypes.data_as(fp), C.byref(found)))
    if not found.value:
        return None
    return float(cut.value), v2, ss, dd


def write_correlation(path: str, lattice: Lattice, cutoff: float, zz, dd) -> bool:
    """Adds one correlation measurement (SU2CorZZ and SU2CorDD) to an observable file;
    False if the file already holds one at this cutoff."""
    lib = load_library()
    zz, dd = _f32(zz), _f32(dd)
    n = lattice.info.n_basis * lattice.info.n_range
    if zz.size != n or dd.size != n:
        raise ValueError(f"correlations must hold n_basis * n_range = {n} values")
    fp = C.POINTER(C.c_float)
    out = C.c_int()
    check(lib.spn_su2_write_correlation(str(path).encode(), lattice._h, float(cutoff), zz.ctypes.data_as(fp),
                                        dd.ctypes.data_as(fp), C.byref(out)))
    return bool(out.value)
