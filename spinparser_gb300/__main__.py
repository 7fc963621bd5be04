"""Command line: ``python -m spinparser_gb300 [options] taskFile``.

The options are those of the reference executable (src/CommandLineOptions.cpp:18-42); the
task runs on one GPU (--device), with an optional FP64 self-energy.
"""
from __future__ import annotations

import argparse
import sys

from . import SpnError
from .task import run_task


def main(argv=None) -> int:
    p = argparse.ArgumentParser(prog="spinparser_gb300", description="pf-FRG solver (SU(2) core on the GPU)")
    p.add_argument("taskFile")
    p.add_argument("-r", "--resourcePath", metavar="DIR", help="search path for .xml resource files")
    p.add_argument("-t", "--checkpointTime", type=int, default=3600, metavar="TIME", help="checkpoint interval in seconds")
    p.add_argument("-f", "--forceRestart", action="store_true", help="start new calculation even if checkpoint data is available")
    p.add_argument("-d", "--defer", action="store_true", help="archive all vertex data for deferred measurements in post processing")
    p.add_argument("-v", "--verbose", action="store_true", help="enable verbose output")
    p.add_argument("--debugLattice", action="store_true", help="print lattice debug information in .ldf format")
    p.add_argument("--device", type=int, default=0, help="CUDA device ordinal")
    p.add_argument("--fp64SelfEnergy", action="store_true", help="keep the self-energy and its flow in FP64")
    a = p.parse_args(argv)
    try:
        run_task(a.taskFile, resource_path=a.resourcePath, checkpoint_time=a.checkpointTime,
                 force_restart=a.forceRestart, defer=a.defer, debug_lattice=a.debugLattice,
                 verbose=1 if a.verbose else 0, device=a.device, fp64_self_energy=a.fp64SelfEnergy)
    except SpnError:
        return 1  # the library has logged "Caught exception: ..."
    return 0  # a diverged flow is a result, not an error (as in the reference)


if __name__ == "__main__":
    sys.exit(main())
