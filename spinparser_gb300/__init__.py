"""GB300-native SU(2) pf-FRG flow core (SpinParser's SU2 hot path) behind a C ABI.

Compute runs in libspn_su2.so (hand-written CUDA for sm_103a); this package is the Python
host layer over that ABI.  Build with ``__graft_entry__.build()`` (or ``python -m
spinparser_gb300._build``).
"""
from ._capi import SpnError, load_library
from .batch import Su2Batch
from .core import (FP64, FP64_SELF_ENERGY, RES_DIR, Lattice, LatticeTables, SpinTables, Su2Flow, cutoff_exponential,
                   device_count, frequency_exponential, measure_fp32_peak, measure_gather_peak)
from .xyz import XyzFlow, xyz_initial_state
from .tri import TRI_COMPONENTS, TriFlow, tri_initial_state, tri_tables

__all__ = [
    "SpnError", "load_library", "Lattice", "LatticeTables", "Su2Flow", "frequency_exponential", "cutoff_exponential",
    "device_count", "measure_fp32_peak", "measure_gather_peak", "RES_DIR", "FP64", "FP64_SELF_ENERGY", "Su2Batch", "SpinTables", "XyzFlow",
    "xyz_initial_state", "TriFlow", "tri_initial_state", "tri_tables", "TRI_COMPONENTS",
]
