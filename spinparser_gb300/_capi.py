"""ctypes binding of include/spn_su2.h (libspn_su2.so).

This is the same binding a Python host of the reference-facing C ABI would write; the
package's Python classes and the tests call the library only through it.  Loading fails
loudly when the library has not been built: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

c_int_p = C.POINTER(C.c_int)
c_float_p = C.POINTER(C.c_float)
c_double_p = C.POINTER(C.c_double)
c_ll_p = C.POINTER(C.c_longlong)


class LatticeInfo(C.Structure):
    _fields_ = [
        ("n_sites", C.c_int),
        ("n_sites_total", C.c_int),
        ("n_basis", C.c_int),
        ("n_range", C.c_int),
        ("n_overlap", C.c_int),
        ("n_interactions", C.c_int),
    ]


class XyzDesc(C.Structure):
    _fields_ = [
        ("n_freq", C.c_int), ("freq", c_float_p), ("n_sites", C.c_int),
        ("sites_rid", c_int_p), ("sites_perm", c_int_p), ("inv_sites_rid", c_int_p), ("inv_sites_perm", c_int_p),
        ("overlap_ptr", c_int_p), ("overlap_rid1", c_int_p), ("overlap_rid2", c_int_p), ("overlap_perm1", c_int_p),
        ("overlap_perm2", c_int_p), ("n_range", C.c_int), ("range_rid", c_int_p), ("range_inv_rid", c_int_p),
        ("n_corr", C.c_int), ("corr_rid", c_int_p), ("corr_perm", c_int_p), ("device", C.c_int), ("flags", C.c_int),
    ]


class Su2Desc(C.Structure):
    _fields_ = [
        ("n_freq", C.c_int),
        ("freq", c_float_p),
        ("n_sites", C.c_int),
        ("sites_rid", c_int_p),
        ("inv_sites_rid", c_int_p),
        ("overlap_ptr", c_int_p),
        ("overlap_rid1", c_int_p),
        ("overlap_rid2", c_int_p),
        ("n_range", C.c_int),
        ("range_rid", c_int_p),
        ("range_inv_rid", c_int_p),
        ("n_corr", C.c_int),
        ("corr_rid", c_int_p),
        ("spin_length", C.c_float),
        ("device", C.c_int),
        ("flags", C.c_int),
    ]


class RunOptions(C.Structure):
    _fields_ = [
        ("resource_path", C.c_char_p),
        ("checkpoint_time", C.c_int),
        ("force_restart", C.c_int),
        ("defer", C.c_int),
        ("debug_lattice", C.c_int),
        ("verbose", C.c_int),
        ("device", C.c_int),
        ("flags", C.c_int),
        ("autotune", C.c_int),
    ]


class RunResult(C.Structure):
    _fields_ = [
        ("status", C.c_int),
        ("steps", C.c_int),
        ("measurements", C.c_int),
        ("diverged", C.c_int),
        ("flow_seconds", C.c_double),
    ]


# name -> (restype, argtypes); every function declared in include/spn_su2.h
SIGNATURES = {
    "spn_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "spn_device_count": (C.c_int, [c_int_p]),
    "spn_device_memory": (C.c_int, [C.c_int, c_ll_p, c_ll_p]),
    "spn_measure_fp32_peak": (C.c_int, [C.c_int, c_double_p, c_double_p]),
    "spn_measure_gather_peak": (C.c_int, [C.c_int, C.c_int, C.c_int, c_double_p]),
    "spn_mesh_probe": (C.c_int, [c_float_p, C.c_int, C.c_float, c_float_p, c_float_p, c_int_p, c_int_p, c_int_p,
                                 c_float_p]),
    "spn_quadrature_nodes": (C.c_int, [c_float_p, C.c_int, C.c_int, C.c_float, C.c_float, c_float_p, c_double_p,
                                       C.c_int, c_int_p]),
    "spn_mesh_index_check": (C.c_int, [c_float_p, C.c_int, c_float_p, C.c_int, c_int_p]),
    "spn_self_energy_probe": (C.c_int, [c_float_p, C.c_int, c_float_p, C.c_float, c_double_p]),
    "spn_vertex_probe": (C.c_int, [c_float_p, C.c_int, C.c_int, c_float_p, c_float_p, C.c_int, C.c_int, C.c_float,
                                   C.c_float, C.c_float, C.c_int, C.c_int, c_float_p]),
    "spn_xyz_vertex_probe": (C.c_int, [c_float_p, C.c_int, C.c_int, c_float_p, c_float_p, c_float_p, c_float_p,
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                                       C.c_int, c_float_p]),
    "spn_tri_vertex_probe": (C.c_int, [c_float_p, C.c_int, C.c_int, c_float_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, c_float_p]),
    "spn_lattice_create": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p, C.c_int,
                                     C.POINTER(C.c_char_p), C.POINTER(C.c_char_p), C.POINTER(C.c_void_p)]),
    "spn_lattice_destroy": (C.c_int, [C.c_void_p]),
    "spn_lattice_get_info": (C.c_int, [C.c_void_p, C.POINTER(LatticeInfo)]),
    "spn_lattice_get_tables": (C.c_int, [C.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p,
                                         c_int_p, c_double_p, c_double_p, c_double_p]),
    "spn_lattice_get_sites": (C.c_int, [C.c_void_p, c_int_p, c_int_p]),
    "spn_lattice_get_interactions": (C.c_int, [C.c_void_p, c_int_p, c_float_p]),
    "spn_lattice_write_ldf": (C.c_int, [C.c_void_p, C.c_char_p]),
    "spn_lattice_get_spin_tables": (C.c_int, [C.c_void_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p,
                                              c_int_p]),
    "spn_rpa_schedule": (C.c_int, [C.c_int, c_int_p, c_int_p, c_int_p, C.c_int, c_int_p, c_int_p, c_int_p, c_int_p,
                                   c_int_p]),
    "spn_rpa_lane_schedule": (C.c_int, [C.c_int, C.c_int, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p,
                                        c_int_p]),
    "spn_frequency_exponential": (C.c_int, [C.c_float, C.c_float, C.c_int, c_float_p]),
    "spn_parse_number": (C.c_int, [C.c_char_p, c_double_p]),
    "spn_cutoff_exponential": (C.c_int, [C.c_float, C.c_float, C.c_float, c_float_p, C.c_int, c_int_p]),
    "spn_su2_initial_state": (C.c_int, [C.c_void_p, C.c_int, C.c_float, c_float_p, c_float_p, c_float_p]),
    "spn_su2_create": (C.c_int, [C.POINTER(Su2Desc), C.POINTER(C.c_void_p)]),
    "spn_su2_destroy": (C.c_int, [C.c_void_p]),
    "spn_su2_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "spn_su2_get_sizes": (C.c_int, [C.c_void_p, c_int_p, c_int_p, c_ll_p]),
    "spn_su2_set_state": (C.c_int, [C.c_void_p, C.c_float, c_float_p, c_float_p, c_float_p]),
    "spn_su2_get_state": (C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p, c_float_p]),
    "spn_su2_set_cutoff": (C.c_int, [C.c_void_p, C.c_float]),
    "spn_su2_get_node_counts": (C.c_int, [C.c_void_p, c_int_p]),
    "spn_su2_compute_step": (C.c_int, [C.c_void_p]),
    "spn_su2_autotune": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_int_p, c_int_p]),
    "spn_su2_set_variant": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "spn_su2_get_flow": (C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p]),
    "spn_su2_finalize_step": (C.c_int, [C.c_void_p, C.c_float]),
    "spn_su2_measure_correlation": (C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p, c_float_p]),
    "spn_su2_launch_correlation": (C.c_int, [C.c_void_p]),
    "spn_xyz_initial_state": (C.c_int, [C.c_void_p, C.c_int, C.c_float, c_float_p, c_float_p, c_float_p, c_float_p,
                                        c_float_p]),
    "spn_xyz_create": (C.c_int, [C.POINTER(XyzDesc), C.POINTER(C.c_void_p)]),
    "spn_xyz_destroy": (C.c_int, [C.c_void_p]),
    "spn_xyz_set_state": (C.c_int, [C.c_void_p, C.c_float, c_float_p, c_float_p, c_float_p, c_float_p, c_float_p]),
    "spn_xyz_get_state": (C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p, c_float_p, c_float_p, c_float_p]),
    "spn_xyz_compute_step": (C.c_int, [C.c_void_p]),
    "spn_xyz_get_flow": (C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p, c_float_p, c_float_p]),
    "spn_xyz_finalize_step": (C.c_int, [C.c_void_p, C.c_float]),
    "spn_xyz_measure_correlation": (C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p, c_float_p, c_float_p]),
    "spn_xyz_is_diverged": (C.c_int, [C.c_void_p, c_int_p]),
    "spn_tri_initial_state": (C.c_int, [C.c_void_p, C.c_int, C.c_float, c_float_p, c_float_p]),
    "spn_tri_create": (C.c_int, [C.POINTER(XyzDesc), C.POINTER(C.c_void_p)]),
    "spn_tri_destroy": (C.c_int, [C.c_void_p]),
    "spn_tri_set_state": (C.c_int, [C.c_void_p, C.c_float, c_float_p, c_float_p]),
    "spn_tri_get_state": (C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p]),
    "spn_tri_compute_step": (C.c_int, [C.c_void_p]),
    "spn_tri_get_flow": (C.c_int, [C.c_void_p, c_float_p, c_float_p]),
    "spn_tri_finalize_step": (C.c_int, [C.c_void_p, C.c_float]),
    "spn_tri_measure_correlation": (C.c_int, [C.c_void_p, c_float_p, c_float_p]),
    "spn_tri_is_diverged": (C.c_int, [C.c_void_p, c_int_p]),
    "spn_tri_tables": (C.c_int, [c_int_p]),
    "spn_rpa_pair_order": (C.c_int, [C.c_int, C.c_int, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p, c_int_p,
                                     C.POINTER(C.c_longlong)]),
    "spn_su2_set_state_f64": (C.c_int, [C.c_void_p, C.c_float, c_double_p, c_double_p, c_double_p]),
    "spn_su2_get_state_f64": (C.c_int, [C.c_void_p, c_float_p, c_double_p, c_double_p, c_double_p]),
    "spn_su2_get_flow_f64": (C.c_int, [C.c_void_p, c_double_p, c_double_p, c_double_p]),
    "spn_su2_measure_correlation_f64": (C.c_int, [C.c_void_p, c_double_p, c_double_p, c_double_p, c_double_p]),
    "spn_su2_get_correlation": (C.c_int, [C.c_void_p, c_float_p, c_float_p, c_float_p, c_float_p]),
    "spn_su2_correlation_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                              C.c_void_p, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p]),
    "spn_su2_is_diverged": (C.c_int, [C.c_void_p, c_int_p]),
    "spn_su2_synchronize": (C.c_int, [C.c_void_p]),
    "spn_su2_set_profiling": (C.c_int, [C.c_void_p, C.c_int]),
    "spn_su2_get_profile": (C.c_int, [C.c_void_p, c_double_p, c_int_p, c_double_p, c_int_p]),
    "spn_batch_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "spn_batch_destroy": (C.c_int, [C.c_void_p]),
    "spn_batch_set_variant": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "spn_batch_set_grouping": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "spn_batch_grouped_flows": (C.c_int, [C.c_void_p, c_int_p]),
    "spn_batch_set_paused": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "spn_batch_autotune": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_int_p, c_int_p, c_float_p]),
    "spn_batch_footprint": (C.c_int, [C.POINTER(Su2Desc), C.c_int, c_ll_p]),
    "spn_batch_add": (C.c_int, [C.c_void_p, C.POINTER(Su2Desc), C.c_int, c_float_p, c_float_p, c_float_p, c_float_p,
                                c_int_p]),
    "spn_batch_step": (C.c_int, [C.c_void_p, c_int_p]),
    "spn_batch_synchronize": (C.c_int, [C.c_void_p]),
    "spn_batch_poll": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_int_p, c_int_p]),
    "spn_batch_get_result": (C.c_int, [C.c_void_p, C.c_int, c_int_p, c_float_p, c_float_p, c_float_p, c_float_p,
                                       c_float_p]),
    "spn_batch_get_state": (C.c_int, [C.c_void_p, C.c_int, c_float_p, c_float_p, c_float_p, c_float_p]),
    "spn_batch_remove": (C.c_int, [C.c_void_p, C.c_int]),
    "spn_batch_stats": (C.c_int, [C.c_void_p, c_ll_p, c_ll_p, c_int_p]),
    "spn_su2_write_checkpoint": (C.c_int, [C.c_char_p, C.c_int, C.c_float, C.c_int, c_float_p, C.c_longlong,
                                           c_float_p, c_float_p, c_int_p]),
    "spn_su2_read_checkpoint": (C.c_int, [C.c_char_p, C.c_int, c_float_p, C.c_int, c_float_p, C.c_longlong,
                                          c_float_p, c_float_p, c_int_p]),
    "spn_su2_write_correlation": (C.c_int, [C.c_char_p, C.c_void_p, C.c_float, c_float_p, c_float_p, c_int_p]),
    "spn_run_options_default": (C.c_int, [C.POINTER(RunOptions)]),
    "spn_run_task": (C.c_int, [C.c_char_p, C.POINTER(RunOptions), C.POINTER(RunResult)]),
}


class SpnError(RuntimeError):
    """A negative status returned by libspn_su2, with the library's message."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


_LIB = None


def load_library() -> C.CDLL:
    """Loads the in-tree libspn_su2.so; raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.library_path()
    if not os.path.exists(path):
        raise RuntimeError(f"libspn_su2.so is not built ({path}); run __graft_entry__.build() first")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int) -> None:
    if status != 0:
        lib = load_library()
        buf = C.create_string_buffer(4096)
        lib.spn_last_error(buf, len(buf))
        raise SpnError(status, buf.value.decode(errors="replace"))
