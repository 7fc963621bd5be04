"""Python host layer over the C ABI: lattice construction, discretisations and one SU(2) flow.

The classes mirror the reference's objects for this path:
  * ``Lattice``  — LatticeModelFactory::newLatticeModel product (src/LatticeModelFactory.cpp:733)
  * ``Su2Flow``  — SU2FrgCore + SU2EffectiveAction + SU2MeasurementCorrelation with the state
                   resident on the GPU (src/SU2/SU2FrgCore.cpp, SU2EffectiveAction.hpp,
                   SU2MeasurementCorrelation.cpp)
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from ._capi import LatticeInfo, Su2Desc, check, load_library

RES_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "res")

FP64_SELF_ENERGY = 0x1
FP64 = 0x2  # the whole flow in double precision (precision reference; plain FP64 kernel)


def _ptr(a: np.ndarray | None, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def frequency_exponential(fmin: float, fmax: float, count: int) -> np.ndarray:
    """Exponential Matsubara mesh exactly as TaskFileParser builds it (src/TaskFileParser.cpp:121-123)."""
    out = np.empty(count, dtype=np.float32)
    check(load_library().spn_frequency_exponential(fmin, fmax, count, _ptr(out, C.c_float)))
    return out


def cutoff_exponential(cmax: float, cmin: float, step: float) -> np.ndarray:
    """Cutoff list by repeated float multiplication (src/TaskFileParser.cpp:171-176)."""
    lib = load_library()
    n = C.c_int(0)
    check(lib.spn_cutoff_exponential(cmax, cmin, step, None, 0, C.byref(n)))
    out = np.empty(n.value, dtype=np.float32)
    check(lib.spn_cutoff_exponential(cmax, cmin, step, _ptr(out, C.c_float), n.value, C.byref(n)))
    return out


@dataclass
class LatticeTables:
    n_sites: int
    n_basis: int
    n_range: int
    sites_rid: np.ndarray
    inv_sites_rid: np.ndarray
    overlap_ptr: np.ndarray
    overlap_rid1: np.ndarray
    overlap_rid2: np.ndarray
    range_rid: np.ndarray
    range_inv_rid: np.ndarray
    corr_rid: np.ndarray
    site_pos: np.ndarray      # [n_basis, n_range, 3]
    basis_pos: np.ndarray     # [n_basis, 3]
    lattice_vectors: np.ndarray  # [3, 3]
    interaction_rid: np.ndarray
    interaction_J: np.ndarray  # [n_interactions, 3, 3]

    @property
    def n_overlap(self) -> int:
        return int(self.overlap_ptr[-1])

    def to_npz(self, path: str) -> None:
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in self.__dict__.items()})

    @classmethod
    def from_npz(cls, path: str) -> "LatticeTables":
        z = np.load(path)
        kw = {}
        for k in cls.__dataclass_fields__:
            v = z[k]
            kw[k] = int(v) if v.ndim == 0 else v
        return cls(**kw)

    def initial_state(self, n_freq: int, normalization: float = 1.0):
        """SU2EffectiveAction initial condition (src/SU2/SU2EffectiveAction.hpp:38-60)."""
        fn = n_freq * n_freq * (n_freq + 1) // 2
        v2 = np.zeros(n_freq, np.float32)
        ss = np.zeros((fn, self.n_sites), np.float32)
        dd = np.zeros((fn, self.n_sites), np.float32)
        for rid, J in zip(self.interaction_rid, self.interaction_J):
            ss[:, rid] += np.float32(J[0, 0]) / np.float32(normalization)
        return v2, ss.reshape(-1), dd.reshape(-1)


# The six spin-component permutations of the lattice tables (index -> images of X, Y, Z).
SPIN_PERMUTATIONS = np.array([[0, 1, 2], [0, 2, 1], [1, 0, 2], [1, 2, 0], [2, 0, 1], [2, 1, 0]], np.int32)


@dataclass
class SpinTables:
    """Spin permutations that accompany the symmetry maps of a lattice (indices into
    SPIN_PERMUTATIONS), parallel to the LatticeTables arrays of the same names."""
    sites_perm: np.ndarray
    inv_sites_perm: np.ndarray
    overlap_perm1: np.ndarray
    overlap_perm2: np.ndarray
    range_perm: np.ndarray
    range_inv_perm: np.ndarray
    corr_perm: np.ndarray

    def to_npz(self, path: str) -> None:
        np.savez_compressed(path, **{k: np.asarray(v) for k, v in self.__dict__.items()})

    @classmethod
    def from_npz(cls, path: str) -> "SpinTables":
        z = np.load(path)
        return cls(**{k: z[k] for k in cls.__dataclass_fields__})


class Lattice:
    """Symmetry-reduced lattice + spin model built by the library's host factory."""

    def __init__(self, lattice: str, lattice_range: int, model: str, params: dict[str, str | float],
                 resource_dir: str | None = None):
        lib = load_library()
        names = [k.encode() for k in params]
        values = [str(v).encode() for v in params.values()]
        arr_n = (C.c_char_p * max(1, len(names)))(*names)
        arr_v = (C.c_char_p * max(1, len(values)))(*values)
        h = C.c_void_p()
        check(lib.spn_lattice_create((resource_dir or RES_DIR).encode(), lattice.encode(), lattice_range, model.encode(),
                                     len(names), arr_n, arr_v, C.byref(h)))
        self._h = h
        self._lib = lib
        info = LatticeInfo()
        check(lib.spn_lattice_get_info(h, C.byref(info)))
        self.info = info

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.spn_lattice_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def tables(self) -> LatticeTables:
        i = self.info
        nl, nr, nb, no = i.n_sites, i.n_range, i.n_basis, i.n_overlap
        sites = np.empty(nl, np.int32)
        inv = np.empty(nl, np.int32)
        optr = np.empty(nl + 1, np.int32)
        r1 = np.empty(max(no, 1), np.int32)
        r2 = np.empty(max(no, 1), np.int32)
        rr = np.empty(nr, np.int32)
        ri = np.empty(nr, np.int32)
        corr = np.empty(nb * nr, np.int32)
        spos = np.empty((nb, nr, 3), np.float64)
        bpos = np.empty((nb, 3), np.float64)
        lv = np.empty((3, 3), np.float64)
        I = C.c_int
        check(self._lib.spn_lattice_get_tables(self._h, _ptr(sites, I), _ptr(inv, I), _ptr(optr, I), _ptr(r1, I),
                                               _ptr(r2, I), _ptr(rr, I), _ptr(ri, I), _ptr(corr, I),
                                               _ptr(spos, C.c_double), _ptr(bpos, C.c_double), _ptr(lv, C.c_double)))
        ni = i.n_interactions
        irid = np.empty(max(ni, 1), np.int32)
        iJ = np.empty((max(ni, 1), 3, 3), np.float32)
        check(self._lib.spn_lattice_get_interactions(self._h, _ptr(irid, I), _ptr(iJ, C.c_float)))
        return LatticeTables(nl, nb, nr, sites, inv, optr, r1[:no], r2[:no], rr, ri, corr, spos, bpos, lv,
                             irid[:ni], iJ[:ni])

    def spin_tables(self) -> SpinTables:
        i = self.info
        nl, nr, nb, no = i.n_sites, i.n_range, i.n_basis, i.n_overlap
        a = [np.empty(nl, np.int32), np.empty(nl, np.int32), np.empty(max(no, 1), np.int32),
             np.empty(max(no, 1), np.int32), np.empty(nr, np.int32), np.empty(nr, np.int32),
             np.empty(nb * nr, np.int32)]
        check(self._lib.spn_lattice_get_spin_tables(self._h, *[_ptr(x, C.c_int) for x in a]))
        return SpinTables(a[0], a[1], a[2][:no], a[3][:no], a[4], a[5], a[6])

    def sites(self, with_pairs: bool = False):
        """(site_params[n_total, 4], pair_rid[n_total, n_total] or None)."""
        n = self.info.n_sites_total
        sp = np.empty((n, 4), np.int32)
        pr = np.empty((n, n), np.int32) if with_pairs else None
        check(self._lib.spn_lattice_get_sites(self._h, _ptr(sp, C.c_int), _ptr(pr, C.c_int)))
        return sp, pr

    def write_ldf(self, path: str) -> None:
        check(self._lib.spn_lattice_write_ldf(self._h, path.encode()))


def device_count() -> int:
    n = C.c_int(0)
    check(load_library().spn_device_count(C.byref(n)))
    return n.value


def measure_fp32_peak(device: int = 0):
    """(TFLOP/s, implied SM clock GHz) of a pure-FFMA kernel on `device`."""
    t, g = C.c_double(), C.c_double()
    check(load_library().spn_measure_fp32_peak(device, C.byref(t), C.byref(g)))
    return t.value, g.value


def measure_gather_peak(n_sites: int, n_slabs: int, device: int = 0) -> float:
    """Segments of n_sites float2 pairs per second that a pure gather kernel reads at random
    starts among n_slabs slabs (spn_measure_gather_peak)."""
    r = C.c_double()
    check(load_library().spn_measure_gather_peak(device, n_sites, n_slabs, C.byref(r)))
    return r.value


def make_desc(tables: LatticeTables, freq: np.ndarray, spin_length: float = 0.5, device: int = 0, flags: int = 0):
    """The spn_su2_desc of a flow, and the arrays it points into (keep them alive while the
    descriptor is used)."""
    freq = np.ascontiguousarray(freq, dtype=np.float32)
    keep = [freq] + [np.ascontiguousarray(x, dtype=np.int32) for x in
                     (tables.sites_rid, tables.inv_sites_rid, tables.overlap_ptr, tables.overlap_rid1,
                      tables.overlap_rid2, tables.range_rid, tables.range_inv_rid, tables.corr_rid)]
    k = keep[1:]
    d = Su2Desc()
    d.n_freq = len(freq)
    d.freq = _ptr(freq, C.c_float)
    d.n_sites = tables.n_sites
    d.sites_rid, d.inv_sites_rid, d.overlap_ptr = _ptr(k[0], C.c_int), _ptr(k[1], C.c_int), _ptr(k[2], C.c_int)
    d.overlap_rid1, d.overlap_rid2 = _ptr(k[3], C.c_int), _ptr(k[4], C.c_int)
    d.n_range = len(k[5])
    d.range_rid, d.range_inv_rid = _ptr(k[5], C.c_int), _ptr(k[6], C.c_int)
    d.n_corr = len(k[7])
    d.corr_rid = _ptr(k[7], C.c_int)
    d.spin_length = spin_length
    d.device = device
    d.flags = flags
    return d, keep


class Su2Flow:
    """One SU(2) flow resident on a GPU: the FrgCore::computeStep / finalizeStep cycle."""

    def __init__(self, tables: LatticeTables, freq: np.ndarray, spin_length: float = 0.5, device: int = 0,
                 flags: int = 0):
        lib = load_library()
        self._lib = lib
        self.tables = tables
        self.freq = np.ascontiguousarray(freq, dtype=np.float32)
        self.n = len(self.freq)
        self.nl = tables.n_sites
        self.fn = self.n * self.n * (self.n + 1) // 2
        d, self._keep = make_desc(tables, self.freq, spin_length, device, flags)
        h = C.c_void_p()
        check(lib.spn_su2_create(C.byref(d), C.byref(h)))
        self._h = h
        self.n_corr = d.n_corr
        self.fp64 = bool(flags & FP64)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.spn_su2_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_stream(self, stream_handle: int | None) -> None:
        check(self._lib.spn_su2_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None))

    def set_state(self, cutoff: float, v2: np.ndarray, v4ss: np.ndarray, v4dd: np.ndarray) -> None:
        v2 = np.ascontiguousarray(v2, np.float32)
        v4ss = np.ascontiguousarray(v4ss, np.float32).reshape(-1)
        v4dd = np.ascontiguousarray(v4dd, np.float32).reshape(-1)
        if v2.size != self.n or v4ss.size != self.fn * self.nl or v4dd.size != self.fn * self.nl:
            raise ValueError("state arrays have the wrong size")
        check(self._lib.spn_su2_set_state(self._h, cutoff, _ptr(v2, C.c_float), _ptr(v4ss, C.c_float),
                                          _ptr(v4dd, C.c_float)))

    def get_state(self, v2=None, ss=None, dd=None):
        """(cutoff, v2, v4ss, v4dd); pass preallocated (e.g. pinned) arrays to fill them in place."""
        v2 = np.empty(self.n, np.float32) if v2 is None else v2
        ss = np.empty(self.fn * self.nl, np.float32) if ss is None else ss
        dd = np.empty(self.fn * self.nl, np.float32) if dd is None else dd
        if v2.size != self.n or ss.size != self.fn * self.nl or dd.size != self.fn * self.nl:
            raise ValueError("state arrays have the wrong size")
        c = C.c_float()
        check(self._lib.spn_su2_get_state(self._h, C.byref(c), _ptr(v2, C.c_float), _ptr(ss, C.c_float),
                                          _ptr(dd, C.c_float)))
        return c.value, v2, ss, dd

    def set_cutoff(self, cutoff: float) -> None:
        check(self._lib.spn_su2_set_cutoff(self._h, cutoff))

    def node_counts(self) -> np.ndarray:
        out = np.empty(self.n, np.int32)
        check(self._lib.spn_su2_get_node_counts(self._h, _ptr(out, C.c_int)))
        return out

    def compute_step(self) -> None:
        check(self._lib.spn_su2_compute_step(self._h))

    def autotune(self, reps: int = 3) -> dict:
        """Times the vertex-flow kernel variants on the current state and keeps the fastest."""
        npi, sm, grid = C.c_int(), C.c_int(), C.c_int()
        check(self._lib.spn_su2_autotune(self._h, reps, C.byref(npi), C.byref(sm), C.byref(grid)))
        return {"nodes_per_iteration": npi.value, "schedule_in_smem": bool(sm.value), "grid": grid.value}

    def set_variant(self, nodes_per_iteration: int, schedule_in_smem: bool) -> None:
        """Kernel variant (all variants give identical results)."""
        check(self._lib.spn_su2_set_variant(self._h, nodes_per_iteration, int(schedule_in_smem)))

    def get_flow(self):
        v2 = np.empty(self.n, np.float32)
        ss = np.empty(self.fn * self.nl, np.float32)
        dd = np.empty(self.fn * self.nl, np.float32)
        check(self._lib.spn_su2_get_flow(self._h, _ptr(v2, C.c_float), _ptr(ss, C.c_float), _ptr(dd, C.c_float)))
        return v2, ss, dd

    def finalize_step(self, new_cutoff: float) -> None:
        check(self._lib.spn_su2_finalize_step(self._h, new_cutoff))

    def measure_correlation(self):
        zz = np.empty(self.n_corr, np.float32)
        dd = np.empty(self.n_corr, np.float32)
        cz = np.empty(self.nl, np.float32)
        cd = np.empty(self.nl, np.float32)
        check(self._lib.spn_su2_measure_correlation(self._h, _ptr(zz, C.c_float), _ptr(dd, C.c_float),
                                                    _ptr(cz, C.c_float), _ptr(cd, C.c_float)))
        return zz, dd, cz, cd

    def launch_correlation(self) -> None:
        check(self._lib.spn_su2_launch_correlation(self._h))

    def get_correlation(self, zz=None, dd=None):
        zz = np.empty(self.n_corr, np.float32) if zz is None else zz
        dd = np.empty(self.n_corr, np.float32) if dd is None else dd
        check(self._lib.spn_su2_get_correlation(self._h, _ptr(zz, C.c_float), _ptr(dd, C.c_float), None, None))
        return zz, dd

    # ---- double-precision data of an FP64 flow (flags=FP64) ----
    def set_state_f64(self, cutoff: float, v2: np.ndarray, v4ss: np.ndarray, v4dd: np.ndarray) -> None:
        v2 = np.ascontiguousarray(v2, np.float64)
        v4ss = np.ascontiguousarray(v4ss, np.float64).reshape(-1)
        v4dd = np.ascontiguousarray(v4dd, np.float64).reshape(-1)
        if v2.size != self.n or v4ss.size != self.fn * self.nl or v4dd.size != self.fn * self.nl:
            raise ValueError("state arrays have the wrong size")
        check(self._lib.spn_su2_set_state_f64(self._h, cutoff, _ptr(v2, C.c_double), _ptr(v4ss, C.c_double),
                                              _ptr(v4dd, C.c_double)))

    def get_state_f64(self):
        v2 = np.empty(self.n, np.float64)
        ss = np.empty(self.fn * self.nl, np.float64)
        dd = np.empty(self.fn * self.nl, np.float64)
        c = C.c_float()
        check(self._lib.spn_su2_get_state_f64(self._h, C.byref(c), _ptr(v2, C.c_double), _ptr(ss, C.c_double),
                                              _ptr(dd, C.c_double)))
        return c.value, v2, ss, dd

    def get_flow_f64(self):
        v2 = np.empty(self.n, np.float64)
        ss = np.empty(self.fn * self.nl, np.float64)
        dd = np.empty(self.fn * self.nl, np.float64)
        check(self._lib.spn_su2_get_flow_f64(self._h, _ptr(v2, C.c_double), _ptr(ss, C.c_double),
                                             _ptr(dd, C.c_double)))
        return v2, ss, dd

    def measure_correlation_f64(self):
        zz = np.empty(self.n_corr, np.float64)
        dd = np.empty(self.n_corr, np.float64)
        cz = np.empty(self.nl, np.float64)
        cd = np.empty(self.nl, np.float64)
        check(self._lib.spn_su2_measure_correlation_f64(self._h, _ptr(zz, C.c_double), _ptr(dd, C.c_double),
                                                        _ptr(cz, C.c_double), _ptr(cd, C.c_double)))
        return zz, dd, cz, cd

    def is_diverged(self) -> bool:
        v = C.c_int(0)
        check(self._lib.spn_su2_is_diverged(self._h, C.byref(v)))
        return bool(v.value)

    def synchronize(self) -> None:
        check(self._lib.spn_su2_synchronize(self._h))

    def set_profiling(self, enable: bool) -> None:
        check(self._lib.spn_su2_set_profiling(self._h, int(enable)))

    def profile(self):
        vm, sm = C.c_double(), C.c_double()
        vl, st = C.c_int(), C.c_int()
        check(self._lib.spn_su2_get_profile(self._h, C.byref(vm), C.byref(vl), C.byref(sm), C.byref(st)))
        return {"vertex_ms": vm.value, "vertex_launches": vl.value, "step_ms": sm.value, "steps": st.value}
