"""One XYZ-core flow resident on a GPU: models with diagonal, possibly anisotropic couplings
(Heisenberg-Kitaev, XXZ, ...).  Mirrors XYZFrgCore + XYZEffectiveAction +
XYZMeasurementCorrelation (src/XYZ/*) over the spn_xyz_* C ABI, with the same cycle as
``Su2Flow``: compute_step, measure, finalize_step.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import XyzDesc, check, load_library
from .core import Lattice, LatticeTables, SpinTables, _ptr

COMPONENTS = ("xx", "yy", "zz", "dd")


def xyz_initial_state(lattice: Lattice, n_freq: int, normalization: float = 1.0):
    """XYZEffectiveAction initial condition: (v2[N], v4[4, F_N*Nl]) with components x, y, z, d."""
    lib = load_library()
    nl = lattice.info.n_sites
    fn = n_freq * n_freq * (n_freq + 1) // 2
    v2 = np.empty(n_freq, np.float32)
    v4 = np.empty((4, fn * nl), np.float32)
    check(lib.spn_xyz_initial_state(lattice._h, n_freq, normalization, _ptr(v2, C.c_float),
                                    *[_ptr(v4[c], C.c_float) for c in range(4)]))
    return v2, v4


class XyzFlow:
    """One XYZ flow on a GPU."""

    def __init__(self, tables: LatticeTables, spin: SpinTables, freq: np.ndarray, device: int = 0):
        lib = load_library()
        self._lib = lib
        self.freq = np.ascontiguousarray(freq, np.float32)
        self.n = len(self.freq)
        self.nl = int(tables.n_sites)
        self.fn = self.n * self.n * (self.n + 1) // 2
        arrs = [tables.sites_rid, spin.sites_perm, tables.inv_sites_rid, spin.inv_sites_perm, tables.overlap_ptr,
                tables.overlap_rid1, tables.overlap_rid2, spin.overlap_perm1, spin.overlap_perm2, tables.range_rid,
                tables.range_inv_rid, tables.corr_rid, spin.corr_perm]
        self._keep = [np.ascontiguousarray(a, np.int32) for a in arrs]
        k = [_ptr(a, C.c_int) for a in self._keep]
        d = XyzDesc()
        d.n_freq, d.freq, d.n_sites = self.n, _ptr(self.freq, C.c_float), self.nl
        (d.sites_rid, d.sites_perm, d.inv_sites_rid, d.inv_sites_perm, d.overlap_ptr, d.overlap_rid1, d.overlap_rid2,
         d.overlap_perm1, d.overlap_perm2) = k[:9]
        d.n_range, d.range_rid, d.range_inv_rid = len(self._keep[9]), k[9], k[10]
        d.n_corr, d.corr_rid, d.corr_perm = len(self._keep[11]), k[11], k[12]
        d.device, d.flags = device, 0
        self.n_corr = d.n_corr
        h = C.c_void_p()
        check(lib.spn_xyz_create(C.byref(d), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.spn_xyz_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_state(self, cutoff: float, v2: np.ndarray, v4: np.ndarray) -> None:
        """v2[N] and v4[4, F_N*Nl] (x, y, z, d) in the reference layout."""
        v2 = np.ascontiguousarray(v2, np.float32)
        v4 = np.ascontiguousarray(v4, np.float32).reshape(4, -1)
        if v2.size != self.n or v4.shape[1] != self.fn * self.nl:
            raise ValueError("state arrays have the wrong size")
        check(self._lib.spn_xyz_set_state(self._h, cutoff, _ptr(v2, C.c_float),
                                          *[_ptr(v4[c], C.c_float) for c in range(4)]))

    def get_state(self):
        v2 = np.empty(self.n, np.float32)
        v4 = np.empty((4, self.fn * self.nl), np.float32)
        c = C.c_float()
        check(self._lib.spn_xyz_get_state(self._h, C.byref(c), _ptr(v2, C.c_float),
                                          *[_ptr(v4[q], C.c_float) for q in range(4)]))
        return c.value, v2, v4

    def compute_step(self) -> None:
        check(self._lib.spn_xyz_compute_step(self._h))

    def get_flow(self):
        v2 = np.empty(self.n, np.float32)
        v4 = np.empty((4, self.fn * self.nl), np.float32)
        check(self._lib.spn_xyz_get_flow(self._h, _ptr(v2, C.c_float), *[_ptr(v4[q], C.c_float) for q in range(4)]))
        return v2, v4

    def finalize_step(self, new_cutoff: float) -> None:
        check(self._lib.spn_xyz_finalize_step(self._h, new_cutoff))

    def measure_correlation(self):
        """(corr[4, n_corr] in the XYZCorXX/YY/ZZ/DD entry order, chi[4, Nl])."""
        corr = np.empty((4, self.n_corr), np.float32)
        chi = np.empty((4, self.nl), np.float32)
        check(self._lib.spn_xyz_measure_correlation(self._h, *[_ptr(corr[q], C.c_float) for q in range(4)],
                                                    _ptr(chi, C.c_float)))
        return corr, chi

    def is_diverged(self) -> bool:
        v = C.c_int(0)
        check(self._lib.spn_xyz_is_diverged(self._h, C.byref(v)))
        return bool(v.value)

    def run(self, cutoffs, v2, v4):
        """The whole flow as SpinParser's loop runs it: measure at every cutoff, then step;
        stops at a divergence.  Returns (cutoffs measured, corr[k, 4, n_corr], diverged)."""
        self.set_state(float(cutoffs[0]), v2, v4)
        out, measured = [], []
        diverged = False
        for k in range(len(cutoffs)):
            corr, _ = self.measure_correlation()
            out.append(corr)
            measured.append(float(cutoffs[k]))
            if k + 1 == len(cutoffs):
                break
            self.compute_step()
            if self.is_diverged():
                diverged = True
                break
            self.finalize_step(float(cutoffs[k + 1]))
        return np.array(measured, np.float32), np.stack(out), diverged
