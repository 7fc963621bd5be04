"""One TRI-core flow resident on a GPU: time-reversal-invariant models with general, also
off-diagonal, couplings (Heisenberg-Kitaev-Gamma, ...).  Mirrors TRIFrgCore +
TRIEffectiveAction + TRIMeasurementCorrelation (src/TRI/*) over the spn_tri_* C ABI, with the
same cycle as ``Su2Flow``: compute_step, measure, finalize_step.

The vertex is one array v4[F_N][16][Nl] in the reference's layout (component 4a + b for the
spin components a, b in X, Y, Z, density), the checkpoint dataset "v4".
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import XyzDesc, check, load_library
from .core import Lattice, LatticeTables, SpinTables, _ptr

# correlation groups in the order of spn_tri_measure_correlation (TRICorXX ... TRICorDD)
TRI_COMPONENTS = ("xx", "xy", "xz", "yx", "yy", "yz", "zx", "zy", "zz", "dd")


def tri_initial_state(lattice: Lattice, n_freq: int, normalization: float = 1.0):
    """TRIEffectiveAction initial condition: (v2[N], v4[F_N*16*Nl])."""
    lib = load_library()
    nl = lattice.info.n_sites
    fn = n_freq * n_freq * (n_freq + 1) // 2
    v2 = np.empty(n_freq, np.float32)
    v4 = np.empty(fn * 16 * nl, np.float32)
    check(lib.spn_tri_initial_state(lattice._h, n_freq, normalization, _ptr(v2, C.c_float), _ptr(v4, C.c_float)))
    return v2, v4


def tri_tables() -> np.ndarray:
    """The coefficient tables the TRI kernels evaluate: rows (table, output, n, a, b, sign)."""
    rows = np.zeros(16 * 72 * 6, np.int32)  # 72 rows per output component
    check(load_library().spn_tri_tables(_ptr(rows, C.c_int)))
    return rows.reshape(-1, 6)


class TriFlow:
    """One TRI flow on a GPU."""

    def __init__(self, tables: LatticeTables, spin: SpinTables, freq: np.ndarray, device: int = 0):
        lib = load_library()
        self._lib = lib
        self.freq = np.ascontiguousarray(freq, np.float32)
        self.n = len(self.freq)
        self.nl = int(tables.n_sites)
        self.fn = self.n * self.n * (self.n + 1) // 2
        self.size = self.fn * 16 * self.nl
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
        check(lib.spn_tri_create(C.byref(d), C.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.spn_tri_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def set_state(self, cutoff: float, v2: np.ndarray, v4: np.ndarray) -> None:
        v2 = np.ascontiguousarray(v2, np.float32)
        v4 = np.ascontiguousarray(v4, np.float32).reshape(-1)
        if v2.size != self.n or v4.size != self.size:
            raise ValueError("state arrays have the wrong size")
        check(self._lib.spn_tri_set_state(self._h, cutoff, _ptr(v2, C.c_float), _ptr(v4, C.c_float)))

    def get_state(self):
        v2 = np.empty(self.n, np.float32)
        v4 = np.empty(self.size, np.float32)
        c = C.c_float()
        check(self._lib.spn_tri_get_state(self._h, C.byref(c), _ptr(v2, C.c_float), _ptr(v4, C.c_float)))
        return c.value, v2, v4

    def compute_step(self) -> None:
        check(self._lib.spn_tri_compute_step(self._h))

    def get_flow(self):
        v2 = np.empty(self.n, np.float32)
        v4 = np.empty(self.size, np.float32)
        check(self._lib.spn_tri_get_flow(self._h, _ptr(v2, C.c_float), _ptr(v4, C.c_float)))
        return v2, v4

    def finalize_step(self, new_cutoff: float) -> None:
        check(self._lib.spn_tri_finalize_step(self._h, new_cutoff))

    def measure_correlation(self):
        """(corr[10, n_corr] in TRI_COMPONENTS order, chi[16, Nl])."""
        corr = np.empty((10, self.n_corr), np.float32)
        chi = np.empty((16, self.nl), np.float32)
        check(self._lib.spn_tri_measure_correlation(self._h, _ptr(corr, C.c_float), _ptr(chi, C.c_float)))
        return corr, chi

    def is_diverged(self) -> bool:
        v = C.c_int(0)
        check(self._lib.spn_tri_is_diverged(self._h, C.byref(v)))
        return bool(v.value)

    def run(self, cutoffs, v2, v4):
        """The whole flow as SpinParser's loop runs it: measure at every cutoff, then step;
        stops at a divergence.  Returns (cutoffs measured, corr[k, 10, n_corr], diverged)."""
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
