"""ORACLE — test infrastructure only (the CPU checker of the GB300 SU(2) flow core).

Python binding of oracle/su2_oracle.cpp, a plain C++ restatement of SpinParser's SU(2) flow
right-hand side, Euler update and correlation measurement.  Imported only by the tests,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg; the product never calls it.
"""
from __future__ import annotations

import ctypes as C
import os
import platform

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))


class OracleDesc(C.Structure):
    _fields_ = [
        ("n_freq", C.c_int), ("freq", C.POINTER(C.c_float)), ("n_sites", C.c_int),
        ("sites_rid", C.POINTER(C.c_int)), ("inv_sites_rid", C.POINTER(C.c_int)),
        ("overlap_ptr", C.POINTER(C.c_int)), ("overlap_rid1", C.POINTER(C.c_int)),
        ("overlap_rid2", C.POINTER(C.c_int)), ("n_range", C.c_int), ("range_rid", C.POINTER(C.c_int)),
        ("range_inv_rid", C.POINTER(C.c_int)), ("spin_length", C.c_float),
    ]


def library_path(timing: bool = False) -> str:
    """The checker build (-O2 -ffp-contract=off) or, with timing=True, the build of the same
    sources with the reference's optimisation flags (-O3, default contraction) that the CPU
    baseline times."""
    name = "liboracle_su2_o3.so" if timing else "liboracle_su2.so"
    return os.path.join(_HERE, "_build", platform.machine(), name)


_LIBS = {}


def _lib(timing: bool = False):
    if timing not in _LIBS:
        path = library_path(timing)
        if not os.path.exists(path):
            raise RuntimeError(f"oracle library not built ({path}); run __graft_entry__.build()")
        lib = C.CDLL(path)
        f, d, i, fp, dp = C.c_float, C.c_double, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_double)
        dsc = C.POINTER(OracleDesc)
        lib.oracle_su2_rhs_f32.argtypes = [dsc, f, fp, fp, fp, fp, fp, fp, i]
        lib.oracle_su2_rhs_f64.argtypes = [dsc, d, dp, dp, dp, dp, dp, dp, i]
        lib.oracle_su2_self_energy_f32.argtypes = [dsc, f, fp, fp, fp, fp]
        lib.oracle_su2_vertex_range_f32.argtypes = [dsc, f, fp, fp, fp, fp, i, i, fp, fp]
        lib.oracle_su2_vertex_range_f64.argtypes = [dsc, d, dp, dp, dp, dp, i, i, dp, dp]
        lib.oracle_su2_vertex_sample_f32.argtypes = [dsc, f, fp, fp, fp, fp, C.POINTER(C.c_int), i, fp, fp, i]
        lib.oracle_su2_correlation_f32.argtypes = [dsc, f, fp, fp, fp, fp, fp]
        lib.oracle_su2_correlation_f64.argtypes = [dsc, d, dp, dp, dp, dp, dp]
        lib.oracle_su2_euler_f32.argtypes = [f, f, C.c_longlong, fp, fp]
        lib.oracle_su2_euler_f32.restype = None
        lib.oracle_su2_flow_f32.argtypes = [dsc, fp, i, fp, fp, fp, fp, fp, i]
        lib.oracle_su2_flow_f64.argtypes = [dsc, fp, i, dp, dp, dp, dp, dp, i]
        _LIBS[timing] = lib
    return _LIBS[timing]


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Oracle:
    """CPU restatement of the reference SU(2) core for one lattice + frequency mesh."""

    def __init__(self, tables, freq, spin_length: float = 0.5, timing: bool = False):
        self.lib = _lib(timing)
        self.freq = np.ascontiguousarray(freq, np.float32)
        self.n = len(self.freq)
        self.nl = int(tables.n_sites)
        self.fn = self.n * self.n * (self.n + 1) // 2
        self._keep = [np.ascontiguousarray(x, np.int32) for x in
                      (tables.sites_rid, tables.inv_sites_rid, tables.overlap_ptr, tables.overlap_rid1,
                       tables.overlap_rid2, tables.range_rid, tables.range_inv_rid)]
        k = self._keep
        d = OracleDesc()
        d.n_freq, d.freq, d.n_sites = self.n, _p(self.freq, C.c_float), self.nl
        d.sites_rid, d.inv_sites_rid = _p(k[0], C.c_int), _p(k[1], C.c_int)
        d.overlap_ptr, d.overlap_rid1, d.overlap_rid2 = _p(k[2], C.c_int), _p(k[3], C.c_int), _p(k[4], C.c_int)
        d.n_range, d.range_rid, d.range_inv_rid = len(k[5]), _p(k[5], C.c_int), _p(k[6], C.c_int)
        d.spin_length = spin_length
        self.desc = d

    def rhs(self, cutoff, v2, ss, dd, fp64: bool = False, threads: int = 0):
        """Self-energy flow [N] and vertex flow [F_N*Nl] x2."""
        t = np.float64 if fp64 else np.float32
        ct = C.c_double if fp64 else C.c_float
        v2, ss, dd = (np.ascontiguousarray(x, t).reshape(-1) for x in (v2, ss, dd))
        dv2 = np.empty(self.n, t)
        dss = np.empty(self.fn * self.nl, t)
        ddd = np.empty(self.fn * self.nl, t)
        fn = self.lib.oracle_su2_rhs_f64 if fp64 else self.lib.oracle_su2_rhs_f32
        rc = fn(C.byref(self.desc), cutoff, _p(v2, ct), _p(ss, ct), _p(dd, ct), _p(dv2, ct), _p(dss, ct), _p(ddd, ct),
                threads)
        assert rc == 0
        return dv2, dss, ddd

    def self_energy(self, cutoff, v2, ss, dd):
        v2, ss, dd = (np.ascontiguousarray(x, np.float32).reshape(-1) for x in (v2, ss, dd))
        dv2 = np.empty(self.n, np.float32)
        f = C.c_float
        assert self.lib.oracle_su2_self_energy_f32(C.byref(self.desc), cutoff, _p(v2, f), _p(ss, f), _p(dd, f),
                                                   _p(dv2, f)) == 0
        return dv2

    def vertex_range(self, cutoff, v2, dv2, ss, dd, it0: int, it1: int, fp64: bool = False):
        """Vertex flow of triples [it0, it1) given the self-energy flow dv2."""
        t = np.float64 if fp64 else np.float32
        ct = C.c_double if fp64 else C.c_float
        v2, dv2, ss, dd = (np.ascontiguousarray(x, t).reshape(-1) for x in (v2, dv2, ss, dd))
        dss = np.empty((it1 - it0) * self.nl, t)
        ddd = np.empty((it1 - it0) * self.nl, t)
        fn = self.lib.oracle_su2_vertex_range_f64 if fp64 else self.lib.oracle_su2_vertex_range_f32
        assert fn(C.byref(self.desc), cutoff, _p(v2, ct), _p(dv2, ct), _p(ss, ct), _p(dd, ct), it0, it1, _p(dss, ct),
                  _p(ddd, ct)) == 0
        return dss, ddd

    def vertex_sample(self, cutoff, v2, dv2, ss, dd, triples, threads: int = 0):
        """Vertex flow of the listed triples, computed in parallel on `threads` host threads."""
        its = np.ascontiguousarray(triples, np.int32)
        v2, dv2, ss, dd = (np.ascontiguousarray(x, np.float32).reshape(-1) for x in (v2, dv2, ss, dd))
        dss = np.empty(len(its) * self.nl, np.float32)
        ddd = np.empty(len(its) * self.nl, np.float32)
        f = C.c_float
        assert self.lib.oracle_su2_vertex_sample_f32(C.byref(self.desc), cutoff, _p(v2, f), _p(dv2, f), _p(ss, f),
                                                     _p(dd, f), _p(its, C.c_int), len(its), _p(dss, f), _p(ddd, f),
                                                     threads) == 0
        return dss, ddd

    def euler(self, cutoff, new_cutoff, x, dx):
        """x += (new_cutoff - cutoff) * dx in place, rounded like SU2FrgCore::finalizeStep."""
        assert x.dtype == np.float32 and dx.dtype == np.float32 and x.flags.c_contiguous and dx.flags.c_contiguous
        self.lib.oracle_su2_euler_f32(cutoff, new_cutoff, x.size, _p(x, C.c_float), _p(dx, C.c_float))

    def correlation(self, cutoff, v2, ss, dd, fp64: bool = False):
        """Per-rid static susceptibility (spin, density)."""
        t = np.float64 if fp64 else np.float32
        ct = C.c_double if fp64 else C.c_float
        v2, ss, dd = (np.ascontiguousarray(x, t).reshape(-1) for x in (v2, ss, dd))
        cs = np.empty(self.nl, t)
        cd = np.empty(self.nl, t)
        fn = self.lib.oracle_su2_correlation_f64 if fp64 else self.lib.oracle_su2_correlation_f32
        assert fn(C.byref(self.desc), cutoff, _p(v2, ct), _p(ss, ct), _p(dd, ct), _p(cs, ct), _p(cd, ct)) == 0
        return cs, cd

    def flow(self, cutoffs, v2, ss, dd, threads: int = 0, fp64: bool = False):
        """Whole flow; returns (n_measured, chi_s[n_cut, Nl], chi_d[n_cut, Nl], final state).
        fp64=True runs every operation in double precision (the FP64 oracle)."""
        cut = np.ascontiguousarray(cutoffs, np.float32)
        t = np.float64 if fp64 else np.float32
        ct = C.c_double if fp64 else C.c_float
        v2, ss, dd = (np.array(x, t).reshape(-1) for x in (v2, ss, dd))
        cs = np.zeros((len(cut), self.nl), t)
        cd = np.zeros((len(cut), self.nl), t)
        fn = self.lib.oracle_su2_flow_f64 if fp64 else self.lib.oracle_su2_flow_f32
        n = fn(C.byref(self.desc), _p(cut, C.c_float), len(cut), _p(v2, ct), _p(ss, ct), _p(dd, ct), _p(cs, ct),
               _p(cd, ct), threads)
        assert n > 0
        return n, cs, cd, (v2, ss, dd)


# ---------------------------------------------------------------------------------------
# XYZ core (oracle/xyz_oracle.cpp): models with diagonal couplings (Kitaev, XXZ, ...)
# ---------------------------------------------------------------------------------------
class XyzOracleDesc(C.Structure):
    _fields_ = [
        ("n_freq", C.c_int), ("freq", C.POINTER(C.c_float)), ("n_sites", C.c_int),
        ("sites_rid", C.POINTER(C.c_int)), ("sites_perm", C.POINTER(C.c_int)),
        ("inv_sites_rid", C.POINTER(C.c_int)), ("inv_sites_perm", C.POINTER(C.c_int)),
        ("overlap_ptr", C.POINTER(C.c_int)), ("overlap_rid1", C.POINTER(C.c_int)),
        ("overlap_rid2", C.POINTER(C.c_int)), ("overlap_perm1", C.POINTER(C.c_int)),
        ("overlap_perm2", C.POINTER(C.c_int)), ("n_range", C.c_int), ("range_rid", C.POINTER(C.c_int)),
        ("range_inv_rid", C.POINTER(C.c_int)),
    ]


SPIN_PERMUTATIONS = np.array([[0, 1, 2], [0, 2, 1], [1, 0, 2], [1, 2, 0], [2, 0, 1], [2, 1, 0]], np.int32)


def xyz_initial_state(tables, n_freq: int, normalization: float = 1.0):
    """XYZEffectiveAction initial condition (src/XYZ/XYZEffectiveAction.hpp:38-60):
    v4[c][it*Nl + rid] += 0.25 J^cc(rid) / normalization for c = X, Y, Z; density and
    self-energy zero."""
    fn = n_freq * n_freq * (n_freq + 1) // 2
    v2 = np.zeros(n_freq, np.float32)
    v4 = np.zeros((4, fn, tables.n_sites), np.float32)
    for rid, J in zip(tables.interaction_rid, tables.interaction_J):
        for c in range(3):
            v4[c, :, rid] += (np.float32(0.25) * np.float32(J[c, c])) / np.float32(normalization)
    return v2, v4.reshape(4, -1)


def xyz_scatter(chi, tables, spin):
    """Correlations per (basis, site in range) of chi[4][Nl] (XYZMeasurementCorrelation.cpp:
    166-184): component c of entry (b, j) reads component perm[c] of its representative."""
    rid = tables.corr_rid.reshape(tables.n_basis, tables.n_range)
    perm = spin.corr_perm.reshape(tables.n_basis, tables.n_range)
    out = np.empty((4, tables.n_basis, tables.n_range), chi.dtype)
    for c in range(3):
        out[c] = chi[SPIN_PERMUTATIONS[perm, c], rid]
    out[3] = chi[3, rid]
    return out


class XyzOracle:
    """CPU restatement of the reference XYZ core for one lattice + frequency mesh."""

    def __init__(self, tables, spin, freq):
        lib = _lib()
        self.lib = lib
        fp, i4 = C.POINTER(C.c_float), C.c_int
        pp = C.POINTER(C.POINTER(C.c_float))
        dsc = C.POINTER(XyzOracleDesc)
        lib.oracle_xyz_rhs_f32.argtypes = [dsc, C.c_float, fp, pp, fp, pp, i4]
        lib.oracle_xyz_correlation_f32.argtypes = [dsc, C.c_float, fp, pp, pp]
        lib.oracle_xyz_flow_f32.argtypes = [dsc, fp, i4, fp, pp, pp, i4]
        self.freq = np.ascontiguousarray(freq, np.float32)
        self.n = len(self.freq)
        self.nl = int(tables.n_sites)
        self.fn = self.n * self.n * (self.n + 1) // 2
        arrs = [tables.sites_rid, spin.sites_perm, tables.inv_sites_rid, spin.inv_sites_perm, tables.overlap_ptr,
                tables.overlap_rid1, tables.overlap_rid2, spin.overlap_perm1, spin.overlap_perm2, tables.range_rid,
                tables.range_inv_rid]
        self._keep = [np.ascontiguousarray(a, np.int32) for a in arrs]
        k = [_p(a, C.c_int) for a in self._keep]
        d = XyzOracleDesc()
        d.n_freq, d.freq, d.n_sites = self.n, _p(self.freq, C.c_float), self.nl
        (d.sites_rid, d.sites_perm, d.inv_sites_rid, d.inv_sites_perm, d.overlap_ptr, d.overlap_rid1, d.overlap_rid2,
         d.overlap_perm1, d.overlap_perm2) = k[:9]
        d.n_range, d.range_rid, d.range_inv_rid = len(self._keep[9]), k[9], k[10]
        self.desc = d

    @staticmethod
    def _pp(arrs):
        return (C.POINTER(C.c_float) * len(arrs))(*[_p(a, C.c_float) for a in arrs])

    def rhs(self, cutoff, v2, v4, threads: int = 0):
        """(dv2[N], dv4[4][F_N*Nl]) of the state (v2[N], v4[4][F_N*Nl])."""
        v2 = np.ascontiguousarray(v2, np.float32)
        v4 = [np.ascontiguousarray(x, np.float32).reshape(-1) for x in v4]
        dv2 = np.empty(self.n, np.float32)
        dv4 = [np.empty(self.fn * self.nl, np.float32) for _ in range(4)]
        assert self.lib.oracle_xyz_rhs_f32(C.byref(self.desc), cutoff, _p(v2, C.c_float), self._pp(v4), _p(dv2, C.c_float),
                                           self._pp(dv4), threads) == 0
        return dv2, np.stack(dv4)

    def correlation(self, cutoff, v2, v4):
        v2 = np.ascontiguousarray(v2, np.float32)
        v4 = [np.ascontiguousarray(x, np.float32).reshape(-1) for x in v4]
        chi = [np.empty(self.nl, np.float32) for _ in range(4)]
        assert self.lib.oracle_xyz_correlation_f32(C.byref(self.desc), cutoff, _p(v2, C.c_float), self._pp(v4),
                                                   self._pp(chi)) == 0
        return np.stack(chi)

    def flow(self, cutoffs, v2, v4, threads: int = 0):
        """Whole flow; returns (n_measured, chi[n_cut, 4, Nl], final (v2, v4))."""
        cut = np.ascontiguousarray(cutoffs, np.float32)
        v2 = np.array(v2, np.float32)
        v4 = [np.array(x, np.float32).reshape(-1) for x in v4]
        chi = [np.zeros(len(cut) * self.nl, np.float32) for _ in range(4)]
        n = self.lib.oracle_xyz_flow_f32(C.byref(self.desc), _p(cut, C.c_float), len(cut), _p(v2, C.c_float),
                                         self._pp(v4), self._pp(chi), threads)
        assert n > 0
        return n, np.stack(chi).reshape(4, len(cut), self.nl).transpose(1, 0, 2), (v2, np.stack(v4))


# ---------------------------------------------------------------------------------------
# TRI core (oracle/tri_oracle.cpp): time-reversal-invariant models with general couplings
# (Heisenberg-Kitaev-Gamma, ...).  The vertex has 16 components (a, b), a, b in X, Y, Z,
# density, stored as v4[F_N][16][Nl] (component 4a + b), the reference's own layout.
# ---------------------------------------------------------------------------------------
TRI_COMPONENTS = ("xx", "xy", "xz", "yx", "yy", "yz", "zx", "zy", "zz", "dd")


def tri_initial_state(tables, n_freq: int, normalization: float = 1.0):
    """TRIEffectiveAction initial condition (src/TRI/TRIEffectiveAction.hpp:38-62):
    v4[it][a][b][rid] += 0.25 J^ab(rid) / normalization for spin components a, b; every
    component with a density index and the self-energy start at zero."""
    fn = n_freq * n_freq * (n_freq + 1) // 2
    v2 = np.zeros(n_freq, np.float32)
    v4 = np.zeros((fn, 4, 4, tables.n_sites), np.float32)
    for rid, J in zip(tables.interaction_rid, tables.interaction_J):
        for a in range(3):
            for b in range(3):
                v4[:, a, b, rid] += (np.float32(0.25) * np.float32(J[a, b])) / np.float32(normalization)
    return v2, v4.reshape(-1)


def tri_scatter(chi, tables, spin):
    """Correlations per (basis, site in range) of chi[16][Nl] (TRIMeasurementCorrelation.cpp:
    262-284): entry (b, j) of component (a, c) reads component (P a, P c) of its representative,
    P the entry's spin permutation; returns [10, n_basis, n_range] in TRI_COMPONENTS order."""
    chi = np.asarray(chi).reshape(16, -1)
    rid = tables.corr_rid.reshape(tables.n_basis, tables.n_range)
    perm = SPIN_PERMUTATIONS[spin.corr_perm.reshape(tables.n_basis, tables.n_range)]
    out = np.empty((10, tables.n_basis, tables.n_range), chi.dtype)
    q = 0
    for a in range(3):
        for c in range(3):
            out[q] = chi[4 * perm[..., a] + perm[..., c], rid]
            q += 1
    out[9] = chi[15, rid]
    return out


class TriOracle:
    """CPU restatement of the reference TRI core for one lattice + frequency mesh."""

    def __init__(self, tables, spin, freq):
        lib = _lib()
        self.lib = lib
        fp, i4 = C.POINTER(C.c_float), C.c_int
        dsc = C.POINTER(XyzOracleDesc)
        lib.oracle_tri_rhs_f32.argtypes = [dsc, C.c_float, fp, fp, fp, fp, i4]
        lib.oracle_tri_correlation_f32.argtypes = [dsc, C.c_float, fp, fp, fp]
        lib.oracle_tri_flow_f32.argtypes = [dsc, fp, i4, fp, fp, fp, i4]
        lib.oracle_tri_tables.argtypes = [C.POINTER(C.c_int)]
        self.freq = np.ascontiguousarray(freq, np.float32)
        self.n = len(self.freq)
        self.nl = int(tables.n_sites)
        self.fn = self.n * self.n * (self.n + 1) // 2
        self.size = self.fn * 16 * self.nl
        arrs = [tables.sites_rid, spin.sites_perm, tables.inv_sites_rid, spin.inv_sites_perm, tables.overlap_ptr,
                tables.overlap_rid1, tables.overlap_rid2, spin.overlap_perm1, spin.overlap_perm2, tables.range_rid,
                tables.range_inv_rid]
        self._keep = [np.ascontiguousarray(a, np.int32) for a in arrs]
        k = [_p(a, C.c_int) for a in self._keep]
        d = XyzOracleDesc()
        d.n_freq, d.freq, d.n_sites = self.n, _p(self.freq, C.c_float), self.nl
        (d.sites_rid, d.sites_perm, d.inv_sites_rid, d.inv_sites_perm, d.overlap_ptr, d.overlap_rid1, d.overlap_rid2,
         d.overlap_perm1, d.overlap_perm2) = k[:9]
        d.n_range, d.range_rid, d.range_inv_rid = len(self._keep[9]), k[9], k[10]
        self.desc = d

    def tables(self):
        """The coefficient tables as rows (table, output, n, a, b, sign)."""
        rows = np.zeros(6 * 16 * 72, np.int32)
        n = self.lib.oracle_tri_tables(_p(rows, C.c_int))
        assert n > 0
        return rows[:6 * n].reshape(n, 6)

    def rhs(self, cutoff, v2, v4, threads: int = 0):
        """(dv2[N], dv4[F_N*16*Nl]) of the state (v2[N], v4[F_N*16*Nl])."""
        v2 = np.ascontiguousarray(v2, np.float32)
        v4 = np.ascontiguousarray(v4, np.float32).reshape(-1)
        assert v4.size == self.size
        dv2 = np.empty(self.n, np.float32)
        dv4 = np.empty(self.size, np.float32)
        assert self.lib.oracle_tri_rhs_f32(C.byref(self.desc), cutoff, _p(v2, C.c_float), _p(v4, C.c_float),
                                           _p(dv2, C.c_float), _p(dv4, C.c_float), threads) == 0
        return dv2, dv4

    def correlation(self, cutoff, v2, v4):
        """chi[16][Nl] at the state (the mixed spin/density components are zero)."""
        v2 = np.ascontiguousarray(v2, np.float32)
        v4 = np.ascontiguousarray(v4, np.float32).reshape(-1)
        chi = np.empty(16 * self.nl, np.float32)
        assert self.lib.oracle_tri_correlation_f32(C.byref(self.desc), cutoff, _p(v2, C.c_float), _p(v4, C.c_float),
                                                   _p(chi, C.c_float)) == 0
        return chi.reshape(16, self.nl)

    def flow(self, cutoffs, v2, v4, threads: int = 0):
        """Whole flow; returns (n_measured, chi[n_cut, 16, Nl], final (v2, v4))."""
        cut = np.ascontiguousarray(cutoffs, np.float32)
        v2 = np.array(v2, np.float32)
        v4 = np.array(v4, np.float32).reshape(-1)
        chi = np.zeros(len(cut) * 16 * self.nl, np.float32)
        n = self.lib.oracle_tri_flow_f32(C.byref(self.desc), _p(cut, C.c_float), len(cut), _p(v2, C.c_float),
                                         _p(v4, C.c_float), _p(chi, C.c_float), threads)
        assert n > 0
        return n, chi.reshape(len(cut), 16, self.nl), (v2, v4)
