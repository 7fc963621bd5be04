"""Known-answer tests of the frequency-mesh lookups and the loop-frequency quadrature rules that
the vertex kernels and node tables use, run on the host by the same code (spn_mesh_probe,
spn_quadrature_nodes; no GPU).  The cases and values are the reference's own unit tests:
test/test_FrequencyDiscretization.cpp:25-121 (mesh {1, ..., 5}) and test/test_Integrator.cpp:39-121
(mesh {1, ..., 10}, integrands x and x^2, tolerance 1e-6)."""
import ctypes as C

import numpy as np
import pytest

from spinparser_gb300._capi import SpnError, check, load_library

fp, ip, dp = C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_double)


def probe(mesh, w):
    lib = load_library()
    pos = np.ascontiguousarray(mesh, np.float32)
    lesser, greater, bias = C.c_float(), C.c_float(), C.c_float()
    offset, lo, hi = C.c_int(), C.c_int(), C.c_int()
    check(lib.spn_mesh_probe(pos.ctypes.data_as(fp), len(pos), w, C.byref(lesser), C.byref(greater), C.byref(offset),
                             C.byref(lo), C.byref(hi), C.byref(bias)))
    return lesser.value, greater.value, offset.value, lo.value, hi.value, bias.value


def nodes(mesh, rule, lo=0.0, hi=0.0):
    lib = load_library()
    pos = np.ascontiguousarray(mesh, np.float32)
    cnt = C.c_int()
    check(lib.spn_quadrature_nodes(pos.ctypes.data_as(fp), len(pos), rule, lo, hi, None, None, 0, C.byref(cnt)))
    wp, w = np.zeros(cnt.value, np.float32), np.zeros(cnt.value, np.float64)
    check(lib.spn_quadrature_nodes(pos.ctypes.data_as(fp), len(pos), rule, lo, hi, wp.ctypes.data_as(fp),
                                   w.ctypes.data_as(dp), cnt.value, C.byref(cnt)))
    return wp.astype(np.float64), w


MESH5 = [1.0, 2.0, 3.0, 4.0, 5.0]
MESH10 = [float(x) for x in range(1, 11)]


@pytest.mark.parametrize("w,lesser,greater", [
    (10.0, 5.0, 5.0), (0.5, 1.0, 1.0), (3.5, 3.0, 4.0), (-10.0, -5.0, -5.0), (-0.5, -1.0, -1.0), (-3.5, -4.0, -3.0),
])
def test_lesser_and_greater(w, lesser, greater):
    """FrequencyDiscretization::lesser / greater on the symmetric mesh, clamped at both ends."""
    got = probe(MESH5, w)
    assert got[0] == lesser and got[1] == greater


@pytest.mark.parametrize("w,offset", [(1.0, 0), (2.0, 1), (5.0, 4)])
def test_offset(w, offset):
    assert probe(MESH5, w)[2] == offset


def test_interpolate_offset():
    """interpolateOffset: clamped above and below the mesh, bias 0.5 half way."""
    _, _, _, lo, hi, b = probe(MESH5, 10.0)
    assert (lo, hi) == (4, 4) and 0.0 <= b <= 1.0
    _, _, _, lo, hi, b = probe(MESH5, 4.5)
    assert (lo, hi) == (3, 4) and b == pytest.approx(0.5, rel=1e-6)
    _, _, _, lo, hi, b = probe(MESH5, 0.1)
    assert (lo, hi) == (0, 0) and 0.0 <= b <= 1.0


@pytest.mark.parametrize("rule,lo,hi,linear,quadratic", [
    (0, 1.5, 0.0, 48.875, 333.5625),   # integrateWithObscureLeftBoundary(1.5, last)
    (2, 1.5, 9.5, 44.0, 285.875),      # integrateWithObscureBoundaries(1.5, 9.5)
    (2, 1.0, 9.5, 44.625, 286.8125),   # from the mesh point 1: the reference's ObscureRightBoundary(begin, 9.5)
    (2, 1.0, 10.0, 49.5, 334.5),       # integrate(begin, last): mesh points only
])
def test_trapezoid_rules(rule, lo, hi, linear, quadratic):
    wp, w = nodes(MESH10, rule, lo, hi)
    assert np.sum(w * wp) == pytest.approx(linear, rel=1e-6)
    assert np.sum(w * wp * wp) == pytest.approx(quadratic, rel=1e-6)


def test_right_boundary_rule_from_the_negative_end():
    """integrateWithObscureRightBoundary(beginNegative, max): the trapezoid rule over every
    symmetric-mesh point up to max and max itself."""
    full = [-x for x in reversed(MESH10)] + MESH10
    for mx in (9.5, 3.0, -2.5, -10.0 + 0.25):
        wp, w = nodes(MESH10, 1, hi=mx)
        pts = np.array([x for x in full if x <= mx] + ([mx] if mx not in full else []))
        for f in (lambda x: x, lambda x: x * x):
            want = np.sum(0.5 * (pts[1:] - pts[:-1]) * (f(pts[1:]) + f(pts[:-1])))
            assert np.sum(w * f(wp)) == pytest.approx(want, rel=1e-6, abs=1e-6)


def test_bad_meshes_are_rejected():
    lib = load_library()
    cnt = C.c_int()
    for mesh in ([2.0, 1.0], [0.0, 1.0], [1.0]):
        pos = np.ascontiguousarray(mesh, np.float32)
        with pytest.raises(SpnError):
            check(lib.spn_quadrature_nodes(pos.ctypes.data_as(fp), len(pos), 0, 1.0, 0.0, None, None, 0, C.byref(cnt)))
