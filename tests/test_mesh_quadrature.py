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


def test_bucket_index_matches_binary_search():
    """The FP32 kernels look the mesh up through a bucket index; it must give the binary
    search's answer everywhere: mesh points, their float neighbours, outside the mesh, NaN."""
    lib = load_library()
    import spinparser_gb300 as spn
    for mesh in (MESH10, list(spn.frequency_exponential(0.005, 100.0, 64)), list(spn.frequency_exponential(0.002, 100.0, 256))):
        pos = np.ascontiguousarray(mesh, np.float32)
        pts = [pos, np.nextafter(pos, 0).astype(np.float32), np.nextafter(pos, np.inf).astype(np.float32),
               np.float32([0.0, 1e-30, 1e-6, 1e3, 1e30, np.inf, np.nan]),
               np.random.default_rng(5).uniform(0, 1.2 * pos[-1], 4000).astype(np.float32)]
        w = np.ascontiguousarray(np.concatenate(pts), np.float32)
        bad = C.c_int()
        check(lib.spn_mesh_index_check(pos.ctypes.data_as(fp), len(pos), w.ctypes.data_as(fp), len(w), C.byref(bad)))
        assert bad.value == 0


# ---- vertex reads (test/test_SU2VertexTwoParticle.cpp:120-245: mesh {1, ..., 5}, square lattice
# range 3, state value i in the spin vertex and i + 1 in the density vertex at element i) ----

def vertex_fixture():
    import spinparser_gb300 as spn
    tab = spn.Lattice("square", 3, "square-heisenberg", {"j": "1"}).tables()
    n, nl = 5, tab.n_sites
    fn = n * n * (n + 1) // 2
    ss = np.arange(fn * nl, dtype=np.float32)
    dd = ss + np.float32(1.0)
    rid12 = 1                                 # the second site of the range of the basis site
    rid21 = int(tab.inv_sites_rid[rid12])     # the same pair, sites exchanged
    return np.float32(MESH5), nl, ss, dd, rid12, rid21


def vread(fx, s, t, u, channel=-1, density=False, exchanged=False):
    pos, nl, ss, dd, r12, r21 = fx
    if exchanged:
        r12, r21 = r21, r12
    out = C.c_float()
    check(load_library().spn_vertex_probe(pos.ctypes.data_as(fp), len(pos), nl, ss.ctypes.data_as(fp),
                                          dd.ctypes.data_as(fp), r12, r21, s, t, u, channel, int(density),
                                          C.byref(out)))
    return out.value


@pytest.mark.parametrize("density", [False, True])
def test_vertex_symmetries(density):
    """getValueSymmetry: s -> -s and u -> -u exchange the sites, t -> -t changes nothing, s <-> u
    flips the sign of the density vertex only."""
    fx = vertex_fixture()
    s, t, u = 1.0, 2.0, 3.0
    v = vread(fx, s, t, u, density=density)
    assert v == vread(fx, -s, t, u, density=density, exchanged=True)
    assert v == vread(fx, s, -t, u, density=density)
    assert v == vread(fx, s, t, -u, density=density, exchanged=True)
    assert v == (-1.0 if density else 1.0) * vread(fx, u, t, s, density=density)


@pytest.mark.parametrize("density", [False, True])
@pytest.mark.parametrize("channel,axis", [(-1, 0), (0, 1), (1, 2), (2, 0)])
def test_vertex_interpolation_is_linear(density, channel, axis):
    """getValueInterpolation: between two mesh values the read is the linear interpolation of the
    reads at them, for the direct read (None) and the s-, t- and u-channel access buffers (the
    interpolated coordinate is one the channel leaves free)."""
    fx = vertex_fixture()
    w_exact, w_lower, w_upper, lam = 1.0, 2.0, 3.0, 0.2
    mid = np.float32((1.0 - lam) * w_lower + lam * w_upper)

    def at(x):
        c = [w_exact, w_exact, w_exact]
        c[axis] = x
        return c
    lower, upper = vread(fx, *at(w_lower), density=density), vread(fx, *at(w_upper), density=density)
    exact = vread(fx, *at(mid), channel=channel, density=density)
    assert exact == pytest.approx((1.0 - lam) * lower + lam * upper, rel=1e-6)


@pytest.mark.parametrize("density", [False, True])
@pytest.mark.parametrize("s,t,u,channel", [
    (1.1, 2.2, 3.3, 3), (2.0, 3.0, 4.0, 3), (2.0, 3.5, 4.5, 0), (2.5, 3.0, 4.5, 1), (2.5, 3.5, 4.0, 2),
    (-2.0, 3.5, 4.5, 0), (2.5, -3.0, -4.5, 1), (-2.5, 3.5, 4.0, 2), (-1.1, 2.2, -3.3, 3),
])
def test_access_buffer_read_equals_direct_read(density, s, t, u, channel):
    """getValueBuffered: a read through an access buffer equals the direct read at the same
    frequencies (the buffer's channel coordinate is a mesh value); negative frequencies fold."""
    fx = vertex_fixture()
    assert vread(fx, s, t, u, channel=channel, density=density) == pytest.approx(
        vread(fx, s, t, u, density=density), rel=1e-6)


@pytest.mark.parametrize("density", [False, True])
def test_local_and_superbundle_reads(density):
    """getValueLocal and getValueSuperbundle: through the trilinear access buffer, the read of the
    pair (origin, origin) and of (origin, rid) for every rid equals the direct read."""
    pos, nl, ss, dd, _, _ = vertex_fixture()
    import spinparser_gb300 as spn
    inv = spn.Lattice("square", 3, "square-heisenberg", {"j": "1"}).tables().inv_sites_rid
    for rid in range(nl):
        fx = (pos, nl, ss, dd, rid, int(inv[rid]))
        assert vread(fx, 1.1, 2.2, 3.3, channel=3, density=density) == pytest.approx(
            vread(fx, 1.1, 2.2, 3.3, density=density), rel=1e-6)


def se_read(data, w):
    out = C.c_double()
    pos = np.float32(MESH5)
    d = np.ascontiguousarray(data, np.float32)
    check(load_library().spn_self_energy_probe(pos.ctypes.data_as(fp), len(pos), d.ctypes.data_as(fp), w,
                                               C.byref(out)))
    return out.value


def test_self_energy_reads():
    """test/test_SU2VertexSingleParticle.cpp:75-105: the value at mesh point i is data[i], the read
    is odd in w, and between two mesh points it is the linear interpolation."""
    data = np.arange(5, dtype=np.float32)
    for i, w in enumerate(MESH5):
        assert se_read(data, w) == data[i]
        assert se_read(data, w) == -se_read(data, -w)
    data = np.float32([2.0, 3.0, 0.0, 0.0, 0.0])
    lam = 0.2
    w = np.float32((1.0 - lam) * MESH5[0] + lam * MESH5[1])
    assert se_read(data, float(w)) == pytest.approx((1.0 - lam) * 2.0 + lam * 3.0, rel=1e-6)
