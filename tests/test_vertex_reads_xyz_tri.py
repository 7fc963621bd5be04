"""Known-answer tests of the XYZ and TRI kernels' vertex reads, run on the host by the kernels'
own code (spn_xyz_vertex_probe, spn_tri_vertex_probe; no GPU).  The cases are the reference's
unit tests test/test_XYZVertexTwoParticle.cpp:75-271 and test/test_TRIVertexTwoParticle.cpp:75-253:
mesh {1, ..., 5}, a square lattice of range 3, state value i at element i (XYZ: i, i + 1, i + 2,
i + 3 in X, Y, Z, D), tolerance 0.0001 % where the reference uses BOOST_CHECK_CLOSE and exact
equality where it uses BOOST_CHECK_EQUAL.  The spin-permutation cases check the superbundle
reads of sites whose representative is reached through a permutation of X, Y, Z against the
direct read of the permuted components (the oracle's permutation table)."""
import ctypes as C

import numpy as np
import pytest

from oracle import SPIN_PERMUTATIONS
from spinparser_gb300._capi import SpnError, check, load_library

fp = C.POINTER(C.c_float)
MESH5 = np.float32([1.0, 2.0, 3.0, 4.0, 5.0])
N = len(MESH5)
FN = N * N * (N + 1) // 2


def lattice():
    import spinparser_gb300 as spn
    tab = spn.Lattice("square", 3, "square-heisenberg", {"j": "1"}).tables()
    return tab.n_sites, np.asarray(tab.inv_sites_rid)


NL, INV = lattice()
RID12 = 1                 # the second site of the range of the basis site
RID21 = int(INV[RID12])   # the same pair, sites exchanged


def frequencies():
    """(frequency index, s, t, u) of every stored element: index (s(s+1)/2 + u) N + t, s >= u."""
    for s in range(N):
        for u in range(s + 1):
            for t in range(N):
                yield (s * (s + 1) // 2 + u) * N + t, float(MESH5[s]), float(MESH5[t]), float(MESH5[u])


# ---- XYZ ----

def xyz_state(by_frequency=False):
    i = np.arange(FN * NL, dtype=np.float32)
    if by_frequency:
        i = np.repeat(np.arange(FN, dtype=np.float32), NL)
    return [np.ascontiguousarray(i + np.float32(k)) for k in range(4)]


XYZ = xyz_state()


def xyz(s, t, u, channel=-1, local=False, rid12=RID12, rid21=RID21, perm=0, exchanged=False, state=None):
    """The four components X, Y, Z, D of one read."""
    st = XYZ if state is None else state
    if exchanged:
        rid12, rid21 = rid21, rid12
    out = np.zeros(4, np.float32)
    check(load_library().spn_xyz_vertex_probe(MESH5.ctypes.data_as(fp), N, NL, *(a.ctypes.data_as(fp) for a in st),
                                              rid12, rid21, perm, perm, s, t, u, channel, int(local),
                                              out.ctypes.data_as(fp)))
    return out


def test_xyz_layout():
    """ExpandIteratorFull / ExpandIteratorFrequency: the direct read at the frequencies and site
    of element i returns that element, in every component."""
    for f, s, t, u in frequencies():
        for rid in range(NL):
            v = xyz(s, t, u, rid12=rid, rid21=int(INV[rid]))
            i = f * NL + rid
            assert v.tolist() == [i, i + 1, i + 2, i + 3]
    byf = xyz_state(by_frequency=True)
    for f, s, t, u in frequencies():
        assert xyz(s, t, u, rid12=0, rid21=0, state=byf).tolist() == [f, f + 1, f + 2, f + 3]


def test_xyz_symmetries():
    """getValueSymmetry: s -> -s and u -> -u exchange the sites, t -> -t changes nothing, s <-> u
    flips the sign of the density component only."""
    s, t, u = 1.0, 2.0, 3.0
    v = xyz(s, t, u)
    assert (v == xyz(-s, t, u, exchanged=True)).all()
    assert (v == xyz(s, -t, u)).all()
    assert (v == xyz(s, t, -u, exchanged=True)).all()
    assert (v == np.float32([1, 1, 1, -1]) * xyz(u, t, s)).all()


@pytest.mark.parametrize("channel,axis", [(-1, 0), (0, 1), (1, 2), (2, 0)])
def test_xyz_interpolation_is_linear(channel, axis):
    """getValueInterpolation: between two mesh values the read is the linear interpolation of the
    reads at them, for the direct read and the s-, t- and u-channel access buffers."""
    w_exact, w_lower, w_upper, lam = 1.0, 2.0, 3.0, 0.2
    mid = float(np.float32((1.0 - lam) * w_lower + lam * w_upper))

    def at(x):
        c = [w_exact, w_exact, w_exact]
        c[axis] = x
        return c
    lower, upper = xyz(*at(w_lower)), xyz(*at(w_upper))
    exact = xyz(*at(mid), channel=channel)
    np.testing.assert_allclose(exact, (1.0 - lam) * lower + lam * upper, rtol=1e-6)


BUFFERED = [(1.1, 2.2, 3.3, 3), (2.0, 3.0, 4.0, 3), (2.0, 3.5, 4.5, 0), (2.5, 3.0, 4.5, 1), (2.5, 3.5, 4.0, 2),
            (-2.0, 3.5, 4.5, 0), (2.5, -3.0, -4.5, 1), (-2.5, 3.5, 4.0, 2), (-1.1, 2.2, -3.3, 3), (2.0, -3.5, 4.5, 0)]
# one point per access buffer: the channel's own coordinate a mesh value (channels 0-2)
POINTS = {0: (2.0, 3.5, 4.5), 1: (2.5, 3.0, 4.5), 2: (2.5, 3.5, 4.0), 3: (1.1, 2.2, 3.3)}


@pytest.mark.parametrize("s,t,u,channel", BUFFERED)
def test_xyz_access_buffer_read_equals_direct_read(s, t, u, channel):
    """getValueBuffered: a read through an access buffer equals the direct read at the same
    frequencies (the buffer's channel coordinate is a mesh value); negative frequencies fold."""
    np.testing.assert_allclose(xyz(s, t, u, channel=channel), xyz(s, t, u), rtol=1e-6)


@pytest.mark.parametrize("s,t,u,channel", BUFFERED)
def test_xyz_local_read(s, t, u, channel):
    """getValueLocal: the read of the pair (origin, origin) through the buffer equals its direct
    read."""
    np.testing.assert_allclose(xyz(s, t, u, channel=channel, local=True), xyz(s, t, u, rid12=0, rid21=0), rtol=1e-6)


@pytest.mark.parametrize("channel", [0, 1, 2, 3])
def test_xyz_superbundle_reads(channel):
    """getValueSuperbundle: for every rid the gather equals the direct read of that pair."""
    s, t, u = POINTS[channel]
    for rid in range(NL):
        for sg in (1.0, -1.0):
            kw = dict(rid12=rid, rid21=int(INV[rid]))
            np.testing.assert_allclose(xyz(sg * s, t, u, channel=channel, **kw), xyz(sg * s, t, u, **kw), rtol=1e-6)


@pytest.mark.parametrize("channel", [0, 1, 2, 3])
@pytest.mark.parametrize("perm", range(6))
def test_xyz_permuted_reads(channel, perm):
    """A site reached through spin permutation p reads X, Y, Z as the components perm[p][X, Y, Z]
    of its representative, D unchanged, whether or not the buffer exchanges the sites."""
    s, t, u = POINTS[channel]
    comp = list(SPIN_PERMUTATIONS[perm]) + [3]
    for sg in (1.0, -1.0):
        got = xyz(sg * s, t, u, channel=channel, perm=perm)
        np.testing.assert_allclose(got, xyz(sg * s, t, u)[comp], rtol=1e-6)


def test_xyz_probe_rejects_bad_arguments():
    with pytest.raises(SpnError):
        xyz(2.1, 3.0, 4.0, channel=0)       # the s channel's own frequency is no mesh value
    with pytest.raises(SpnError):
        xyz(2.0, 3.0, 4.0, perm=1)          # the direct read takes identity permutations only
    with pytest.raises(SpnError):
        xyz(2.0, 3.0, 4.0, channel=0, rid12=NL)


# ---- TRI ----

XI = np.float32([-1.0, -1.0, -1.0, 1.0])   # xi(a): -1 for X, Y, Z, +1 for the density


def tri_state(by_frequency=False):
    if by_frequency:
        return np.ascontiguousarray(np.repeat(np.arange(FN, dtype=np.float32), 16 * NL))
    return np.arange(FN * 16 * NL, dtype=np.float32)


TRI = tri_state()


def tri(s, t, u, channel=-1, local=False, rid12=RID12, rid21=RID21, perm=0, exchanged=False, state=None):
    """The 16 components (a, b) of one read as a 4 x 4 array."""
    st = TRI if state is None else state
    if exchanged:
        rid12, rid21 = rid21, rid12
    out = np.zeros(16, np.float32)
    check(load_library().spn_tri_vertex_probe(MESH5.ctypes.data_as(fp), N, NL, st.ctypes.data_as(fp), rid12, rid21,
                                              perm, perm, s, t, u, channel, int(local), out.ctypes.data_as(fp)))
    return out.reshape(4, 4)


def test_tri_layout():
    """ExpandIteratorFull / ExpandIteratorFrequency: element ((f * 16) + 4a + b) * Nl + rid is
    the direct read of components (a, b) of that site at the frequencies of f."""
    comp = np.arange(16).reshape(4, 4)
    for f, s, t, u in frequencies():
        for rid in range(NL):
            v = tri(s, t, u, rid12=rid, rid21=int(INV[rid]))
            assert (v == ((f * 16 + comp) * NL + rid)).all()
    byf = tri_state(by_frequency=True)
    for f, s, t, u in frequencies():
        assert (tri(s, t, u, rid12=0, rid21=0, state=byf) == f).all()


def test_tri_symmetries():
    """getValueSymmetry (TRIVertexTwoParticle's sign table): with xi = -1 for a spin and +1 for
    the density component,
    v(i1, i2, s, t, u, a, b) = v(i2, i1, -s, t, u, b, a)
                             = xi(a) xi(b) v(i1, i2, s, -t, u, a, b)
                             = xi(a) xi(b) v(i2, i1, s, t, -u, b, a)
                             = -xi(b) v(i1, i2, u, t, s, a, b)."""
    s, t, u = 1.0, 2.0, 3.0
    v = tri(s, t, u)
    xx = np.outer(XI, XI)
    assert (v == tri(-s, t, u, exchanged=True).T).all()
    assert (v == xx * tri(s, -t, u)).all()
    assert (v == xx * tri(s, t, -u, exchanged=True).T).all()
    assert (v == -XI[None, :] * tri(u, t, s)).all()


@pytest.mark.parametrize("channel,axis", [(-1, 0), (0, 1), (1, 2), (2, 0)])
def test_tri_interpolation_is_linear(channel, axis):
    """getValueInterpolation, all 16 components."""
    w_exact, w_lower, w_upper, lam = 1.0, 2.0, 3.0, 0.2
    mid = float(np.float32((1.0 - lam) * w_lower + lam * w_upper))

    def at(x):
        c = [w_exact, w_exact, w_exact]
        c[axis] = x
        return c
    lower, upper = tri(*at(w_lower)), tri(*at(w_upper))
    np.testing.assert_allclose(tri(*at(mid), channel=channel), (1.0 - lam) * lower + lam * upper, rtol=1e-6)


@pytest.mark.parametrize("s,t,u,channel", BUFFERED)
def test_tri_access_buffer_read_equals_direct_read(s, t, u, channel):
    """getValueBuffered: the vertex kernel's slab gather (channels S, T, U) and the correlation's
    trilinear read equal the direct read, the access buffers' sign table included."""
    np.testing.assert_allclose(tri(s, t, u, channel=channel), tri(s, t, u), rtol=1e-6)


@pytest.mark.parametrize("s,t,u,channel", BUFFERED + [(-4.0, 3.5, 2.5, 0), (4.5, 3.0, -2.5, 1), (-3.3, 2.2, 1.1, 3)])
def test_tri_local_read(s, t, u, channel):
    """getValueLocal (the chalice diagrams' and the egg diagram's site-local reads) equals the
    direct read of the pair (origin, origin) where the buffer does not exchange the sites, the
    reference's own case (positive frequencies).  Where it does, the reference exchanges the two
    components before it indexes its sign table (TRIVertexTwoParticle.hpp:347-356), where
    getValue and getValueSuperbundle use the original order: a support whose stored sector swaps
    s and u (|s| < |u| at every support of these points) then carries xi(a) xi(b) against the
    direct read, a sign flip of the mixed spin/density components.  The kernels keep the
    reference's convention (the mixed components are small but not zero in a TRI flow, and the
    bit-exact reference golden depends on it)."""
    local, direct = tri(s, t, u, channel=channel, local=True), tri(s, t, u, rid12=0, rid21=0)
    exchanged = (s < 0) != (u < 0)
    factor = np.outer(XI, XI) if exchanged and abs(s) < abs(u) else 1.0
    np.testing.assert_allclose(local, factor * direct, rtol=1e-6)
    same = np.outer(XI, XI) > 0   # spin-spin and density-density: no difference in any case
    np.testing.assert_allclose(local[same], direct[same], rtol=1e-6)


@pytest.mark.parametrize("channel", [0, 1, 2, 3])
def test_tri_superbundle_reads(channel):
    """getValueSuperbundle: for every rid the gather equals the direct read of that pair."""
    s, t, u = POINTS[channel]
    for rid in range(NL):
        for sg in (1.0, -1.0):
            kw = dict(rid12=rid, rid21=int(INV[rid]))
            np.testing.assert_allclose(tri(sg * s, t, u, channel=channel, **kw), tri(sg * s, t, u, **kw), rtol=1e-6)


@pytest.mark.parametrize("channel", [0, 1, 2, 3])
@pytest.mark.parametrize("perm", range(6))
def test_tri_permuted_reads(channel, perm):
    """Components (a, b) of a site reached through spin permutation p are the components
    (perm[p][a], perm[p][b]) of its representative (the density maps to itself), the signs
    unchanged, whether or not the buffer exchanges the sites."""
    s, t, u = POINTS[channel]
    comp = list(SPIN_PERMUTATIONS[perm]) + [3]
    for sg in (1.0, -1.0):
        direct = tri(sg * s, t, u)
        np.testing.assert_allclose(tri(sg * s, t, u, channel=channel, perm=perm), direct[np.ix_(comp, comp)], rtol=1e-6)


def test_tri_probe_rejects_bad_arguments():
    with pytest.raises(SpnError):
        tri(2.0, 3.1, 4.0, channel=1)
    with pytest.raises(SpnError):
        tri(2.0, 3.0, 4.0, local=True)      # a local read needs an access buffer
    with pytest.raises(SpnError):
        tri(2.0, 3.0, 4.0, channel=4)
