"""The RPA schedule the vertex-flow kernel walks (spn_rpa_schedule, host only).

Decoding the schedule exactly as the kernel does and summing must reproduce, for every rid,
the reference's RPA lattice sum over getOverlap(rid) (SU2FrgCore.cpp:249-266), and every index
must stay inside the arrays the kernel allocates for it (rid1, rid2 < Nl; slots < n_seg).
"""
import ctypes as C

import numpy as np
import pytest

import spinparser_gb300 as spn
from spinparser_gb300._capi import check, load_library

LATTICES = [
    ("square", 3, "square-heisenberg", {"j": "1"}),
    ("honeycomb", 3, "honeycomb-heisenberg", {"j": "1"}),
    ("square", 7, "square-j1j2heisenberg", {"j1": "1", "j2": "0.5"}),
    ("cubic", 6, "cubic-j1j2heisenberg", {"j1": "1", "j2": "0.25"}),
    ("pyrochlore", 5, "pyrochlore-heisenberg", {"j": "1"}),
    ("square", 11, "square-heisenberg", {"j": "1"}),
]


def schedule(tab, lanes):
    lib = load_library()
    ip = C.POINTER(C.c_int)
    ptr, r1, r2 = (np.ascontiguousarray(x, np.int32) for x in (tab.overlap_ptr, tab.overlap_rid1, tab.overlap_rid2))
    info = np.zeros(5, np.int32)
    args = (tab.n_sites, ptr.ctypes.data_as(ip), r1.ctypes.data_as(ip), r2.ctypes.data_as(ip), lanes)
    check(lib.spn_rpa_schedule(*args, info.ctypes.data_as(ip), None, None, None, None))
    sched = np.zeros(info[2], np.int32)
    count = np.zeros(lanes, np.int32)
    base = np.zeros(lanes, np.int32)
    seg = np.zeros(tab.n_sites + 1, np.int32)
    check(lib.spn_rpa_schedule(*args, info.ctypes.data_as(ip), sched.ctypes.data_as(ip), count.ctypes.data_as(ip),
                               base.ctypes.data_as(ip), seg.ctypes.data_as(ip)))
    return info, sched, count, base, seg


def decode(nl, lanes, info, sched, count, base, seg, A, B):
    """The kernel's walk: per lane, accumulate m * M[a][b] (M = outer(A, B), Nl <= 32) or
    (A[a] * m) * B[b] (Nl > 32), flush at segment ends."""
    L, n_seg, packed, width = info[0], info[1], bool(info[3]), int(info[4])
    assert info[2] == L * lanes and packed == (nl <= 32)
    slots = np.zeros(n_seg)
    for l in range(lanes):
        assert 0 <= count[l] <= L
        acc, slot = 0.0, base[l]
        for i in range(count[l]):
            e = int(np.uint32(sched[i * lanes + l]))
            if packed:  # byte offset of the float2 element M[a][b] of a width x width matrix
                assert width >= nl and width % 8 == 0
                off = e & 0xFFFF
                assert off % 8 == 0 and off < width * width * 8
                a, b = divmod(off // 8, width)
                m, last = float((e >> 16) & 0xFF), bool(e >> 31)
                assert (e >> 24) & 0x7F == 0
            else:
                a, b, m, last = e & 0x7F, (e >> 7) & 0x7F, float((e >> 14) & 0xFF), bool(e & (1 << 22))
            assert a < nl and b < nl and m >= 1
            acc += A[a] * m * B[b]
            if last:
                assert 0 <= slot < n_seg
                slots[slot] = acc
                acc, slot = 0.0, slot + 1
        assert acc == 0.0  # every chunk ends with a flushed segment
    assert seg[0] == 0 and seg[nl] == n_seg and np.all(np.diff(seg) >= 0)
    return np.array([slots[seg[r]:seg[r + 1]].sum() for r in range(nl)])


@pytest.mark.parametrize("lat", LATTICES, ids=lambda x: f"{x[0]}-r{x[1]}")
def test_schedule_reproduces_rpa_sums(lat):
    tab = spn.Lattice(*lat).tables()
    nl = tab.n_sites
    rng = np.random.default_rng(7)
    A, B = rng.standard_normal(nl), rng.standard_normal(nl)
    ptr, r1, r2 = tab.overlap_ptr, tab.overlap_rid1, tab.overlap_rid2
    want = np.array([np.sum(A[r1[ptr[r]:ptr[r + 1]]] * B[r2[ptr[r]:ptr[r + 1]]]) for r in range(nl)])
    lanes = 32
    got = decode(nl, lanes, *schedule(tab, lanes), A, B)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)
    # merging repeated pairs shortens the walk
    assert schedule(tab, lanes)[0][0] * lanes < ptr[-1] + lanes

