"""The RPA schedule the vertex-flow kernel walks (spn_rpa_schedule, host only).

Decoding the schedule exactly as the kernel does and summing must reproduce, for every rid,
the reference's RPA lattice sum over getOverlap(rid) (SU2FrgCore.cpp:249-266); every index
must stay inside the arrays the kernel allocates for it; and the product encoding must spread
each half-warp's product reads over the shared-memory banks (distinct 8-byte words modulo
min(lanes, 16)) far better than the unordered pair list would.
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


def schedule(tab, lanes, products):
    lib = load_library()
    ip = C.POINTER(C.c_int)
    ptr, r1, r2 = (np.ascontiguousarray(x, np.int32) for x in (tab.overlap_ptr, tab.overlap_rid1, tab.overlap_rid2))
    info = np.zeros(4, np.int32)
    args = (tab.n_sites, ptr.ctypes.data_as(ip), r1.ctypes.data_as(ip), r2.ctypes.data_as(ip), lanes, int(products))
    check(lib.spn_rpa_schedule(*args, info.ctypes.data_as(ip), None, None, None, None))
    sched = np.zeros(info[3], np.int32)
    count = np.zeros(lanes, np.int32)
    base = np.zeros(lanes, np.int32)
    seg = np.zeros(tab.n_sites + 1, np.int32)
    check(lib.spn_rpa_schedule(*args, info.ctypes.data_as(ip), sched.ctypes.data_as(ip), count.ctypes.data_as(ip),
                               base.ctypes.data_as(ip), seg.ctypes.data_as(ip)))
    return info, sched, count, base, seg


def decode(tab, lanes, products, info, sched, count, base, seg, A, B):
    """The kernel's walk: per lane, accumulate m * A[a] * B[b], flush at segment ends."""
    nl = tab.n_sites
    L, n_seg = info[0], info[1]
    assert info[2] == int(products) and info[3] == L * lanes
    slots = np.zeros(n_seg)
    for l in range(lanes):
        assert 0 <= count[l] <= L
        acc, slot = 0.0, base[l]
        for i in range(count[l]):
            at = i * lanes + l
            if products:
                x = int(np.uint32(sched[at]))
                last = bool(x & (1 << 15))
                ab = x & 0x7FFF
                assert ab < nl * nl
                a, b = divmod(ab, nl)
                m = float(np.frombuffer(np.uint16(x >> 16).tobytes(), np.float16)[0])
            else:
                e = int(sched[at])
                a, b, m, last = e & 0x7F, (e >> 7) & 0x7F, float((e >> 14) & 0xFF), bool(e & (1 << 22))
            assert a < nl and b < nl and m >= 1
            acc += m * A[a] * B[b]
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
    wsite = 1 << max(0, (nl - 1).bit_length())
    lanes = wsite if nl <= 32 else 32
    encodings = [False, True] if nl <= 32 else [False]
    for products in encodings:
        s = schedule(tab, lanes, products)
        got = decode(tab, lanes, products, *s, A, B)
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)


def _conflicts(nl, lanes, L, ab, count):
    """Extra shared-memory wavefronts of the product reads: per step and half-warp, the
    largest number of lanes on one bank pair minus one.  ab[i * lanes + l] = product index."""
    hw = min(lanes, 16)
    extra = 0
    for i in range(L):
        for h0 in range(0, lanes, hw):
            keys = [int(ab[i * lanes + l]) % hw for l in range(h0, h0 + hw) if i < count[l]]
            if keys:
                extra += max(np.bincount(keys)) - 1
    return extra


@pytest.mark.parametrize("lat", [x for x in LATTICES if x[1] != 11], ids=lambda x: f"{x[0]}-r{x[1]}")
def test_product_schedule_spreads_banks(lat):
    tab = spn.Lattice(*lat).tables()
    nl = tab.n_sites
    lanes = 1 << max(0, (nl - 1).bit_length())
    info, sched, count, _, _ = schedule(tab, lanes, True)
    L = info[0]
    ordered = _conflicts(nl, lanes, L, sched.view(np.uint32) & 0x7FFF, count)
    # the factor encoding walks the pairs in the same order
    f = schedule(tab, lanes, False)[1]
    assert np.array_equal((f & 0x7F) * nl + ((f >> 7) & 0x7F), (sched.view(np.uint32) & 0x7FFF).astype(np.int64))
    # the same chunks in plain (rid, rid1, rid2) order
    ptr, r1, r2 = tab.overlap_ptr, tab.overlap_rid1, tab.overlap_rid2
    pairs = sorted({(r, a, b) for r in range(nl) for a, b in zip(r1[ptr[r]:ptr[r + 1]], r2[ptr[r]:ptr[r + 1]])})
    naive = np.zeros(L * lanes, np.int64)
    for l in range(lanes):
        for i, (_, a, b) in enumerate(pairs[l * L:(l + 1) * L]):
            naive[i * lanes + l] = a * nl + b
    baseline = _conflicts(nl, lanes, L, naive, count)
    print(f"{lat[0]} r{lat[1]}: extra wavefronts ordered {ordered} vs plain order {baseline}")
    assert ordered <= baseline
    if nl >= 8:
        assert ordered <= 0.5 * baseline
