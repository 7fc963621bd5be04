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



def half_warp_wavefronts(nl, lanes, packed, width, entries):
    """Mean shared-memory wavefronts of one half warp's 64-bit reads of M per walk step: the
    largest number of distinct elements in one of the 16 bank pairs.  `entries(l, i)` gives the
    (rid1, rid2) lane l reads at step i, or None."""
    tot = steps = 0
    for h0 in range(0, lanes, 16):
        i = 0
        while True:
            per, any_ = {}, False
            for l in range(h0, h0 + 16):
                e = entries(l, i)
                if e is None:
                    continue
                any_ = True
                a, b = e
                elem = a * width + b if packed else a * 128 + b
                per.setdefault((a * width + b if packed else b) & 15, set()).add(elem)
            if not any_:
                break
            tot += max(len(v) for v in per.values())
            steps += 1
            i += 1
    return tot / steps


@pytest.mark.parametrize("lattice,rng,model,params,lanes", [
    ("cubic", 6, "cubic-j1j2heisenberg", {"j1": "1", "j2": "0.25"}, 32),
    ("pyrochlore", 7, "pyrochlore-j1j2heisenberg", {"j1": "1", "j2": "0.25"}, 256),
])
def test_schedule_orders_segments_against_bank_collisions(lattice, rng, model, params, lanes):
    """The entries inside each segment are ordered against bank collisions of the walk's reads of
    M: fewer wavefronts per half-warp step than the same chunks in (rid, rid1, rid2) order."""
    tab = spn.Lattice(lattice, rng, model, params).tables()
    nl = tab.n_sites
    info, sched, count, base, seg = schedule(tab, lanes)
    L, packed, width = int(info[0]), bool(info[3]), int(info[4])

    def ordered(l, i):
        if i >= count[l]:
            return None
        e = int(np.uint32(sched[i * lanes + l]))
        if packed:
            return divmod((e & 0xFFFF) // 8, width)
        return e & 0x7F, (e >> 7) & 0x7F
    ptr, r1, r2 = tab.overlap_ptr, tab.overlap_rid1, tab.overlap_rid2
    merged = [(r, a, b) for r in range(nl) for (a, b) in sorted(set(zip(r1[ptr[r]:ptr[r + 1]].tolist(),
                                                                        r2[ptr[r]:ptr[r + 1]].tolist())))]
    assert len(merged) == int(count.sum())

    def plain(l, i):
        j = l * L + i
        return merged[j][1:] if i < L and j < min(len(merged), (l + 1) * L) else None
    got = half_warp_wavefronts(nl, lanes, packed, width, ordered)
    before = half_warp_wavefronts(nl, lanes, packed, width, plain)
    assert got < 0.75 * before, (got, before)


# ---- the lane-balanced walk of the XYZ and TRI t channels (spn_rpa_lane_schedule) ----

# images of (X, Y, Z) under the six spin permutations (X,Y,Z) (X,Z,Y) (Y,X,Z) (Y,Z,X) (Z,X,Y) (Z,Y,X)
PERM_IMAGES = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]


def lane_words(tab, st, layout):
    """The site-ordered pair words of the XYZ (layout 1) or TRI (layout 2) kernel."""
    r1, r2 = np.asarray(tab.overlap_rid1), np.asarray(tab.overlap_rid2)
    p1, p2 = np.asarray(st.overlap_perm1), np.asarray(st.overlap_perm2)
    w = r1 | (r2 << 7)
    if layout == 1:
        return (w | (p1 << 14) | (p2 << 17)).astype(np.int32)
    img = lambda p, sh: sum(np.array([PERM_IMAGES[int(x)][q] for x in p]) << (sh + 2 * q) for q in range(3))  # noqa: E731
    return (w | img(p1, 14) | img(p2, 20)).astype(np.int32)


def lane_schedule(layout, tab, words):
    lib = load_library()
    ip = C.POINTER(C.c_int)
    ptr = np.ascontiguousarray(tab.overlap_ptr, np.int32)
    info = np.zeros(4, np.int32)
    args = (layout, tab.n_sites, ptr.ctypes.data_as(ip), words.ctypes.data_as(ip))
    check(lib.spn_rpa_lane_schedule(*args, info.ctypes.data_as(ip), None, None, None, None))
    sched = np.zeros(info[2], np.int32)
    count, base = np.zeros(32, np.int32), np.zeros(32, np.int32)
    seg = np.zeros(tab.n_sites + 1, np.int32)
    check(lib.spn_rpa_lane_schedule(*args, info.ctypes.data_as(ip), sched.ctypes.data_as(ip), count.ctypes.data_as(ip),
                                    base.ctypes.data_as(ip), seg.ctypes.data_as(ip)))
    return info, sched, count, base, seg


def walk_collisions(info, sched, count, nl, layout):
    """Extra shared-memory wavefronts of the walk under the kernel's bank model."""
    L, last = int(info[0]), 1 << int(info[3])
    if layout == 1:
        reads, group = 2, 8
        bank = lambda e, k: ((((e >> 14) & 7) * nl + (e & 127)) if k == 0 else (((e >> 17) & 7) * nl + ((e >> 7) & 127)))  # noqa: E731
    else:
        reads, group = 32, 32

        def bank(e, k):
            f, a, b = k >> 4, (k >> 2) & 3, k & 3
            rid, sh = ((e >> 7) & 127, 20) if f else (e & 127, 14)
            pa = 3 if a == 3 else (e >> (sh + 2 * a)) & 3
            pb = 3 if b == 3 else (e >> (sh + 2 * b)) & 3
            return (4 * pa + pb) * nl + rid
    nb = 8 if layout == 1 else 32
    extra = 0
    for g0 in range(0, 32, group):
        for i in range(L):
            for k in range(reads):
                per = {}
                for l in range(g0, g0 + group):
                    if i < count[l]:
                        addr = bank(int(sched[i * 32 + l]) & (last - 1), k)
                        per.setdefault(addr % nb, set()).add(addr)
                extra += sum(len(v) - 1 for v in per.values())
    return extra


@pytest.mark.parametrize("layout,lattice,rng,model,params,gain", [
    (1, "honeycomb", 9, "honeycomb-kitaev", {"j": "0.1", "k": "-1.0"}, 0.3),
    (2, "honeycomb", 9, "honeycomb-kitaev-gamma", {"j": "0.2", "k": "1.0", "g": "-0.1"}, 0.3),
    (1, "pyrochlore", 3, "pyrochlore-heisenberg", {"j": "1"}, 0.5),
])
def test_lane_schedule_covers_every_pair_and_orders_against_banks(layout, lattice, rng, model, params, gain):
    """Every site's pairs appear exactly once, in runs of that site only, whose slots the site
    sums in order; the bank-ordered walk has well below the collisions of the same chunks
    unordered."""
    lat = spn.Lattice(lattice, rng, model, params)
    tab, st = lat.tables(), lat.spin_tables()
    nl, ptr = tab.n_sites, np.asarray(tab.overlap_ptr)
    words = lane_words(tab, st, layout)
    info, sched, count, base, seg = lane_schedule(layout, tab, words)
    L, n_seg, last = int(info[0]), int(info[1]), 1 << int(info[3])
    assert info[2] == 32 * L and count.sum() == len(words) and count.max() - count.min() <= L
    runs = [[] for _ in range(n_seg)]
    for l in range(32):
        slot = int(base[l])
        for i in range(int(count[l])):
            e = int(sched[i * 32 + l])
            runs[slot].append(e & (last - 1))
            if e & last:
                slot += 1
        assert slot == (base[l + 1] if l < 31 else n_seg)
    assert seg[0] == 0 and seg[nl] == n_seg and np.all(np.diff(seg) >= 0)
    for j in range(nl):
        got = sorted(e for q in range(seg[j], seg[j + 1]) for e in runs[q])
        assert got == sorted(words[ptr[j]:ptr[j + 1]].tolist()), j
    plain = lane_schedule(0, tab, words)
    assert walk_collisions(info, sched, count, nl, layout) < gain * walk_collisions(*plain[:3], nl, layout)
