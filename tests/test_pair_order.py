"""Order of the RPA pairs the XYZ and TRI vertex kernels walk (host logic, no GPU): per site a
permutation of its overlap pairs, chosen so that the 32 sites of a warp read fewer colliding
shared-memory banks than in the lattice's own order."""
import ctypes as C
import os

import numpy as np
import pytest

import spinparser_gb300 as spn
from spinparser_gb300._capi import load_library

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def pair_order(layout, tab, st):
    lib = load_library()
    arrs = [np.ascontiguousarray(a, np.int32) for a in (tab.overlap_ptr, tab.overlap_rid1, tab.overlap_rid2,
                                                         st.overlap_perm1, st.overlap_perm2)]
    order = np.empty(tab.n_overlap, np.int32)
    coll = (C.c_longlong * 2)()
    p = [a.ctypes.data_as(C.POINTER(C.c_int)) for a in arrs]
    assert lib.spn_rpa_pair_order(layout, tab.n_sites, *p, order.ctypes.data_as(C.POINTER(C.c_int)), coll) == 0
    return order, coll[0], coll[1]


@pytest.mark.parametrize("layout", [0, 1])
@pytest.mark.parametrize("rng", [6, 11])
def test_order_is_a_per_site_permutation_with_fewer_collisions(layout, rng):
    lat = spn.Lattice("honeycomb", rng, "honeycomb-kitaev-gamma", {"j": "0.2", "k": "1.0", "g": "-0.1"},
                      resource_dir=os.path.join(GOLDEN, "res_honeycomb"))
    tab, st = lat.tables(), lat.spin_tables()
    order, natural, chosen = pair_order(layout, tab, st)
    for j in range(tab.n_sites):
        a, b = tab.overlap_ptr[j], tab.overlap_ptr[j + 1]
        assert sorted(order[a:b].tolist()) == list(range(a, b))
    assert chosen <= natural
    assert chosen < natural or natural == 0


def test_bad_pair_entries_are_rejected():
    lat = spn.Lattice("square", 3, "square-heisenberg", {"j": "1.0"})
    tab, st = lat.tables(), lat.spin_tables()
    st.overlap_perm1 = st.overlap_perm1.copy()
    st.overlap_perm1[0] = 7
    with pytest.raises(AssertionError):
        pair_order(1, tab, st)
