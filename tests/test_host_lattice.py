"""Host lattice factory and discretisations (CPU only), against the reference's known
answers: test/test_Lattice.cpp (square and honeycomb, range 3) and the grid formulas of
src/TaskFileParser.cpp:107-198."""
import json
import os
import shutil

import numpy as np
import pytest

import spinparser_gb300 as spn

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KATS = json.load(open(os.path.join(GOLDEN, "lattice_kats.json")))


@pytest.fixture(scope="module")
def anisotropic_honeycomb_res(tmp_path_factory):
    """Resource dir with the honeycomb fixture model of test_Lattice.cpp:47-66
    (bond-dependent xx / yy / zz couplings, which lower the symmetry)."""
    d = tmp_path_factory.mktemp("res")
    shutil.copy(os.path.join(spn.RES_DIR, "lattices.xml"), d / "lattices.xml")
    (d / "models.xml").write_text(
        '<model name="honeycomb-kat">\n'
        '<interaction parameter="a" from="0,0,0,0" to="0,0,0,1" type="xx" />\n'
        '<interaction parameter="b" from="0,0,0,0" to="0,-1,0,1" type="yy" />\n'
        '<interaction parameter="c" from="0,0,0,0" to="-1,0,0,1" type="zz" />\n'
        '</model>\n')
    return str(d)


def _lattice(name, res):
    if name.startswith("Square"):
        return spn.Lattice("square", 3, "square-heisenberg", {"j": "1.0"})
    return spn.Lattice("honeycomb", 3, "honeycomb-kat", {"a": "0.1", "b": "0.2", "c": "0.2"}, resource_dir=res)


@pytest.mark.parametrize("prefix", ["Square", "Honeycomb"])
def test_lattice_counts(prefix, anisotropic_honeycomb_res):
    lat = _lattice(prefix, anisotropic_honeycomb_res)
    kat = KATS[prefix + "LatticeIterate"]
    assert lat.info.n_range == kat["n_in_range"]
    assert lat.info.n_sites == kat["size"]
    sites, _ = lat.sites()
    assert tuple(sites[0]) == (0, 0, 0, 0)


@pytest.mark.parametrize("prefix", ["Square", "Honeycomb"])
def test_lattice_symmetry_table(prefix, anisotropic_honeycomb_res):
    lat = _lattice(prefix, anisotropic_honeycomb_res)
    sites, pairs = lat.sites(with_pairs=True)
    index = {tuple(s): i for i, s in enumerate(sites.tolist())}
    lists = KATS[prefix + "LatticeSymmetry"]["lists"]
    for a, b, t in zip(lists["i1List"], lists["i2List"], lists["targetList"]):
        assert pairs[index[tuple(a)], index[tuple(b)]] == pairs[0, index[tuple(t)]]


@pytest.mark.parametrize("prefix", ["Square", "Honeycomb"])
def test_lattice_overlap(prefix, anisotropic_honeycomb_res):
    lat = _lattice(prefix, anisotropic_honeycomb_res)
    sites, pairs = lat.sites(with_pairs=True)
    index = {tuple(s): i for i, s in enumerate(sites.tolist())}
    tab = lat.tables()
    kat = KATS[prefix + "LatticeOverlap"]
    rid = pairs[0, index[tuple(kat["overlap_site"])]]
    lo, hi = tab.overlap_ptr[rid], tab.overlap_ptr[rid + 1]
    assert hi - lo == kat["overlap_size"]
    expected = [(pairs[0, index[tuple(a)]], pairs[0, index[tuple(b)]])
                for a, b in zip(kat["lists"]["i1List"], kat["lists"]["i2List"])]
    got = list(zip(tab.overlap_rid1[lo:hi].tolist(), tab.overlap_rid2[lo:hi].tolist()))
    assert sorted(got) == sorted(expected)


def test_representatives_and_tables_are_consistent():
    tab = spn.Lattice("cubic", 4, "cubic-j1j2heisenberg", {"j1": "1", "j2": "0.25"}).tables()
    assert np.array_equal(tab.sites_rid, np.arange(tab.n_sites))
    assert tab.overlap_rid1.min() >= 0 and tab.overlap_rid1.max() < tab.n_sites
    assert tab.overlap_rid2.min() >= 0 and tab.overlap_rid2.max() < tab.n_sites
    assert tab.range_rid[0] == 0 and tab.range_inv_rid[0] == 0
    # the origin's coupling to its nearest neighbours and J2 neighbours
    assert sorted(set(tab.interaction_J[:, 0, 0].tolist())) == [0.25, 1.0]


@pytest.mark.parametrize("lattice,rng,model,params,nl,nr,so", [
    ("square", 3, "square-heisenberg", {"j": 1}, 6, 25, 94),
    ("square", 7, "square-j1j2heisenberg", {"j1": 1, "j2": 0.5}, 20, 113, 1340),
    ("cubic", 6, "cubic-j1j2heisenberg", {"j1": 1, "j2": 0.25}, 23, 377, 4095),
    ("pyrochlore", 5, "pyrochlore-heisenberg", {"j": 1}, 31, 277, 4156),
])
def test_benchmark_lattice_sizes(lattice, rng, model, params, nl, nr, so):
    """Sizes of the benchmark configurations (Nl, sites in range, RPA pairs)."""
    lat = spn.Lattice(lattice, rng, model, params)
    assert (lat.info.n_sites, lat.info.n_range, lat.info.n_overlap) == (nl, nr, so)


def test_number_syntax_of_unit_cells():
    tab = spn.Lattice("honeycomb", 1, "honeycomb-heisenberg", {"j": "1/2"}).tables()
    assert tab.lattice_vectors[0, 1] == np.sqrt(3.0) / 2
    assert tab.lattice_vectors[1, 1] == -np.sqrt(3.0) / 2
    assert np.float32(tab.interaction_J[0, 0, 0]) == np.float32(0.5)


def parse_number(text):
    import ctypes as C
    from spinparser_gb300._capi import check, load_library
    v = C.c_double()
    check(load_library().spn_parse_number(text.encode(), C.byref(v)))
    return v.value


@pytest.mark.parametrize("text,value", [
    ("1.5*3.9", 1.5 * 3.9), ("1.5/3.9", 1.5 / 3.9), ("-1.5*3.9", -1.5 * 3.9), ("-1.5/3.9", -1.5 / 3.9),
    ("1.5*3.9/2.1", 1.5 * 3.9 / 2.1), ("1.5/3.9*2.1", 1.5 / 3.9 * 2.1), ("-1.5*3.9/2.1", -1.5 * 3.9 / 2.1),
    ("-1.5/3.9*2.1", -1.5 / 3.9 * 2.1), ("-1.5*sqrt(3.9)/2.1", -1.5 * np.sqrt(3.9) / 2.1),
    ("0.25", 0.25), ("-2", -2.0), ("sqrt(2)", np.sqrt(2.0)),
])
def test_number_syntax(text, value):
    """test/test_InputParser.cpp:8-37: stringToDouble equals the double arithmetic exactly and
    stringToFloat within 1e-4 %."""
    assert parse_number(text) == value
    assert np.float32(parse_number(text)) == pytest.approx(value, rel=1e-6)


def test_number_syntax_rejects_garbage():
    with pytest.raises(spn.SpnError):
        parse_number("one half")


def test_cutoff_grid_is_repeated_float_multiplication():
    got = spn.cutoff_exponential(50.0, 0.05, 0.98)
    exp, v = [], np.float32(50.0)
    while v > np.float32(0.05):
        exp.append(v)
        v = np.float32(v * np.float32(0.98))
    assert np.array_equal(got, np.array(exp, np.float32))
    assert len(got) == 342


def test_frequency_grid_matches_exponential_formula():
    got = spn.frequency_exponential(0.005, 50.0, 32)
    assert got[0] == np.float32(0.005)
    assert abs(got[-1] - 50.0) <= 1e-4 * 50
    assert np.all(np.diff(got) > 0)
    ratio = got[1:] / got[:-1]
    assert np.allclose(ratio, ratio[0], rtol=1e-5)


def test_bad_inputs_raise_typed_errors():
    with pytest.raises(spn.SpnError) as e:
        spn.Lattice("no-such-lattice", 3, "square-heisenberg", {"j": 1})
    assert e.value.code == -3
    with pytest.raises(spn.SpnError) as e:
        spn.Lattice("square", 3, "square-heisenberg", {})
    assert "not defined" in str(e.value)
    with pytest.raises(spn.SpnError):
        spn.cutoff_exponential(1.0, 2.0, 0.5)
    with pytest.raises(spn.SpnError):
        spn.frequency_exponential(-1.0, 2.0, 4)
