"""Checkpoint and observable files (HDF5) written and read by the library, on the CPU.

The files must carry the reference's structure and libhdf5's encodings: the member skeleton
and encoding fingerprint of test/scripted/assets/test_reference1.ref are committed as a
fixture, and every file is also read back by an independent reader (tests/golden/h5lite.py,
itself checked against the reference's .ref files when the fixtures were made).
"""
import json
import os
import sys

import numpy as np
import pytest

import spinparser_gb300 as spn
from spinparser_gb300 import task

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
import h5lite  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _state(rng, n2=8, n4=1000):
    return (rng.standard_normal(n2).astype(np.float32), rng.standard_normal(n4).astype(np.float32),
            rng.standard_normal(n4).astype(np.float32))


def test_checkpoint_round_trip_ids_and_duplicates(tmp_path):
    p = str(tmp_path / "a.data")
    rng = np.random.default_rng(1)
    states = []
    for k in range(20):
        s = _state(rng)
        c = np.float32(10 * 0.9 ** k)
        assert task.write_checkpoint(p, c, *s, append=True) == k
        states.append((c, s))
    # same cutoff again: skipped, id -1, nothing written
    size = os.path.getsize(p)
    assert task.write_checkpoint(p, states[4][0], *states[4][1], append=True) == -1
    assert os.path.getsize(p) == size
    for k, (c, s) in enumerate(states):
        got = task.read_checkpoint(p, 8, 1000, k)
        assert got[0] == c and all(np.array_equal(a, b) for a, b in zip(got[1:], s))
    assert task.read_checkpoint(p, 8, 1000, -1)[0] == states[-1][0]
    assert task.read_checkpoint(p, 8, 1000, 20) is None
    # append=False truncates: one checkpoint, id 0
    assert task.write_checkpoint(p, states[0][0], *states[0][1], append=False) == 0
    assert h5lite.open_file(p).keys() == ["checkpoint_0"]


def test_checkpoint_layout_and_size_checks(tmp_path):
    p = str(tmp_path / "b.checkpoint")
    rng = np.random.default_rng(2)
    v2, ss, dd = _state(rng, 6, 300)
    task.write_checkpoint(p, 2.5, v2, ss, dd)
    f = h5lite.open_file(p)
    g = f["checkpoint_0"]
    assert g.keys() == ["cutoff", "v2", "v4dd", "v4ss"]
    assert float(g.attrs["cutoff"][0]) == 2.5 and float(g["cutoff"].read()[0]) == 2.5
    assert np.array_equal(g["v4dd"].read(), dd) and np.array_equal(g["v4ss"].read(), ss)
    with pytest.raises(spn.SpnError) as e:
        task.read_checkpoint(p, 6, 301)
    assert e.value.code == -2
    with pytest.raises(spn.SpnError) as e:
        task.read_checkpoint(str(tmp_path / "missing.checkpoint"), 6, 300)
    assert e.value.code == -4


def test_many_checkpoints_multilevel_btree(tmp_path):
    """More than 256 members need a second B-tree level (32 nodes x 8 symbols per leaf)."""
    p = str(tmp_path / "c.data")
    rng = np.random.default_rng(3)
    states = [_state(rng, 4, 16) for _ in range(300)]
    for k, s in enumerate(states):
        assert task.write_checkpoint(p, 50 * 0.99 ** k, *s, append=True) == k
    f = h5lite.open_file(p)
    assert len(f.keys()) == 300
    for k in (0, 255, 256, 299):
        assert np.array_equal(f[f"checkpoint_{k}/v4ss"].read(), states[k][1])
        got = task.read_checkpoint(p, 4, 16, k)
        assert np.array_equal(got[3], states[k][2])
    # appending rewrites only the root's metadata: the file stays within a small factor of its data
    data_bytes = 300 * (4 + 32 + 1) * 4
    assert os.path.getsize(p) < data_bytes + 300 * 40_000


def test_observable_file_structure_matches_reference(tmp_path):
    """An .obs written through the library has the member skeleton of the reference's
    test_reference1.ref (given the same lattice and cutoffs) and libhdf5's encodings."""
    ref = json.load(open(os.path.join(GOLDEN, "reference1_layout.json")))
    gold = np.load(os.path.join(GOLDEN, "reference1_su2.npz"))
    lat = spn.Lattice("hyperkagome", 3, "hyperkagome-heisenberg", {"j": "1.0"},
                      resource_dir=os.path.join(GOLDEN, "res_hyperkagome"))
    o = str(tmp_path / "r1.obs")
    for c, zz, dd in zip(gold["cutoffs"], gold["zz"], gold["dd"]):
        assert task.write_correlation(o, lat, float(c), zz, dd)
    assert h5lite.skeleton(o) == ref["skeleton"]
    assert h5lite.layout_fingerprint(o) == ref["fingerprint"]
    # values: meta from the package's lattice, data as written
    m = h5lite.open_file(o)["SU2CorZZ/meta"]
    np.testing.assert_allclose(m["sites"].read(), gold["sites"], atol=1e-6)
    np.testing.assert_allclose(m["basis"].read(), gold["basis"], atol=1e-6)
    np.testing.assert_allclose(m["latticeVectors"].read(), gold["lattice_vectors"], atol=1e-6)
    cut, zz = h5lite.read_correlations(o, "SU2CorZZ")
    assert np.array_equal(cut, gold["cutoffs"]) and np.array_equal(zz, gold["zz"])


def test_observable_duplicates_and_reopen(tmp_path):
    lat = spn.Lattice("square", 2, "square-heisenberg", {"j": "1"})
    n = lat.info.n_basis * lat.info.n_range
    o = str(tmp_path / "s.obs")
    rng = np.random.default_rng(4)
    vals = [(rng.standard_normal(n), rng.standard_normal(n)) for _ in range(5)]
    for k in range(3):
        assert task.write_correlation(o, lat, 4.0 - k, *vals[k])
    assert not task.write_correlation(o, lat, 3.0, *vals[4])  # duplicate cutoff: discarded
    for k in range(3, 5):  # a later call extends the existing file
        assert task.write_correlation(o, lat, 4.0 - k, *vals[k])
    cut, zz = h5lite.read_correlations(o, "SU2CorZZ")
    _, dd = h5lite.read_correlations(o, "SU2CorDD")
    assert cut.tolist() == [4.0, 3.0, 2.0, 1.0, 0.0]
    assert np.array_equal(zz.reshape(5, -1), np.array([v[0] for v in vals], np.float32))
    assert np.array_equal(dd.reshape(5, -1), np.array([v[1] for v in vals], np.float32))
    h5lite.compare(o, o)
