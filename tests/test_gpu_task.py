"""Task files run end to end on the GPU through the driver (SpinParser::run), with the
reference's scripted tests as the model (test/scripted/test_*.sh):

  * test_reference1 / test_referenceFail: the hyperkagome task reproduces the golden .obs
    of the reference (structure exact, values within the evaluator's 1e-5), and J = -1 does not;
  * test_pythonObs: the honeycomb task's .obs answers the reference's obs.py queries;
  * test_checkpoint: a calculation stopped at a larger cutoff and resumed from its checkpoint
    with an extended cutoff list writes the same .obs as an uninterrupted run;
  * test_defer: deferred measurements (method="defer" or --defer), evaluated in the
    post-processing stage from the .data archive, write the same .obs as direct ones.
"""
import json
import os
import re

import numpy as np
import pytest

from spinparser_gb300 import task
from taskfiles import exponential_cutoffs, manual_frequencies, write

import h5lite

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
REF_RES = os.path.join(GOLDEN, "res_hyperkagome")
HONEYCOMB = dict(lattice="honeycomb", rng=3, model="honeycomb-heisenberg")


def reference1_task(tmp_path, j="1.0", name="r1.xml"):
    g = np.load(os.path.join(GOLDEN, "reference1_su2.npz"))
    cmax, cmin, step = (float(x) for x in g["cutoff_spec"])
    return write(tmp_path, name, lattice="hyperkagome", rng=3, model="hyperkagome-heisenberg", params=f"<j>{j}</j>",
                 freq=manual_frequencies(), cutoff=exponential_cutoffs(f"{cmax:g}", f"{cmin:g}", f"{step:g}")), g


def status_of(task_path):
    m = re.search(r'status="(\w+)"', open(task_path).read())
    return m.group(1) if m else None


def test_reference1_task_reproduces_golden_obs(tmp_path):
    p, g = reference1_task(tmp_path)
    s = task.run_task(p, resource_path=REF_RES, verbose=-1)
    assert s.status == "finished" and not s.diverged and s.steps == len(g["cutoffs"]) - 1
    assert status_of(p) == "finished"
    obs = str(tmp_path / "r1.obs")
    layout = json.load(open(os.path.join(GOLDEN, "reference1_layout.json")))
    assert h5lite.skeleton(obs) == layout["skeleton"]
    assert h5lite.layout_fingerprint(obs) == layout["fingerprint"]
    for group, key in (("SU2CorZZ", "zz"), ("SU2CorDD", "dd")):
        cut, data = h5lite.read_correlations(obs, group)
        assert np.array_equal(cut, g["cutoffs"])
        assert float(np.abs(data - g[key]).max()) < 1e-5, group
        meta = h5lite.open_file(obs)[group + "/meta"]
        assert float(np.abs(meta["sites"].read() - g["sites"]).max()) < 1e-5
        assert float(np.abs(meta["basis"].read() - g["basis"]).max()) < 1e-5
        assert float(np.abs(meta["latticeVectors"].read() - g["lattice_vectors"]).max()) < 1e-5
    # a finished task has nothing left to do
    assert task.run_task(p, resource_path=REF_RES, verbose=-1).steps == 0


def test_reference_fail_task_differs_from_golden(tmp_path):
    p, g = reference1_task(tmp_path, j="-1.0")
    task.run_task(p, resource_path=REF_RES, verbose=-1)
    cut, zz = h5lite.read_correlations(str(tmp_path / "r1.obs"), "SU2CorZZ")
    n = min(len(cut), len(g["cutoffs"]))
    assert float(np.abs(zz[:n] - g["zz"][:n]).max()) > 1e-5


def test_python_obs_task(tmp_path):
    """test_pythonObs.sh: honeycomb r3 through the driver; the .obs answers obs.py's queries."""
    import spinparser_gb300 as spn
    from obs_queries import evaluate_query

    spec = json.load(open(os.path.join(GOLDEN, "python_obs_honeycomb.json")))
    t = spec["task"]
    p = write(tmp_path, "po.xml", lattice=t["lattice"], rng=t["range"], model=t["model"], params=f"<j>{t['j']}</j>",
              freq=manual_frequencies(t["frequencies"]),
              cutoff=exponential_cutoffs(t["cutoff_max"], t["cutoff_min"], t["cutoff_step"]))
    task.run_task(p, verbose=-1)
    cut, zz = h5lite.read_correlations(str(tmp_path / "po.obs"), "SU2CorZZ")
    tab = spn.Lattice(t["lattice"], t["range"], t["model"], {"j": str(t["j"])}).tables()
    for q in spec["queries"]:
        got = evaluate_query(q, cut, zz, tab)
        atol = 1e-16
        if q["what"] == "structure_factor":
            atol = 1e-5 * float(np.max(evaluate_query(q, cut, np.abs(zz), tab)))
        assert np.isclose(got, np.array(q["expect"]), rtol=1e-5, atol=atol).all(), q["what"]


def test_checkpoint_resume_equals_uninterrupted_run(tmp_path):
    """test_checkpoint.sh: run to cutoff 0.5, then resume (status running) down to 0.3."""
    full = write(tmp_path, "full.xml", cutoff=exponential_cutoffs(10, 0.3, 0.9), freq=manual_frequencies(), **HONEYCOMB)
    part = write(tmp_path, "part.xml", cutoff=exponential_cutoffs(10, 0.5, 0.9), freq=manual_frequencies(), **HONEYCOMB)
    task.run_task(full, force_restart=True, verbose=-1)
    first = task.run_task(part, force_restart=True, verbose=-1)
    assert first.status == "finished"
    # rewrite the task with the longer cutoff list and a "running" calculation log
    write(tmp_path, "part.xml", cutoff=exponential_cutoffs(10, 0.3, 0.9), freq=manual_frequencies(), **HONEYCOMB,
          extra='<calculation status="running" startTime="1970-Jan-01 00:00:00" checkpointTime="1970-Jan-01 00:00:00" />')
    second = task.run_task(part, verbose=-1)
    assert second.status == "finished" and 0 < second.steps < first.steps
    assert status_of(part) == "finished"
    a, b = str(tmp_path / "full.obs"), str(tmp_path / "part.obs")
    h5lite.compare(a, b, tolerance=1e-5)
    # the device arithmetic is deterministic: the resumed run is bit-identical
    for group in ("SU2CorZZ", "SU2CorDD"):
        ca, da = h5lite.read_correlations(a, group)
        cb, db = h5lite.read_correlations(b, group)
        assert np.array_equal(ca, cb) and np.array_equal(da, db)
    # the final checkpoint holds the state at the last cutoff
    ck = h5lite.open_file(str(tmp_path / "part.checkpoint"))
    assert ck.keys() == ["checkpoint_0"]
    cut = np.float32(10.0)
    while np.float32(cut * np.float32(0.9)) > np.float32(0.3):
        cut = np.float32(cut * np.float32(0.9))
    assert float(ck["checkpoint_0"].attrs["cutoff"][0]) == float(cut)


def test_periodic_checkpoints_keep_status_running(tmp_path):
    """--checkpointTime 0 writes a checkpoint (and a 'running' status) whenever a second
    has passed; the end of the run records 'finished' and the final state."""
    p = write(tmp_path, "pc.xml", cutoff=exponential_cutoffs(10, 0.3, 0.9), freq=manual_frequencies(), **HONEYCOMB)
    s = task.run_task(p, checkpoint_time=0, verbose=-1)
    assert s.status == "finished" and status_of(p) == "finished"
    calc = re.search(r"<calculation[^>]*>", open(p).read()).group(0)
    assert all(k in calc for k in ("startTime=", "checkpointTime=", "endTime="))


@pytest.mark.parametrize("how", ["method", "option"])
def test_deferred_measurements_equal_direct_ones(tmp_path, how):
    """test_defer.sh: deferred measurements archive the vertex at every cutoff (.data) and
    evaluate it in a second, post-processing run."""
    direct = write(tmp_path, "nd.xml", freq=manual_frequencies(), **HONEYCOMB)
    meas = '<measurements><measurement name="correlation" method="defer" /></measurements>'
    deferred = write(tmp_path, "d.xml", freq=manual_frequencies(), **HONEYCOMB,
                     measurements=meas if how == "method" else
                     '<measurements><measurement name="correlation" /></measurements>')
    task.run_task(direct, force_restart=True, verbose=-1)
    s1 = task.run_task(deferred, force_restart=True, defer=(how == "option"), verbose=-1)
    assert s1.status == "postprocessing" and s1.measurements == 0
    assert status_of(deferred) == "postprocessing"
    assert not os.path.exists(str(tmp_path / "d.obs"))
    archive = h5lite.open_file(str(tmp_path / "d.data"))
    assert len(archive.keys()) == s1.steps + 1
    s2 = task.run_task(deferred, defer=(how == "option"), verbose=-1)
    assert s2.status == "finished" and s2.steps == 0 and s2.measurements == s1.steps + 1
    assert status_of(deferred) == "finished"
    h5lite.compare(str(tmp_path / "nd.obs"), str(tmp_path / "d.obs"), tolerance=1e-5)
    for group in ("SU2CorZZ", "SU2CorDD"):
        ca, da = h5lite.read_correlations(str(tmp_path / "nd.obs"), group)
        cb, db = h5lite.read_correlations(str(tmp_path / "d.obs"), group)
        assert np.array_equal(ca, cb) and np.array_equal(da, db)


def test_measurement_cutoff_window_and_fp64_self_energy(tmp_path):
    meas = '<measurements><measurement name="correlation" minCutoff="1.0" maxCutoff="5.0" /></measurements>'
    p = write(tmp_path, "w.xml", freq=manual_frequencies(), measurements=meas, **HONEYCOMB)
    task.run_task(p, verbose=-1, fp64_self_energy=True)
    cut, _ = h5lite.read_correlations(str(tmp_path / "w.obs"), "SU2CorZZ")
    assert len(cut) > 0 and cut.max() <= 5.0 and cut.min() >= 1.0


# ---------------------------------------------------------------------------------------
# XYZ core through the driver (test_reference2.sh, XYZ task)
# ---------------------------------------------------------------------------------------
REF2_RES = os.path.join(GOLDEN, "res_hyperhoneycomb")


def reference2_task(tmp_path, name="r2.xml", cutoff=None, extra=""):
    g = np.load(os.path.join(GOLDEN, "reference2_xyz.npz"))
    cmax, cmin, step = (float(x) for x in g["cutoff_spec"])
    cut = cutoff or exponential_cutoffs(f"{cmax:g}", f"{cmin:g}", f"{step:g}")
    return write(tmp_path, name, lattice="hyperhoneycomb", rng=3, model="hyperhoneycomb-kitaev", symmetry="XYZ",
                 params=f"<j>{float(g['j']):g}</j><k>{float(g['k']):g}</k>", freq=manual_frequencies(), cutoff=cut,
                 extra=extra), g


def test_reference2_xyz_task_reproduces_golden_obs(tmp_path):
    p, g = reference2_task(tmp_path)
    s = task.run_task(p, resource_path=REF2_RES, verbose=-1)
    assert s.status == "finished" and not s.diverged and s.steps == len(g["cutoffs"]) - 1
    obs = str(tmp_path / "r2.obs")
    layout = json.load(open(os.path.join(GOLDEN, "reference2_layout.json")))
    assert h5lite.skeleton(obs) == layout["skeleton"]
    assert h5lite.layout_fingerprint(obs) == layout["fingerprint"]
    for group, key in (("XYZCorXX", "xx"), ("XYZCorYY", "yy"), ("XYZCorZZ", "zz"), ("XYZCorDD", "dd")):
        cut, data = h5lite.read_correlations(obs, group)
        assert np.array_equal(cut, g["cutoffs"])
        assert float(np.abs(data - g[key]).max()) < 1e-5, group
    # the checkpoint holds the XYZ arrays in the reference's order
    ck = h5lite.open_file(str(tmp_path / "r2.checkpoint"))["checkpoint_0"]
    assert ck.keys() == ["cutoff", "v2", "v4dd", "v4xx", "v4yy", "v4zz"]


def test_reference2_xyz_sign_flip_fails_golden(tmp_path):
    """test_referenceFail.sh in XYZ form: k -> -k must not reproduce the golden values."""
    g = np.load(os.path.join(GOLDEN, "reference2_xyz.npz"))
    p = write(tmp_path, "f.xml", lattice="hyperhoneycomb", rng=3, model="hyperhoneycomb-kitaev", symmetry="XYZ",
              params=f"<j>{float(g['j']):g}</j><k>{-float(g['k']):g}</k>", freq=manual_frequencies(),
              cutoff=exponential_cutoffs("10", "0.3", "0.9"))
    task.run_task(p, resource_path=REF2_RES, verbose=-1)
    _, data = h5lite.read_correlations(str(tmp_path / "f.obs"), "XYZCorXX")
    assert float(np.abs(data - g["xx"]).max()) > 1e-3


def test_xyz_checkpoint_resume_equals_uninterrupted_run(tmp_path):
    full, _ = reference2_task(tmp_path, "full.xml")
    part, _ = reference2_task(tmp_path, "part.xml", cutoff=exponential_cutoffs("10", "0.5", "0.9"))
    task.run_task(full, resource_path=REF2_RES, force_restart=True, verbose=-1)
    first = task.run_task(part, resource_path=REF2_RES, force_restart=True, verbose=-1)
    assert first.status == "finished"
    reference2_task(tmp_path, "part.xml", extra='<calculation status="running" startTime="1970-Jan-01 00:00:00" '
                                                'checkpointTime="1970-Jan-01 00:00:00" />')
    second = task.run_task(part, resource_path=REF2_RES, verbose=-1)
    assert second.status == "finished" and 0 < second.steps < first.steps
    a, b = str(tmp_path / "full.obs"), str(tmp_path / "part.obs")
    for group in ("XYZCorXX", "XYZCorYY", "XYZCorZZ", "XYZCorDD"):
        ca, da = h5lite.read_correlations(a, group)
        cb, db = h5lite.read_correlations(b, group)
        assert np.array_equal(ca, cb) and np.array_equal(da, db)


# ---------------------------------------------------------------------------------------
# TRI core through the driver (test_reference3.sh; test_reference2.sh's TRI task)
# ---------------------------------------------------------------------------------------
REF3_RES = os.path.join(GOLDEN, "res_honeycomb")
TRI_GROUPS = ("TRICorXX", "TRICorXY", "TRICorXZ", "TRICorYX", "TRICorYY", "TRICorYZ", "TRICorZX", "TRICorZY",
              "TRICorZZ", "TRICorDD")


def reference3_task(tmp_path, name="r3.xml", cutoff=None, extra="", g_sign=1.0):
    g = np.load(os.path.join(GOLDEN, "reference3_tri.npz"))
    cmax, cmin, step = (float(x) for x in g["cutoff_spec"])
    cut = cutoff or exponential_cutoffs(f"{cmax:g}", f"{cmin:g}", f"{step:g}")
    params = f"<j>{float(g['j']):g}</j><k>{float(g['k']):g}</k><g>{g_sign * float(g['g']):g}</g>"
    return write(tmp_path, name, lattice="honeycomb", rng=3, model="honeycomb-kitaev-gamma", symmetry="TRI",
                 params=params, freq=manual_frequencies(), cutoff=cut, extra=extra), g


def test_reference3_tri_task_reproduces_golden_obs(tmp_path):
    p, g = reference3_task(tmp_path)
    s = task.run_task(p, resource_path=REF3_RES, verbose=-1)
    assert s.status == "finished" and not s.diverged and s.steps == len(g["cutoffs"]) - 1
    obs = str(tmp_path / "r3.obs")
    layout = json.load(open(os.path.join(GOLDEN, "reference3_layout.json")))
    assert h5lite.skeleton(obs) == layout["skeleton"]
    assert h5lite.layout_fingerprint(obs) == layout["fingerprint"]
    for group in TRI_GROUPS:
        cut, data = h5lite.read_correlations(obs, group)
        assert np.array_equal(cut, g["cutoffs"])
        assert float(np.abs(data - g[group[-2:].lower()]).max()) < 1e-5, group
    # the checkpoint holds the TRI vertex as one array (TRIEffectiveAction.hpp:146-148)
    ck = h5lite.open_file(str(tmp_path / "r3.checkpoint"))["checkpoint_0"]
    assert ck.keys() == ["cutoff", "v2", "v4"]


def test_reference3_tri_sign_flip_fails_golden(tmp_path):
    """test_referenceFail.sh in TRI form: g -> -g must not reproduce the golden values."""
    p, g = reference3_task(tmp_path, "f.xml", g_sign=-1.0)
    task.run_task(p, resource_path=REF3_RES, verbose=-1)
    _, data = h5lite.read_correlations(str(tmp_path / "f.obs"), "TRICorXY")
    assert float(np.abs(data - g["xy"]).max()) > 1e-3


def test_reference2_tri_task_reproduces_golden_obs(tmp_path):
    """test_reference2.sh's second task: the XYZ golden through the TRI core."""
    g = np.load(os.path.join(GOLDEN, "reference2_xyz.npz"))
    cmax, cmin, step = (float(x) for x in g["cutoff_spec"])
    p = write(tmp_path, "r2t.xml", lattice="hyperhoneycomb", rng=3, model="hyperhoneycomb-kitaev", symmetry="TRI",
              params=f"<j>{float(g['j']):g}</j><k>{float(g['k']):g}</k>", freq=manual_frequencies(),
              cutoff=exponential_cutoffs(f"{cmax:g}", f"{cmin:g}", f"{step:g}"))
    s = task.run_task(p, resource_path=REF2_RES, verbose=-1)
    assert s.status == "finished" and not s.diverged
    obs = str(tmp_path / "r2t.obs")
    for group, key in (("TRICorXX", "xx"), ("TRICorYY", "yy"), ("TRICorZZ", "zz"), ("TRICorDD", "dd")):
        cut, data = h5lite.read_correlations(obs, group)
        assert np.array_equal(cut, g["cutoffs"])
        assert float(np.abs(data - g[key]).max()) < 1e-5, group


def test_tri_checkpoint_resume_equals_uninterrupted_run(tmp_path):
    full, _ = reference3_task(tmp_path, "full.xml")
    part, _ = reference3_task(tmp_path, "part.xml", cutoff=exponential_cutoffs("10", "0.5", "0.9"))
    task.run_task(full, resource_path=REF3_RES, force_restart=True, verbose=-1)
    first = task.run_task(part, resource_path=REF3_RES, force_restart=True, verbose=-1)
    assert first.status == "finished"
    reference3_task(tmp_path, "part.xml", extra='<calculation status="running" startTime="1970-Jan-01 00:00:00" '
                                                'checkpointTime="1970-Jan-01 00:00:00" />')
    second = task.run_task(part, resource_path=REF3_RES, verbose=-1)
    assert second.status == "finished" and 0 < second.steps < first.steps
    a, b = str(tmp_path / "full.obs"), str(tmp_path / "part.obs")
    for group in TRI_GROUPS:
        ca, da = h5lite.read_correlations(a, group)
        cb, db = h5lite.read_correlations(b, group)
        assert np.array_equal(ca, cb) and np.array_equal(da, db)


def test_tri_deferred_measurements_equal_direct_ones(tmp_path):
    """test_defer.sh with the TRI core: the archived 16-component vertex (.data, dataset v4)
    evaluated in the post-processing run gives the direct run's ten groups."""
    direct, _ = reference3_task(tmp_path, "nd.xml", cutoff=exponential_cutoffs("10", "1", "0.8"))
    meas = '<measurements><measurement name="correlation" method="defer" /></measurements>'
    g = np.load(os.path.join(GOLDEN, "reference3_tri.npz"))
    params = f"<j>{float(g['j']):g}</j><k>{float(g['k']):g}</k><g>{float(g['g']):g}</g>"
    deferred = write(tmp_path, "d.xml", lattice="honeycomb", rng=3, model="honeycomb-kitaev-gamma", symmetry="TRI",
                     params=params, freq=manual_frequencies(), cutoff=exponential_cutoffs("10", "1", "0.8"),
                     measurements=meas)
    task.run_task(direct, resource_path=REF3_RES, force_restart=True, verbose=-1)
    s1 = task.run_task(deferred, resource_path=REF3_RES, force_restart=True, verbose=-1)
    assert s1.status == "postprocessing" and s1.measurements == 0
    archive = h5lite.open_file(str(tmp_path / "d.data"))
    assert len(archive.keys()) == s1.steps + 1
    assert archive[archive.keys()[0]].keys() == ["cutoff", "v2", "v4"]
    s2 = task.run_task(deferred, resource_path=REF3_RES, verbose=-1)
    assert s2.status == "finished" and s2.measurements == s1.steps + 1
    for group in TRI_GROUPS:
        ca, da = h5lite.read_correlations(str(tmp_path / "nd.obs"), group)
        cb, db = h5lite.read_correlations(str(tmp_path / "d.obs"), group)
        assert np.array_equal(ca, cb) and np.array_equal(da, db), group
