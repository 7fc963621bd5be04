"""Task-file driver on the CPU: parsing, validation and file handling of the reference's
TaskFileParser / SpinParser::run, exercised through paths that need no GPU (--debugLattice,
a finished task, and every error raised before the core is created)."""
import os

import pytest

import spinparser_gb300 as spn
from spinparser_gb300 import task
from spinparser_gb300.__main__ import main as cli_main

from taskfiles import write


def run_err(path, **kw):
    with pytest.raises(spn.SpnError) as e:
        task.run_task(path, verbose=-1, **kw)
    return e.value


def test_debug_lattice_writes_ldf_and_needs_no_device(tmp_path):
    p = write(tmp_path)
    before = open(p).read()
    s = task.run_task(p, debug_lattice=True, verbose=-1)
    assert s.status == "new" and s.steps == 0
    ldf = open(str(tmp_path / "t.ldf")).read()
    assert ldf.startswith("<lattice>") and "<site id=" in ldf
    # no outputs and the task file is untouched
    assert not os.path.exists(str(tmp_path / "t.obs")) and not os.path.exists(str(tmp_path / "t.checkpoint"))
    assert open(p).read() == before
    # the same .ldf as the lattice factory writes directly
    lat = spn.Lattice("square", 2, "square-heisenberg", {"j": "1.0"})
    lat.write_ldf(str(tmp_path / "direct.ldf"))
    assert open(str(tmp_path / "direct.ldf")).read() == ldf


@pytest.mark.parametrize("symmetry", ["SU2", "XYZ", "TRI"])
def test_every_core_identifier_is_accepted(tmp_path, symmetry):
    """FrgCoreFactory's identifiers (src/FrgCoreFactory.cpp:25-51); the lattice stage needs no
    device.  Every core accepts a normalization option."""
    s = task.run_task(write(tmp_path, symmetry=symmetry), debug_lattice=True, verbose=-1)
    assert s.status == "new"
    p = write(tmp_path, "n.xml", symmetry=symmetry, params="<j>1.0</j><normalization>2</normalization>")
    assert task.run_task(p, debug_lattice=True, verbose=-1).status == "new"


def test_cli_debug_lattice(tmp_path, capfd):
    p = write(tmp_path)
    assert cli_main(["--debugLattice", p]) == 0
    out = capfd.readouterr().out
    assert "Number of parametrized sites: " in out and "Lattice debug output complete" in out
    assert cli_main([str(tmp_path / "missing.xml")]) == 1


@pytest.mark.parametrize("kw,code,message", [
    (dict(freq='<frequency discretization="weird"><value>1</value></frequency>'), -3,
     "Unknown attribute value 'weird' (task.parameters.frequency.discretization)"),
    (dict(freq='<frequency discretization="exponential"><min>0.1</min><max>1</max></frequency>'), -3,
     "Missing parameter 'task.parameters.frequency.count'"),
    (dict(freq='<frequency discretization="exponential"><min>1</min><max>0.5</max><count>8</count></frequency>'), -3,
     "'task.parameters.frequency.max' must be greater than 'task.parameters.frequency.min'"),
    (dict(freq='<frequency discretization="manual"><value>1</value><value>1.0</value></frequency>'), -3,
     "Duplicate value in task.parameters.frequency.value"),
    (dict(cutoff='<cutoff discretization="exponential"><max>10</max><min>1</min><step>1.5</step></cutoff>'), -3,
     "'task.parameters.cutoff.step' must be in the range (0,1)"),
    (dict(cutoff='<cutoff discretization="exponential" bogus="1"><max>10</max><min>1</min><step>0.5</step></cutoff>'), -3,
     "Unknown attribute 'task.parameters.cutoff.bogus'"),
    (dict(extra="<surprise/>"), -3, "Unknown parameter 'task.surprise'"),
    (dict(measurements='<measurements><measurement name="magnetization" /></measurements>'), -3,
     "Measurement: Unknown measurement type 'magnetization'."),
    (dict(params="<j>1.0</j><colour>red</colour>"), -3, "Unknown spin model option 'colour'."),
    (dict(params=""), -3, "Interaction parameter 'j' is not defined in the taskfile"),
    (dict(symmetry="U1"), -2, "Spin model identifier 'U1' does not exist."),
    (dict(symmetry="su2"), -2, "Spin model identifier 'su2' does not exist."),
    # the XYZ and TRI cores take only a normalization (XYZFrgCore.cpp:19-28, TRIFrgCore.cpp:19-28)
    (dict(symmetry="TRI", params="<j>1.0</j><spin>0.5</spin>"), -3, "Unknown spin model option 'spin'."),
    (dict(symmetry="XYZ", params="<j>1.0</j><spin>0.5</spin>"), -3, "Unknown spin model option 'spin'."),
    (dict(lattice="nonexistent"), -3, "nonexistent"),
])
def test_task_validation_errors(tmp_path, kw, code, message):
    err = run_err(write(tmp_path, **kw), debug_lattice=True)
    assert err.code == code, err
    assert message in str(err), err


def test_existing_outputs_need_force_restart(tmp_path):
    p = write(tmp_path)
    for ext, what in (("checkpoint", "Checkpoint"), ("data", "Data"), ("obs", "Observable")):
        f = tmp_path / f"t.{ext}"
        f.write_bytes(b"old")
        err = run_err(p, debug_lattice=True)
        assert err.code == -4 and f"{what} file [" in str(err) and "--forceRestart" in str(err)
        task.run_task(p, debug_lattice=True, force_restart=True, verbose=-1)
        assert not f.exists()


def test_measurement_output_path_is_relative_to_task(tmp_path):
    p = write(tmp_path, measurements='<measurements><measurement name="correlation" output="other.obs" '
                                     'minCutoff="0.5" maxCutoff="5" method="defer"/></measurements>')
    (tmp_path / "other.obs").write_bytes(b"old")
    assert run_err(p, debug_lattice=True).code == -4
    (tmp_path / "t.obs").write_bytes(b"unrelated")  # not this task's output: left alone
    task.run_task(p, debug_lattice=True, force_restart=True, verbose=-1)
    assert not (tmp_path / "other.obs").exists() and (tmp_path / "t.obs").exists()


def test_finished_task_does_nothing(tmp_path, capfd):
    extra = '<calculation startTime="2020-Jan-01 00:00:00" checkpointTime="2020-Jan-01 00:10:00" ' \
            'endTime="2020-Jan-01 01:00:00" status="finished" />'
    p = write(tmp_path, extra=extra)
    s = task.run_task(p)
    assert s.status == "finished" and s.steps == 0
    assert "Nothing left to do" in capfd.readouterr().out


@pytest.mark.parametrize("calc,message", [
    ('<calculation status="running" />', "Checkpoint is corrupted [start time is not specified]."),
    ('<calculation status="finished" startTime="2020-01-01 00:00:00" checkpointTime="2020-01-01 00:00:00" />',
     "end time is not specified"),
    ('<calculation status="running" startTime="yesterday" />', "Invalid timestamp 'yesterday'."),
    ('<calculation status="paused" startTime="2020-Jan-01 00:00:00" />', "Checkpoint is corrupted"),
])
def test_corrupt_calculation_status(tmp_path, calc, message):
    err = run_err(write(tmp_path, extra=calc))
    assert err.code == -3 and message in str(err), err
