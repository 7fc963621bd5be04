"""Regenerates the golden fixtures under tests/golden/ from the SpinParser reference tree.

Run in a checkout where the reference sources are available:
    python tests/golden/make_fixtures.py /path/to/SpinParser

Outputs (committed, so the tests need no reference tree at run time):
  reference1_su2.npz      golden SU(2) correlations of test/scripted/test_reference1.sh
                          (hyperkagome r=3, 14 manual frequencies, cutoff 10 -> 0.3 x0.9),
                          read from test/scripted/assets/test_reference1.ref, plus the task's
                          frequency list and cutoff specification parsed from the script
  hyperkagome_r3_tables.npz  lattice tables of that task, built by this package's lattice
                          factory from the reference's res/ unit cell and model
  python_obs_honeycomb.json  the numeric expectations of test/scripted/assets/test_python_obs.py
                          (honeycomb r=3 SU(2) run of test_pythonObs.sh) and the task parameters
  reference1_layout.json  member structure and HDF5 encoding fingerprint of test_reference1.ref
  res_hyperkagome/        the hyperkagome unit cell and Heisenberg model of the reference's
                          res/ files (the input of test_reference1), so that the task-file
                          driver can run that task end to end
  reference2_xyz.npz      golden XYZ-core correlations of test/scripted/test_reference2.sh
                          (hyperhoneycomb r=3 Heisenberg-Kitaev j=0.1, k=-1, 14 manual
                          frequencies, cutoff 10 -> 0.3 x0.9), read from
                          test/scripted/assets/test_reference2.ref (XYZCorXX/YY/ZZ/DD)
  reference2_layout.json  member structure and HDF5 encoding fingerprint of test_reference2.ref
  res_hyperhoneycomb/     the hyperhoneycomb unit cell and Heisenberg-Kitaev model of the
                          reference's res/ files (the input of test_reference2)

  reference3_tri.npz      golden TRI-core correlations of test/scripted/test_reference3.sh
                          (honeycomb r=3 Heisenberg-Kitaev-Gamma j=0.2, k=1, g=-0.1, 14 manual
                          frequencies, cutoff 10 -> 0.3 x0.9), read from
                          test/scripted/assets/test_reference3.ref (TRICorXX ... TRICorDD)
  reference3_layout.json  member structure and HDF5 encoding fingerprint of test_reference3.ref
  res_honeycomb/          the honeycomb unit cell and Heisenberg-Kitaev-Gamma model of the
                          reference's res/ files (the input of test_reference3)

`python tests/golden/make_fixtures.py <reference root> reference2` (or `reference3`)
regenerates only the fixtures of that script.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import h5lite  # noqa: E402


def task_parameters(script: str) -> dict:
    freq = [float(x) for x in re.findall(r"<value>([0-9.]+)</value>", script)]
    cmax = float(re.search(r"<max>([0-9.]+)</max>", script).group(1))
    cmin = float(re.search(r"<min>([0-9.]+)</min>", script).group(1))
    step = float(re.search(r"<step>([0-9.]+)</step>", script).group(1))
    lat = re.search(r'<lattice name="([^"]+)" range="(\d+)"', script)
    model = re.search(r'<model name="([^"]+)"', script)
    j = float(re.search(r"<j>([-0-9.]+)</j>", script).group(1))
    return {"frequencies": sorted(freq), "cutoff_max": cmax, "cutoff_min": cmin, "cutoff_step": step,
            "lattice": lat.group(1), "range": int(lat.group(2)), "model": model.group(1), "j": j}


def lattice_kats(src: str) -> dict:
    """Site lists and counts of test/test_Lattice.cpp, per test case."""
    out = {}
    cases = re.split(r"BOOST_FIXTURE_TEST_CASE\(", src)[1:]
    for case in cases:
        name = case.split(",")[0].strip()
        lists = {}
        for lname, body in re.findall(r"std::vector<SiteParameters> (\w+) = \{(.*?)\};", case, re.S):
            lists[lname] = [[int(x) for x in t.split(",")] for t in re.findall(r"SiteParameters\(([-0-9, ]+)\)", body)]
        entry = {"lists": lists}
        m = re.search(r"getOverlap\(l->symmetryTransform\(l->zero\(\), fromParameters\(SiteParameters\(([-0-9, ]+)\)\)\)\)", case)
        if m:
            entry["overlap_site"] = [int(x) for x in m.group(1).split(",")]
            entry["overlap_size"] = int(re.search(r"BOOST_CHECK_EQUAL\(o\.size, (\d+)\)", case).group(1))
        m = re.search(r"BOOST_CHECK_EQUAL\(n, (\d+)\);\s*BOOST_CHECK_EQUAL\(l->size, (\d+)\)", case)
        if m:
            entry["n_in_range"], entry["size"] = int(m.group(1)), int(m.group(2))
        out[name] = entry
    return out


def extract_resource(ref_root: str, kind: str, tag: str, name: str) -> str:
    """The <tag name="name">...</tag> element of res/<kind>.xml, verbatim."""
    src = open(os.path.join(ref_root, "res", kind + ".xml")).read()
    m = re.search(r'<%s name="%s">.*?</%s>' % (tag, re.escape(name), tag), src, re.S)
    return m.group(0)


def write_hyperkagome_resources(ref_root: str) -> None:
    out = os.path.join(HERE, "res_hyperkagome")
    os.makedirs(out, exist_ok=True)
    head = '<?xml version="1.0" encoding="utf-8"?>\n'
    with open(os.path.join(out, "lattices.xml"), "w") as f:
        f.write(head + extract_resource(ref_root, "lattices", "unitcell", "hyperkagome") + "\n")
    with open(os.path.join(out, "models.xml"), "w") as f:
        f.write(head + extract_resource(ref_root, "models", "model", "hyperkagome-heisenberg") + "\n")


def write_reference2(ref_root: str) -> None:
    """XYZ golden of test_reference2 (the XYZ task of the script's XYZ/TRI pair) and its
    resource files."""
    scripted = os.path.join(ref_root, "test", "scripted")
    script = open(os.path.join(scripted, "test_reference2.sh")).read()
    p = task_parameters(script.replace("${CORE}", "XYZ"))
    k = float(re.search(r"<k>([-0-9.]+)</k>", script).group(1))
    ref = os.path.join(scripted, "assets", "test_reference2.ref")
    comps = {}
    cut = None
    for c in ("XX", "YY", "ZZ", "DD"):
        cc, v = h5lite.read_correlations(ref, "XYZCor" + c)
        assert cut is None or np.array_equal(cut, cc)
        cut = cc
        comps[c.lower()] = v
    meta = h5lite.open_file(ref)["XYZCorXX/meta"]
    np.savez_compressed(os.path.join(HERE, "reference2_xyz.npz"), cutoffs=cut, **comps,
                        frequencies=np.array(p["frequencies"], np.float32),
                        cutoff_spec=np.array([p["cutoff_max"], p["cutoff_min"], p["cutoff_step"]], np.float32),
                        j=np.float32(p["j"]), k=np.float32(k), sites=meta["sites"].read(), basis=meta["basis"].read(),
                        lattice_vectors=meta["latticeVectors"].read())
    with open(os.path.join(HERE, "reference2_layout.json"), "w") as f:
        json.dump({"fingerprint": h5lite.layout_fingerprint(ref), "skeleton": h5lite.skeleton(ref)}, f, indent=0)
    out = os.path.join(HERE, "res_hyperhoneycomb")
    os.makedirs(out, exist_ok=True)
    head = '<?xml version="1.0" encoding="utf-8"?>\n'
    with open(os.path.join(out, "lattices.xml"), "w") as f:
        f.write(head + extract_resource(ref_root, "lattices", "unitcell", p["lattice"]) + "\n")
    with open(os.path.join(out, "models.xml"), "w") as f:
        f.write(head + extract_resource(ref_root, "models", "model", p["model"]) + "\n")


TRI_COMPONENTS = ("XX", "XY", "XZ", "YX", "YY", "YZ", "ZX", "ZY", "ZZ", "DD")


def write_reference3(ref_root: str) -> None:
    """TRI golden of test_reference3 (Heisenberg-Kitaev-Gamma on the honeycomb lattice) and its
    resource files."""
    scripted = os.path.join(ref_root, "test", "scripted")
    script = open(os.path.join(scripted, "test_reference3.sh")).read()
    p = task_parameters(script)
    k = float(re.search(r"<k>([-0-9.]+)</k>", script).group(1))
    g = float(re.search(r"<g>([-0-9.]+)</g>", script).group(1))
    ref = os.path.join(scripted, "assets", "test_reference3.ref")
    comps = {}
    cut = None
    for c in TRI_COMPONENTS:
        cc, v = h5lite.read_correlations(ref, "TRICor" + c)
        assert cut is None or np.array_equal(cut, cc)
        cut = cc
        comps[c.lower()] = v
    meta = h5lite.open_file(ref)["TRICorXX/meta"]
    np.savez_compressed(os.path.join(HERE, "reference3_tri.npz"), cutoffs=cut, **comps,
                        frequencies=np.array(p["frequencies"], np.float32),
                        cutoff_spec=np.array([p["cutoff_max"], p["cutoff_min"], p["cutoff_step"]], np.float32),
                        j=np.float32(p["j"]), k=np.float32(k), g=np.float32(g), sites=meta["sites"].read(),
                        basis=meta["basis"].read(), lattice_vectors=meta["latticeVectors"].read())
    with open(os.path.join(HERE, "reference3_layout.json"), "w") as f:
        json.dump({"fingerprint": h5lite.layout_fingerprint(ref), "skeleton": h5lite.skeleton(ref)}, f, indent=0)
    out = os.path.join(HERE, "res_honeycomb")
    os.makedirs(out, exist_ok=True)
    head = '<?xml version="1.0" encoding="utf-8"?>\n'
    with open(os.path.join(out, "lattices.xml"), "w") as f:
        f.write(head + extract_resource(ref_root, "lattices", "unitcell", p["lattice"]) + "\n")
    with open(os.path.join(out, "models.xml"), "w") as f:
        f.write(head + extract_resource(ref_root, "models", "model", p["model"]) + "\n")


def write_reference1_layout(ref: str) -> None:
    """Structure (members, attributes, shapes) and encoding fingerprint of the libhdf5-written
    test_reference1.ref, for checking the package's .obs writer without the file itself."""
    with open(os.path.join(HERE, "reference1_layout.json"), "w") as f:
        json.dump({"fingerprint": h5lite.layout_fingerprint(ref), "skeleton": h5lite.skeleton(ref)}, f, indent=0)


def main(ref_root: str) -> None:
    import spinparser_gb300 as spn

    # --- test_Lattice.cpp: lattice known-answer tests ---
    kats = lattice_kats(open(os.path.join(ref_root, "test", "test_Lattice.cpp")).read())
    with open(os.path.join(HERE, "lattice_kats.json"), "w") as f:
        json.dump(kats, f)

    scripted = os.path.join(ref_root, "test", "scripted")
    # --- test_reference1: hyperkagome golden ---
    p1 = task_parameters(open(os.path.join(scripted, "test_reference1.sh")).read())
    ref = os.path.join(scripted, "assets", "test_reference1.ref")
    cut, zz = h5lite.read_correlations(ref, "SU2CorZZ")
    cut_dd, dd = h5lite.read_correlations(ref, "SU2CorDD")
    assert np.array_equal(cut, cut_dd)
    meta = h5lite.open_file(ref)["SU2CorZZ/meta"]
    np.savez_compressed(os.path.join(HERE, "reference1_su2.npz"), cutoffs=cut, zz=zz, dd=dd,
                        frequencies=np.array(p1["frequencies"], np.float32),
                        cutoff_spec=np.array([p1["cutoff_max"], p1["cutoff_min"], p1["cutoff_step"]], np.float32),
                        j=np.float32(p1["j"]), sites=meta["sites"].read(), basis=meta["basis"].read(),
                        lattice_vectors=meta["latticeVectors"].read())
    lat = spn.Lattice(p1["lattice"], p1["range"], p1["model"], {"j": str(p1["j"])},
                      resource_dir=os.path.join(ref_root, "res"))
    lat.tables().to_npz(os.path.join(HERE, "hyperkagome_r3_tables.npz"))
    write_hyperkagome_resources(ref_root)
    write_reference1_layout(ref)

    # --- test_pythonObs: honeycomb expectations ---
    p2 = task_parameters(open(os.path.join(scripted, "test_pythonObs.sh")).read())
    src = open(os.path.join(scripted, "assets", "test_python_obs.py")).read()
    refs = [json.loads(m) for m in re.findall(r"reference = (\[.*\])", src)]
    queries = [
        {"what": "basis", "expect": refs[0]},
        {"what": "primitives", "expect": refs[1]},
        {"what": "sites", "reference": [0.0, 0.0, 0.0], "expect": refs[2]},
        {"what": "sites", "reference": [1.0, 0.0, 0.0], "expect": refs[3]},
        {"what": "correlation", "cutoff": "all", "site": [1.0, 0.0, 0.0], "reference": [0.0, 0.0, 0.0],
         "component": "all", "expect": refs[4]},
        {"what": "correlation", "cutoff": "all", "site": [1.0, 0.0, 0.0], "reference": [0.0, 0.0, 0.0],
         "component": "XX", "expect": refs[5]},
        {"what": "correlation", "cutoff": [0.309031], "site": "all", "reference": [0.0, 0.0, 0.0],
         "component": "ZZ", "expect": refs[6]},
        {"what": "correlation", "cutoff": [0.381520, 2.058910], "site": [[0.0, 0.0, 0.0], [2.5, 0.866025, 0.0]],
         "reference": [1.0, 0.0, 0.0], "component": "ZZ", "expect": refs[7]},
        {"what": "structure_factor", "momentum": [[0.0, 0.0, 0.0], [4.188790, 0.0, 0.0]], "cutoff": [0.381520],
         "expect": refs[8]},
    ]
    with open(os.path.join(HERE, "python_obs_honeycomb.json"), "w") as f:
        json.dump({"task": p2, "queries": queries}, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_fixtures.py <reference checkout> [reference2|reference3]")
    root = sys.argv[1]
    if len(sys.argv) > 2 and sys.argv[2] == "reference2":
        write_reference2(root)
    elif len(sys.argv) > 2 and sys.argv[2] == "reference3":
        write_reference3(root)
    else:
        main(root)
        write_reference2(root)
        write_reference3(root)
