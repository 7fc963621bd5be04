"""The C ABI library loads without a GPU, exports every function include/spn_su2.h declares,
and rejects bad descriptors before touching the device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import spinparser_gb300 as spn
from spinparser_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for hdr in os.listdir(os.path.join(ROOT, "include")):
        if hdr.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", hdr)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names += re.findall(r"^\s*int\s+(spn_\w+)\s*\(", txt, flags=re.M)
    return names


def test_every_declared_symbol_is_exported_and_bound():
    lib = spn.load_library()
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n
        assert n in _capi.SIGNATURES, n


def test_descriptor_validation_happens_before_device_use():
    lib = spn.load_library()
    h = C.c_void_p()
    assert lib.spn_su2_create(None, C.byref(h)) == -2
    buf = C.create_string_buffer(256)
    assert lib.spn_last_error(buf, 256) > 0 and b"descriptor" in buf.value
    tab = spn.Lattice("square", 2, "square-heisenberg", {"j": 1}).tables()
    with pytest.raises(spn.SpnError) as e:
        spn.Su2Flow(tab, np.array([1.0, 0.5, 2.0], np.float32))  # not ascending
    assert e.value.code == -2
    with pytest.raises(spn.SpnError) as e:
        spn.Su2Flow(tab, np.linspace(0.1, 1, 300).astype(np.float32))  # N above the supported maximum
    assert e.value.code == -8
    with pytest.raises(spn.SpnError) as e:  # one frequency above the largest supported mesh (256)
        spn.Su2Flow(tab, spn.frequency_exponential(0.005, 50.0, 257))
    assert e.value.code == -8 and "n_freq" in str(e.value)
    big = spn.Lattice("square", 21, "square-heisenberg", {"j": 1}).tables()
    assert big.n_sites == 132  # above the largest supported lattice (128 reduced sites)
    with pytest.raises(spn.SpnError) as e:
        spn.Su2Flow(big, spn.frequency_exponential(0.005, 50.0, 8))
    assert e.value.code == -8 and "n_sites" in str(e.value)
    bad = spn.Lattice("square", 2, "square-heisenberg", {"j": 1}).tables()
    bad.overlap_rid1 = bad.overlap_rid1.copy()
    bad.overlap_rid1[0] = 99
    with pytest.raises(spn.SpnError) as e:
        spn.Su2Flow(bad, np.array([0.5, 1.0, 2.0], np.float32))
    assert "overlap_rid1" in str(e.value)


def test_device_count_without_gpu_is_not_an_error():
    assert spn.device_count() >= 0


def test_probe_arguments_are_checked_before_device_use():
    """spn_measure_gather_peak validates its shape on the host (one warp request per segment)."""
    for n_sites, n_slabs in ((0, 10), (33, 10), (8, 0)):
        with pytest.raises(spn.SpnError) as e:
            spn.measure_gather_peak(n_sites, n_slabs)
        assert e.value.code == -2


def test_header_is_plain_c(tmp_path):
    """include/spn_su2.h is the FFI boundary: it must compile as ISO C99 (cgo, ctypes, JNI stubs)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "use.c"
    src.write_text('#include "spn_su2.h"\nint main(void) { spn_tri_desc d; spn_su2_desc s; (void)d; (void)s; return 0; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(root, "include"),
                        "-c", str(src), "-o", str(tmp_path / "use.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
