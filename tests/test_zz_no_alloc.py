"""spn_su2_correlation_noalloc: the correlation measurement for callers that cannot allocate
device memory when they measure (a framework that reserves the GPU's memory in its own pool,
a loop that must not enter the CUDA allocator).  The caller owns every device buffer; the
entry point's scratch is a fixed array inside the library.

Called through the C ABI with device pointers and checked against the handle-based entry
point spn_su2_measure_correlation on the same state, on two calls in a row with different
states and cutoffs, with the normwise tolerance of the other parity tests (1e-5).  The test
allocates its device buffers with PyTorch, as such a caller would with its own allocator.
This file is collected last so that a stop-at-first-failure run has run everything else.
"""
import ctypes as C

import numpy as np
import pytest

import spinparser_gb300 as spn

pytestmark = pytest.mark.gpu
TOL = 1e-5


def normwise(g, r):
    return float(np.max(np.abs(np.asarray(g, np.float64) - r)) / max(float(np.max(np.abs(r))), 1e-300))


def _state(tab, freq, cut, steps):
    """Flow state after `steps` GPU steps from the initial condition, and its cutoff."""
    flow = spn.Su2Flow(tab, freq)
    flow.set_state(float(cut[0]), *tab.initial_state(len(freq)))
    for k in range(steps):
        flow.compute_step()
        flow.finalize_step(float(cut[k + 1]))
    c, v2, ss, dd = flow.get_state()
    flow.close()
    return c, v2, ss, dd


def _perturbed_initial_state(tab, n, seed):
    """The model's initial condition plus a seeded perturbation of every entry (a state no
    flow step is needed for, so the largest frequency count stays cheap)."""
    v2, ss, dd = tab.initial_state(n)
    rng = np.random.default_rng(seed)
    v2 = (v2 + 0.01 * rng.standard_normal(v2.shape)).astype(np.float32)
    ss = (ss + 0.05 * rng.standard_normal(ss.shape)).astype(np.float32)
    dd = (dd + 0.05 * rng.standard_normal(dd.shape)).astype(np.float32)
    return v2, ss, dd


# (lattice, range, model, couplings, N, states): square r3 runs the one-site-per-lane kernel,
# r11 (42 sites) two sites per lane, r15 (72 sites) four; N = 256 fills the scratch's rows
# (2N + 4 of 2 * 256 + 8 node rows).  States: GPU flow steps from the initial condition, or
# seeded perturbations of it at two cutoffs.
CASES = [
    ("square", 3, "square-j1j2heisenberg", {"j1": "1.0", "j2": "0.3"}, 20, ("steps", 6, 30)),
    ("square", 11, "square-heisenberg", {"j": "1.0"}, 10, ("steps", 2, 5)),
    ("square", 15, "square-heisenberg", {"j": "1.0"}, 8, ("steps", 2, 5)),
    ("square", 3, "square-heisenberg", {"j": "1.0"}, 256, ("perturbed", 0.8, 0.05)),
]


@pytest.mark.parametrize("lattice,rng_,model,params,n,states", CASES,
                         ids=["sites6-n20", "sites42-n10", "sites72-n8", "sites6-n256"])
def test_noalloc_correlation_matches_handle_entry_point_twice(lattice, rng_, model, params, n, states):
    torch = pytest.importorskip("torch")
    lib = spn.load_library()
    tab = spn.Lattice(lattice, rng_, model, params).tables()
    freq = spn.frequency_exponential(0.005, 50.0, n)
    cut = spn.cutoff_exponential(50.0, 0.05, 0.9)
    dev = torch.device("cuda:0")

    def d(a, dtype):
        return torch.from_numpy(np.ascontiguousarray(a, dtype)).to(dev)

    freq_d = d(freq, np.float32)
    sites_d = d(tab.sites_rid, np.int32)
    inv_d = d(tab.inv_sites_rid, np.int32)
    corr_d = d(tab.corr_rid, np.int32)
    n_corr, nl = len(tab.corr_rid), tab.n_sites
    out_d = torch.full((2 * n_corr + 2 * nl,), float("nan"), dtype=torch.float32, device=dev)

    first = None
    for k, x in enumerate(states[1:]):  # two calls in a row, different states and cutoffs
        if states[0] == "steps":
            c, v2, ss, dd = _state(tab, freq, cut, x)
        else:
            c = np.float32(x)
            v2, ss, dd = _perturbed_initial_state(tab, n, 20261204 + k)
        v2_d, ss_d, dd_d = d(v2, np.float32), d(ss, np.float32), d(dd, np.float32)
        rc = lib.spn_su2_correlation_noalloc(
            len(freq), C.c_void_p(freq_d.data_ptr()), nl, C.c_void_p(sites_d.data_ptr()),
            C.c_void_p(inv_d.data_ptr()), n_corr, C.c_void_p(corr_d.data_ptr()), 0.5, float(c),
            C.c_void_p(v2_d.data_ptr()), C.c_void_p(ss_d.data_ptr()), C.c_void_p(dd_d.data_ptr()),
            C.c_void_p(out_d.data_ptr()), None)
        spn._capi.check(rc)
        torch.cuda.synchronize()
        out = out_d.cpu().numpy()
        del v2_d, ss_d, dd_d

        flow = spn.Su2Flow(tab, freq)
        flow.set_state(float(c), v2, ss, dd)
        zz, ddc, cz, cd = flow.measure_correlation()
        flow.close()
        assert np.all(np.isfinite(out))
        assert normwise(out[:n_corr], zz) <= TOL
        assert normwise(out[n_corr:2 * n_corr], ddc) <= TOL
        assert normwise(out[2 * n_corr:2 * n_corr + nl], cz) <= TOL
        assert normwise(out[2 * n_corr + nl:], cd) <= TOL
        if first is None:
            first = out.copy()
        else:
            assert not np.array_equal(first, out)  # the second call saw its own state


def test_noalloc_correlation_rejects_sizes_beyond_its_scratch():
    lib = spn.load_library()
    dummy = C.c_void_p(16)  # never dereferenced: the size check comes first
    rc = lib.spn_su2_correlation_noalloc(300, dummy, 6, dummy, dummy, 1, dummy, 0.5, 1.0, dummy, dummy, dummy, dummy,
                                         None)
    assert rc == -8
    buf = C.create_string_buffer(256)
    lib.spn_last_error(buf, 256)
    assert b"n_freq" in buf.value
    rc = lib.spn_su2_correlation_noalloc(16, dummy, 200, dummy, dummy, 1, dummy, 0.5, 1.0, dummy, dummy, dummy, dummy,
                                         None)
    assert rc == -8
