"""In-tree build of libspn_su2.so (CUDA kernels for sm_103a + host C++) and of the CPU oracle.

Products go to ``spinparser_gb300/_build/<machine>/`` so that an x86_64 build and an aarch64
build never shadow each other.  Host objects are compiled with ``-ffp-contract=off``: the
lattice factory and the grid generators must round exactly like the reference's scalar C++.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
ORACLE_DIR = os.path.join(ROOT, "oracle")

HOST_SOURCES = ["host/xml.cpp", "host/lattice.cpp", "host/capi_host.cpp", "host/pair_order.cpp", "host/h5.cpp", "host/task.cpp",
                "host/su2_files.cpp", "host/run.cpp", "host/rpa_schedule.cpp"]
CUDA_SOURCES = ["su2_flow.cu", "su2_vertex.cu", "su2_vertex64.cu", "su2_batch.cu", "xyz_flow.cu", "tri_flow.cu"]
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def build_dir() -> str:
    return os.path.join(PKG, "_build", platform.machine())


def library_path() -> str:
    return os.path.join(build_dir(), "libspn_su2.so")


def oracle_library_path() -> str:
    return os.path.join(ORACLE_DIR, "_build", platform.machine(), "liboracle_su2.so")


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libspn_su2.so")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build command failed:\n" + " ".join(cmd) + "\n" + proc.stdout)
    if proc.stdout.strip() and os.environ.get("SPN_BUILD_VERBOSE"):
        sys.stderr.write(proc.stdout)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _all_headers() -> list[str]:
    out = []
    for base, _, files in os.walk(CSRC):
        out += [os.path.join(base, f) for f in files if f.endswith((".hpp", ".cuh", ".h"))]
    out.append(os.path.join(ROOT, "include", "spn_su2.h"))
    return out


def build_library(force: bool = False) -> str:
    """Compiles libspn_su2.so; returns its path."""
    bdir = build_dir()
    os.makedirs(bdir, exist_ok=True)
    nvcc = _nvcc()
    headers = _all_headers()
    jobs = []
    objects = []
    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(bdir, os.path.basename(src) + ".o")
        objects.append(o)
        if force or _stale(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-c", s, "-o", o])
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(bdir, os.path.basename(src) + ".o")
        objects.append(o)
        if force or _stale(o, [s] + headers):
            # 20011: a __host__ __device__ function calling a host-only function compiles to
            # undefined device code; it must never build.
            jobs.append([nvcc, *ARCH_FLAGS, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                         "--diag-error=20011", "-diag-suppress=128", "-Xptxas", "-warn-spills", "-c", s, "-o", o])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    lib = library_path()
    if force or _stale(lib, objects):
        _run([nvcc, *ARCH_FLAGS, "-shared", "-o", lib, *objects, "-lcudart_static", "-lpthread", "-ldl", "-lrt"])
    return lib


def oracle_timing_library_path() -> str:
    return os.path.join(ORACLE_DIR, "_build", platform.machine(), "liboracle_su2_o3.so")


def build_oracle(force: bool = False) -> str:
    """Compiles the CPU oracle (test infrastructure) into oracle/_build/<machine>/: the checker
    (-O2 -ffp-contract=off: every float operation rounded on its own, as the reference's
    x86-64 build rounds) and, from the same sources, the timed CPU baseline built with the
    reference's own optimisation flags (-O3, the compiler's default floating-point contraction;
    CMakeLists.txt of the reference), in parallel."""
    out = oracle_library_path()
    timing = oracle_timing_library_path()
    os.makedirs(os.path.dirname(out), exist_ok=True)
    srcs = [os.path.join(ORACLE_DIR, f) for f in ("su2_oracle.cpp", "xyz_oracle.cpp", "tri_oracle.cpp")]
    jobs = []
    if force or _stale(out, srcs):
        jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", *srcs, "-o", out])
    if force or _stale(timing, srcs):
        jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", *srcs, "-o", timing])
    with ThreadPoolExecutor(max_workers=2) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    return out


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv))
    print(build_oracle(force="--force" in sys.argv))
