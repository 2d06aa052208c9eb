"""Build recipe for the native parts of suqa_gb300 (in-tree, sm_103a only).

    python -m suqa_gb300.build            # libsq.so (+ the C++ drop-in shim and drivers)

Outputs go to suqa_gb300/_build/.  Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
SHIM_INCLUDE = os.path.join(PKG, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction so host-side
# coefficients (W factors, phases) round exactly as the reference computes them
# on any host architecture (an FMA turns Enew*c - E_old*c = 0 into +-1e-17).
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "-I" + INCLUDE, "-I" + CSRC]

LIB_SOURCES = ["sq_engine.cu", "sq_pass_f64.cu", "sq_pass_f32.cu", "sq_pass_tc.cu", "sq_pass_df.cu", "sq_noalloc.cu",
               "sq_batch.cu", "sq_mlp.cu", "sq_evo.cu", "sq_walk.cu"] + [
    "sq_batch_%s_m%d.cu" % (t, m) for t in ("f32", "f64") for m in (0, 1, 2)]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsq")
    return exe


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_libsq(force=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(INCLUDE, "sq.h"))
    objs = []
    jobs = []
    for src in LIB_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([nvcc()] + NVCC_FLAGS + ["-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))
    lib = os.path.join(BUILD, "libsq.so")
    if force or jobs or not os.path.exists(lib):
        _run([nvcc()] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])
    return lib


def build_probe(force=False):
    """libsq_probe.so: the benchmark's device characterisation (FP64 FMA rate),
    kept out of libsq's product ABI."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(CSRC, "bench_probe.cu")
    out = os.path.join(BUILD, "libsq_probe.so")
    if force or not _newer(out, [src]):
        _run([nvcc()] + NVCC_FLAGS + ["-shared", src, "-o", out, "-lcudart"])
    return out


CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-w", "-I" + SHIM_INCLUDE, "-I" + INCLUDE]
DRIVERS = ["qms", "qsa", "evo"]
GC_DRIVERS = ["qms", "qsa"]


def cxx():
    return shutil.which("g++") or "g++"


def build_dropin(force=False):
    """The suqa:: shim, the triangle system plugin and the qms/qsa/evo drivers
    (C++ over libsq)."""
    headers = [os.path.join(SHIM_INCLUDE, f) for f in os.listdir(SHIM_INCLUDE)] + [os.path.join(INCLUDE, "sq.h")]
    units = {"suqa_shim": os.path.join(PKG, "shim", "suqa_shim.cpp"),
             "triangle": os.path.join(PKG, "systems", "triangle.cpp")}
    for d in DRIVERS:
        units["app_" + d] = os.path.join(PKG, "apps", d + ".cpp")
    for d in GC_DRIVERS:  # the same drivers with the reference's gate-cost counters
        units["app_" + d + "_gc"] = os.path.join(PKG, "apps", d + ".cpp")
    jobs, objs = [], {}
    for name, src in units.items():
        o = os.path.join(BUILD, name + ".o")
        objs[name] = o
        if force or not _newer(o, [src] + headers):
            extra = ["-DGATECOUNT"] if name.endswith("_gc") else []
            jobs.append([cxx()] + CXX_FLAGS + extra + ["-c", src, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))
    lib = os.path.join(BUILD, "libsq.so")
    outs = []
    for d in DRIVERS + [g + "_gc" for g in GC_DRIVERS]:
        exe = os.path.join(BUILD, d)
        deps = [objs["app_" + d], objs["suqa_shim"], objs["triangle"], lib]
        if force or jobs or not _newer(exe, deps):
            _run([cxx(), objs["app_" + d], objs["suqa_shim"], objs["triangle"], "-L" + BUILD, "-lsq",
                  "-Wl,-rpath," + BUILD, "-o", exe])
        outs.append(exe)
    return outs


TFIM_SPINS = range(4, 13)


def build_tfim_drivers(force=False):
    """qms drivers with the transverse-field Ising ring plugin, one per ring length
    (the plugin API fixes the system width at compile time)."""
    tdir = os.path.join(PKG, "systems", "tfim")
    src_app = os.path.join(PKG, "apps", "qms.cpp")
    src_sys = os.path.join(PKG, "systems", "tfim_ring.cpp")
    headers = [os.path.join(SHIM_INCLUDE, f) for f in os.listdir(SHIM_INCLUDE)] + [os.path.join(tdir, "system.cuh")]
    shim = os.path.join(BUILD, "suqa_shim.o")
    lib = os.path.join(BUILD, "libsq.so")
    jobs = []
    for sp in TFIM_SPINS:
        exe = os.path.join(BUILD, f"qms_tfim_s{sp}")
        if force or not _newer(exe, [src_app, src_sys, shim, lib] + headers):
            jobs.append([cxx(), "-std=c++17", "-O2", "-ffp-contract=off", "-w", f"-DTFIM_SPINS={sp}", "-I" + tdir,
                         "-I" + SHIM_INCLUDE, "-I" + INCLUDE, src_app, src_sys, shim, "-L" + BUILD, "-lsq",
                         "-Wl,-rpath," + BUILD, "-o", exe])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))


def build_all(force=False):
    lib = build_libsq(force)
    build_probe(force)
    build_dropin(force)
    build_tfim_drivers(force)
    return lib


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
