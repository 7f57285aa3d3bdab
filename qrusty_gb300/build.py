"""Build libqrusty_gpu.so (sm_103a) in-tree with nvcc.

Translation units are compiled in parallel and linked into
``qrusty_gb300/libqrusty_gpu.so``.  Used by ``__graft_entry__.build()`` and
by ``python -m qrusty_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libqrusty_gpu.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

SOURCES = ["qr_host.cu", "qr_apply.cu", "qr_csr.cu", "qr_reduce.cu", "qr_vec.cu", "qr_coef.cu",
           "qr_group.cu"]
HOST_SOURCES = ["qr_io.cpp"]  # host-only C++ (file formats), compiled by the host compiler
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
         "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", INCLUDE]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "include")


PROBE = os.path.join(PKG, "libqrusty_probe.so")


def _build_probe(force: bool, verbose: bool) -> None:
    """libqrusty_probe.so: measurement kernels of the benchmark (the FP64
    peak behind the complex128 roofline); not part of the product ABI."""
    src = os.path.join(CSRC, "qr_probe.cu")
    if not force and not _stale(PROBE, [src]):
        return
    tmp = PROBE + ".tmp%d" % os.getpid()
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", src, "-o", tmp]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    os.replace(tmp, PROBE)


def build(force: bool = False, verbose: bool = False, extra=()) -> str:
    os.makedirs(OBJ, exist_ok=True)
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(INCLUDE, "qrusty_gpu.h"))
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + hdrs):
            jobs.append((s, o))

    for src in HOST_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OBJ, src.replace(".cpp", ".o"))
        if force or _stale(o, [s] + hdrs):
            jobs.append((s, o))

    def compile_one(job):
        s, o = job
        if s.endswith(".cpp"):
            cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
            cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", INCLUDE,
                   "-I", cuda_include(), "-c", s, "-o", o + ".tmp"]
        else:
            cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", s, "-o", o + ".tmp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (s, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, file=sys.stderr)
        os.replace(o + ".tmp", o)

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES) + len(HOST_SOURCES)) as ex:
        list(ex.map(compile_one, jobs))
    _build_probe(force, verbose)
    objs = [os.path.join(OBJ, s.replace(".cu", ".o")) for s in SOURCES]
    objs += [os.path.join(OBJ, s.replace(".cpp", ".o")) for s in HOST_SOURCES]
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp%d" % os.getpid()
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    force = "--force" in sys.argv
    verbose = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else []
    print(build(force=force or bool(extra), verbose=verbose or bool(extra), extra=extra))
