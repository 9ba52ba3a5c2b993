"""Build libassist_gb300.so (sm_103a) and the oracle checker library.

The library is a plain C ABI over hand-written CUDA kernels: every translation
unit is compiled by nvcc for sm_103a only, in parallel, and linked in place
(assist_gb300/libassist_gb300.so).  The oracle (test infrastructure) is built
by oracle/Makefile; the reference checker oracle/_ref/ only where the ASSIST
sources are present.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libassist_gb300.so")
SOURCES = ["kernels_forces.cu", "kernels_ias15.cu", "kernels_coop.cu", "kernels_shared.cu", "static_batch.cu", "kernels_mlp.cu",
           "kernels_pilot.cu", "host_ephem.cpp", "api.cpp", "autotune.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-lineinfo",
          "--expt-relaxed-constexpr", "-I", CSRC, "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libassist_gb300")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    objs, jobs = [], []
    for src in SOURCES:
        sp = os.path.join(CSRC, src)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [sp] + headers):
            # every unit is compiled as CUDA: the host units share the device structs
            cmd = [nv] + ARCH + COMMON + ["-x", "cu", "-c", sp, "-o", obj]
            if src.endswith(".cu"):
                cmd += ["-Xptxas", "-v"] if verbose else []
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    if force or jobs or _stale(LIB, objs):
        _run([nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    return LIB


def build_oracle() -> str:
    odir = os.path.join(ROOT, "oracle")
    _run(["make", "-s", "-C", odir])
    ref_src = os.environ.get("ASSIST_REFERENCE", "/root/reference")
    if os.path.isfile(os.path.join(ref_src, "src", "forces.c")):
        _run(["sh", os.path.join(odir, "build_ref.sh"), ref_src])
    return os.path.join(odir, "liboracle.so")


if __name__ == "__main__":
    print(build_library(verbose="-v" in sys.argv, force="-f" in sys.argv))
    print(build_oracle())
