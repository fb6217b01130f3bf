"""Build libecmg.so in-tree with nvcc for sm_103a (no CMake, no torch).

Translation units are compiled in parallel; the shared library lands in
ecmgenerator_gb300/_build/.  Device code is compiled with -fmad=false and host
code with -ffp-contract=off: the tick reproduces the reference's sequence of
separately rounded float operations.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libecmg.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["kernels.cu", "ctx.cu", "api_host.cu", "knn_static.cu", "mlp.cu", "spawn.cu", "kdtree.cu"]
CXX_SOURCES = ["host_scene.cpp", "ref_planner.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(PKG, "..", "include", "ecmg.h"))
    nv = nvcc()
    cuda_home = os.path.dirname(os.path.dirname(nv))
    common_dev = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "--expt-relaxed-constexpr",
                  "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", CSRC] + (extra or [])
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([nv] + common_dev + ["-c", s, "-o", o])
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append(["g++", "-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-I", CSRC,
                         "-I", os.path.join(cuda_home, "include"), "-c", s, "-o", o])
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    failed = []
    for j, p in procs:
        out, _ = p.communicate()
        if verbose and out:
            sys.stdout.write(out.decode(errors="replace"))
        if p.returncode != 0:
            failed.append((j, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(" ".join(j) + "\n" + o for j, o in failed)
        raise RuntimeError("libecmg build failed:\n" + msg)
    if force or jobs or not _newer(LIB, objs):
        link = [nv, ARCH, "-shared", "-o", LIB] + objs + ["-Xcompiler", "-pthread", "-cudart", "static"]
        r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("libecmg link failed:\n" + r.stdout.decode(errors="replace"))
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
