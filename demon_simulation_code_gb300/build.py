"""Builds the sm_103a library libdemon_gb300.so in-tree with nvcc.

The library exports only the C ABI of include/demon_gb300.h (no torch
types); Python reaches it through ctypes (demon_simulation_code_gb300._lib).
"""
from __future__ import annotations

import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "libdemon_gb300.so")
BUILD = os.path.join(PKG, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-I" + os.path.join(ROOT, "include")]
SOURCES = ["dm_api.cu", "dm_noalloc.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
            if f.endswith((".cu", ".cuh", ".h"))]
    deps.append(os.path.join(ROOT, "include", "demon_gb300.h"))
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    objs = []
    procs = []
    for src in SOURCES:
        obj = os.path.join(BUILD, src.replace(".cu", ".o"))
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), cmd))
        objs.append(obj)
    for p, cmd in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode(errors="replace")))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (" ".join(cmd), r.stdout.decode(errors="replace")))
    os.replace(tmp, LIB)
    return LIB


HOST = os.path.join(PKG, "host")
HOST_LIB = os.path.join(PKG, "libdemon_gb300_host.so")
DRIVER = os.path.join(PKG, "demon_gb300")
HOST_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
              "-Wno-ignored-qualifiers",  # the reference's signatures return const values
              "-I" + os.path.join(ROOT, "include"), "-I" + HOST]


def cxx() -> str:
    return os.environ.get("CXX") or "g++"


def build_host(force: bool = False, verbose: bool = False) -> tuple[str, str]:
    """The C++ host classes (libdemon_gb300_host.so, linked to the CUDA
    library) and the demon_gb300 driver program."""
    lib = build(force=force, verbose=verbose)
    srcs = sorted(os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".cpp") and f != "driver.cpp")
    deps = srcs + [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")]
    deps += [os.path.join(ROOT, "include", "demon_gb300.h"), lib]
    link = ["-L" + PKG, "-ldemon_gb300", "-Wl,-rpath,$ORIGIN"]
    if force or _stale(HOST_LIB, deps):
        tmp = HOST_LIB + ".tmp"
        cmd = [cxx(), *HOST_FLAGS, "-shared", "-o", tmp, *srcs, *link]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("host build failed: %s\n%s" % (" ".join(cmd), r.stdout.decode(errors="replace")))
        os.replace(tmp, HOST_LIB)
    drv = os.path.join(HOST, "driver.cpp")
    if force or _stale(DRIVER, deps + [drv, HOST_LIB]):
        tmp = DRIVER + ".tmp"
        cmd = [cxx(), *HOST_FLAGS, "-o", tmp, drv, "-L" + PKG, "-ldemon_gb300_host", *link]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("driver build failed: %s\n%s" % (" ".join(cmd), r.stdout.decode(errors="replace")))
        os.replace(tmp, DRIVER)
    return HOST_LIB, DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_host(force="--force" in sys.argv, verbose=True))
