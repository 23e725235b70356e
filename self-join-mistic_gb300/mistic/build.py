"""Builds libmistic.so, the `mistic` CLI and the `mistic_peaks` probe for
sm_103a with nvcc, in-tree under self-join-mistic_gb300/_build/.

Translation units compile in parallel; a rebuild happens only when a source
or the public header is newer than the library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REPO_ROOT = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
INCLUDE = os.path.join(REPO_ROOT, "include")
LIB = os.path.join(BUILD, "libmistic.so")
CLI = os.path.join(BUILD, "mistic")
PEAKS = os.path.join(BUILD, "mistic_peaks")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC"] + ARCH
LIB_CU = ["sort.cu", "index.cu", "join.cu", "join_tc.cu", "join_tcw.cu", "mistic.cu", "noalloc.cu", "brute.cu", "probe.cu"]
LIB_CPP = ["rp.cpp", "io.cpp"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _sources() -> list[str]:
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    out.append(os.path.join(INCLUDE, "mistic.h"))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(p) > t for p in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile everything that is stale; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = _sources()
    nvcc = _nvcc()
    if force or _stale(LIB, deps):
        objs = []
        cmds = []
        for f in LIB_CU + LIB_CPP:
            o = os.path.join(BUILD, os.path.splitext(f)[0] + ".o")
            objs.append(o)
            cmds.append([nvcc] + NVCC_FLAGS + ["-c", os.path.join(CSRC, f), "-o", o])
        with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
            list(ex.map(_run, cmds))
        _run([nvcc, "-shared"] + ARCH + ["-o", LIB] + objs)
        if verbose:
            print("built", LIB, file=sys.stderr)
    if force or _stale(CLI, deps + [LIB]):
        _run([nvcc, "-std=c++17", "-O2", os.path.join(CSRC, "cli.cpp"), "-o", CLI,
              "-L" + BUILD, "-lmistic", "-Xlinker", "-rpath=$ORIGIN"])
    if force or _stale(PEAKS, [os.path.join(CSRC, "peaks.cu")]):
        _run([nvcc] + ["-O3"] + ARCH + [os.path.join(CSRC, "peaks.cu"), "-o", PEAKS])
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
