"""Build recipe for libswalbe_gb300.so (sm_103a, GB300).

Each translation unit is compiled by nvcc in parallel, then linked into one
shared library in swalbe.jl_gb300/lib/.  Float64 kernels are compiled with
--fmad=false so that their arithmetic matches the reference operation by
operation.
"""
from __future__ import annotations

import os
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(PKG_DIR, "csrc")
LIB_DIR = os.path.join(PKG_DIR, "lib")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libswalbe_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]
UNITS = {
    "swb_step_f64.cu": ["--fmad=false"],
    # no implicit FMA contraction: every kernel that inlines the step (single,
    # batch) must round identically for results to be independent of it
    "swb_step_f32.cu": ["--fmad=false"],
    "swb_run_f32.cu": ["--fmad=false"],
    "swb_resident.cu": ["--fmad=false"],
    "swb_api.cu": [],
    "swb_batch.cu": [],
    "swb_server.cu": [],
    "swb_noalloc.cu": [],
    "swb_analysis.cu": [],
    "swb_d1q3.cu": ["--fmad=false"],
}


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = os.path.join(cuda, "bin", "nvcc")
    return p if os.path.exists(p) else "nvcc"


def _deps_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(os.path.dirname(PKG_DIR), "include")):
        for f in os.listdir(d):
            m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= _deps_mtime()):
        return LIB_PATH
    procs = []
    objs = []
    for unit, extra in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(BUILD_DIR, unit.replace(".cu", ".o"))
        objs.append(obj)
        cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
