"""Build the GB300 library and the host programs in-tree.

Outputs (git-ignored) under ``capsid-souffle_gb300/_build/``:
  libsouffle_gb300.so   CUDA kernels + C ABI (include/souffle_gpu.h), sm_103a only
  souffle_gb300         C++ MD driver with the reference's command line and outfiles

Translation units compile in parallel with nvcc; no cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
OUT = os.path.join(PKG, "_build")
INCLUDE = os.path.join(REPO, "include")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["pairlist.cu", "forces.cu", "energies.cu", "souffle_gpu.cu", "noalloc.cu", "gemm.cu", "mlp.cu", "mlp_fused.cu", "surrogate.cu",
              "analysis.cu"]
LIB = os.path.join(OUT, "libsouffle_gb300.so")
DRIVER = os.path.join(OUT, "souffle_gb300")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", INCLUDE,
                     "-I", CSRC, "--expt-relaxed-constexpr"]
    if verbose:
        common += ["-Xptxas", "-v"]
    objs = []
    jobs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([NVCC] + common + ["-c", s, "-o", o])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    if force or jobs or not _newer(LIB, objs):
        _run([NVCC] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    drv_src = [os.path.join(HOST, f) for f in sorted(os.listdir(HOST)) if f.endswith(".cpp")] \
        if os.path.isdir(HOST) else []
    drv_hdr = [os.path.join(HOST, f) for f in os.listdir(HOST) if f.endswith(".h")] if os.path.isdir(HOST) else []
    if drv_src and (force or not _newer(DRIVER, drv_src + drv_hdr + [LIB] + headers)):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-pthread", "-I", INCLUDE, "-o", DRIVER] + drv_src +
             ["-L", OUT, "-lsouffle_gb300", f"-Wl,-rpath,{OUT}"])
    text = "\n".join(logs)
    if verbose:
        print(text)
    return text


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
